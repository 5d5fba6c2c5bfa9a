// fixed.h -- launchers of the compile-time-sized cluster plane kernels
// (fixed.cu).  Each launcher starts the variant built for the plane size,
// cluster size, BC pair kinds and input/output functor of the call and sets
// *handled; when no variant is built it sets *handled = false and launches
// nothing (the caller then runs the run-time-sized kernels).
#pragma once
#include "kernels.cuh"

namespace fg {

// Built variants: FP32, square planes N x N with N = 256 and clusters of 8
// CTAs, x and y transforms of kind PP or NN.
bool fixed_supported(int nx, int ny, int C, int px, int py);

template <typename T, typename In>
cudaError_t xyfwd_fixed(const AxisPlan &, const AxisPlan &, const In &, T *, const Geo &, double *, int,
                        cudaStream_t, bool *handled) {
  *handled = false;
  return cudaSuccess;
}
cudaError_t xyfwd_fixed(const AxisPlan &ax, const AxisPlan &ay, const InKeep<InFillps> &in, float *S, const Geo &g,
                        double *nrm, int C, cudaStream_t st, bool *handled);
cudaError_t xyfwd_fixed(const AxisPlan &ax, const AxisPlan &ay, const InKeep<InHalo> &in, float *S, const Geo &g,
                        double *nrm, int C, cudaStream_t st, bool *handled);
cudaError_t xyfwd_fixed(const AxisPlan &ax, const AxisPlan &ay, const InResidual &in, float *S, const Geo &g,
                        double *nrm, int C, cudaStream_t st, bool *handled);
cudaError_t xyfwd_fixed(const AxisPlan &ax, const AxisPlan &ay, const InF32 &in, float *S, const Geo &g,
                        double *nrm, int C, cudaStream_t st, bool *handled);

template <typename T, typename Out>
cudaError_t xyinv_fixed(const AxisPlan &, const AxisPlan &, const T *, const Out &, const Geo &, int, cudaStream_t,
                        bool *handled) {
  *handled = false;
  return cudaSuccess;
}
cudaError_t xyinv_fixed(const AxisPlan &ax, const AxisPlan &ay, const float *S, const OutHalo &out, const Geo &g,
                        int C, cudaStream_t st, bool *handled);
cudaError_t xyinv_fixed(const AxisPlan &ax, const AxisPlan &ay, const float *S, const OutHaloAdd &out, const Geo &g,
                        int C, cudaStream_t st, bool *handled);

}  // namespace fg
