// fixed.h -- launchers of the compile-time-sized cluster plane kernels
// (fixed.cu).  Each launcher starts the variant built for the plane size,
// cluster size, BC pair kinds and input/output functor of the call and sets
// *handled; when no variant is built it sets *handled = false and launches
// nothing (the caller then runs the run-time-sized kernels).
#pragma once
#include "kernels.cuh"

namespace fg {

// Built variants: FP32, square planes N x N with N = 256 (clusters of 8 CTAs,
// three per SM) or N = 512 (clusters of 16, one per SM), x and y transforms of
// kind PP or NN, input already evaluated in FP32 (k_stencil_pass).
bool fixed_supported(int nx, int ny, int C, int px, int py);
// Cluster size of the built variant for this plane, 0 when none is built or
// this device cannot place its cluster.
int fixed_cluster_size(int nx, int ny, int px, int py);

template <typename T, typename In>
cudaError_t xyfwd_fixed(const AxisPlan &, const AxisPlan &, const In &, T *, const Geo &, double *, int,
                        cudaStream_t, bool *handled) {
  *handled = false;
  return cudaSuccess;
}
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
