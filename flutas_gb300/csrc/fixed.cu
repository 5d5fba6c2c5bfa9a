// fixed.cu -- compile-time-sized cluster plane kernels.
//
// The x and y transforms of one z-plane, shared by a cluster of C CTAs as in
// k_xyfwd_cluster / k_xyinv_cluster (kernels.cuh), with the plane size, the
// cluster size and the BC pair kinds as template parameters, so that the
// transforms use the fixed-size passes of fft_fixed.cuh (no run-time index
// arithmetic, pre/post passes folded into the Stockham stages) and the
// exchange through distributed shared memory has constant trip counts.
// Twiddle and pre/post tables live in shared memory.
#define FG_NO_PLAIN_KERNELS
#include "fixed.h"
#include "fft_fixed.cuh"

#include <cstdint>
#include <cstdlib>
#include <type_traits>
#include <mutex>
#include <set>

namespace fg {
namespace {

// Built variants: (N, C, threads) = (256, 8, 256) with three CTAs per SM and
// (512, 16, 512) with one (non-portable cluster size).  NBUF: plane buffers
// per CTA.  With two Stockham stages (N = 256) two buffers suffice: every pass
// writes the buffer its first stage has finished reading (see the kernels),
// which brings a CTA to 72 KB of shared memory and three CTAs to an SM (at
// most 80 registers a thread, no spills); N = 512 (three stages) keeps three.
template <int N> struct FixCfg;
template <> struct FixCfg<256> { static constexpr int C = 8, NTH = 256, NBUF = 2, MINB = 3; };
template <> struct FixCfg<512> { static constexpr int C = 16, NTH = 512, NBUF = 3, MINB = 1; };

template <typename T, int N, int C> struct FixGeo {
  static constexpr int ROWS = N / C, COLS = N / C, P = N + 1, BX = ROWS / 2, BY = COLS / 2;
  static constexpr size_t A = (size_t)ROWS * P, BN = (size_t)N * COLS;
  static constexpr size_t BUF = ((sizeof(T) * (A > BN ? A : BN)) + 255) & ~(size_t)255;
  static constexpr size_t TAB = sizeof(C2<T>) * N;
  static constexpr int NBUF = FixCfg<N>::NBUF;
  static constexpr size_t SMEM = NBUF * BUF + 3 * TAB;
  static_assert(N % C == 0 && ROWS % 2 == 0, "plane must split into an even number of rows per CTA");
  static_assert(NBUF == 3 || fix::Plan<N>::NST == 2, "two buffers need exactly two stages per transform");
};

struct Barrier {
  __device__ void operator()() const { __syncthreads(); }
};

// Columns [r*COLS, (r+1)*COLS) of every CTA's x-spectrum rows (pitch P) into
// this CTA's column block (N x COLS, row-major).
template <typename T, int N, int C, int FIX_NTH>
__device__ __forceinline__ void gather_cols(cg::cluster_group &cl, T *slab, T *blk, int r) {
  using G = FixGeo<T, N, C>;
  constexpr int TOT = N * G::COLS, U = 8;
  const int x0 = r * G::COLS;
  for (int b = threadIdx.x; b < TOT; b += FIX_NTH * U) {
    T v[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const unsigned idx = b + u * FIX_NTH;
      if (idx < (unsigned)TOT) {
        const unsigned gl = idx / G::COLS, xc = idx % G::COLS, s = gl / G::ROWS, lr = gl % G::ROWS;
        v[u] = cl.map_shared_rank(slab, (int)s)[lr * G::P + x0 + xc];
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const unsigned idx = b + u * FIX_NTH;
      if (idx < (unsigned)TOT) blk[idx] = v[u];
    }
  }
}

// This CTA's rows (ROWS x N, pitch P) from every CTA's column block.
template <typename T, int N, int C, int FIX_NTH>
__device__ __forceinline__ void gather_rows(cg::cluster_group &cl, T *blk, T *slab, int r) {
  using G = FixGeo<T, N, C>;
  constexpr int TOT = G::ROWS * N, U = 8;
  for (int b = threadIdx.x; b < TOT; b += FIX_NTH * U) {
    T v[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const unsigned idx = b + u * FIX_NTH;
      if (idx < (unsigned)TOT) {
        const unsigned lr = idx / N, xg = idx % N, s = xg / G::COLS, xc = xg % G::COLS;
        v[u] = cl.map_shared_rank(blk, (int)s)[(r * G::ROWS + lr) * G::COLS + xc];
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const unsigned idx = b + u * FIX_NTH;
      if (idx < (unsigned)TOT) slab[idx + idx / N] = v[u];
    }
  }
}

template <typename T, int N, int PX, int PY, int FIX_NTH>
__device__ __forceinline__ void load_tables(const AxisPlan &ax, const AxisPlan &ay, C2<T> *Wt, C2<T> *Qx, C2<T> *Qy) {
  for (int i = threadIdx.x; i < N; i += FIX_NTH) {
    Wt[i] = ((const C2<T> *)ax.W)[i];
    if (PX != BC_PP) Qx[i] = ((const C2<T> *)ax.Q)[i];
    if (PY != BC_PP) Qy[i] = ((const C2<T> *)ay.Q)[i];
  }
}

template <typename T, int N, int C, int FIX_NTH, int PX, int PY, typename In>
__global__ void __launch_bounds__(FIX_NTH, FixCfg<N>::MINB) k_xyfwd_fix(AxisPlan ax, AxisPlan ay, In in, T *S, Geo g, double *nrm) {
  using G = FixGeo<T, N, C>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank(), tid = threadIdx.x;
  constexpr bool TWO = G::NBUF == 2;
  T *B0 = (T *)smem_raw, *B1 = (T *)(smem_raw + G::BUF), *B2 = (T *)(smem_raw + (G::NBUF - 1) * G::BUF);
  C2<T> *Wt = (C2<T> *)(smem_raw + G::NBUF * G::BUF), *Qx = Wt + N, *Qy = Qx + N;
  load_tables<T, N, PX, PY, FIX_NTH>(ax, ay, Wt, Qx, Qy);
  const Barrier bar;
  const int y0 = r * G::ROWS;
  float ss = 0.0f;
  for (int k = blockIdx.x / C; k < g.nz; k += gridDim.x / C) {
    bool copied = false;
    if constexpr (std::is_same_v<In, InF32> && std::is_same_v<T, float>) {
      if (!nrm) {  // this CTA's rows of plane k, copied into the pitched slab (no norm to take on the way)
        const float *src = in.f + ((long)k * N + y0) * N;
        for (int u = tid; u < G::ROWS * N; u += FIX_NTH) cp_async4(B0 + u + u / N, src + u);
        cp_async_wait_all();
        copied = true;
      }
    }
    if (!copied)
      load_cells<T>(
          in, G::ROWS * N,
          [&](int idx, int &x, int &y, int &kk) -> bool {
            const unsigned u = idx;
            x = (int)(u % N);
            y = y0 + (int)(u / N);
            kk = k;
            return true;
          },
          [&](int idx, T t) {
            const unsigned u = idx;
            B0[u + u / N] = t;  // row ly = u / N at pitch P = N + 1
          },
          ss);
    __syncthreads();
    if constexpr (TWO) {
      // x: rows in B0 -> stage B1 -> stage B0 (read after the first stage) -> split
      // into the x-spectrum rows, B1; gathered into the column block, B0
      fix::forward<T, N, PX, G::BX, FIX_NTH>(B0, G::P, 1, (C2<T> *)B1, (C2<T> *)B0, Wt, Qx,
                                              StorePlaneReal<T>{B1, G::P, 0}, tid, bar);
      cluster.sync();  // every CTA's x-spectrum rows are complete
      gather_cols<T, N, C, FIX_NTH>(cluster, B1, B0, r);
      cluster.sync();  // every CTA has read the rows
      // y: columns in B0 -> stage B1 -> stage B0 -> split into S
      fix::forward<T, N, PY, G::BY, FIX_NTH>(B0, 1, G::COLS, (C2<T> *)B1, (C2<T> *)B0, Wt, Qy,
                                              StoreColsS<T>{S, (long)k * N * N, N, r * G::COLS, G::COLS}, tid, bar);
    } else {
      // x: rows in B0 -> stages in B1/B2 -> split into the x-spectrum rows, B0
      fix::forward<T, N, PX, G::BX, FIX_NTH>(B0, G::P, 1, (C2<T> *)B1, (C2<T> *)B2, Wt, Qx,
                                              StorePlaneReal<T>{B0, G::P, 0}, tid, bar);
      cluster.sync();  // every CTA's x-spectrum rows are complete
      gather_cols<T, N, C, FIX_NTH>(cluster, B0, B1, r);
      cluster.sync();  // every CTA has read the rows
      // y: columns in B1 -> stages in B2/B0 -> split into S
      fix::forward<T, N, PY, G::BY, FIX_NTH>(B1, 1, G::COLS, (C2<T> *)B2, (C2<T> *)B0, Wt, Qy,
                                              StoreColsS<T>{S, (long)k * N * N, N, r * G::COLS, G::COLS}, tid, bar);
    }
    __syncthreads();
  }
  if (nrm) block_sum_add((double)ss, nrm);
}

template <typename T, int N, int C, int FIX_NTH, int PX, int PY, typename Out>
__global__ void __launch_bounds__(FIX_NTH, FixCfg<N>::MINB) k_xyinv_fix(AxisPlan ax, AxisPlan ay, const T *S, Out out, Geo g) {
  using G = FixGeo<T, N, C>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank(), tid = threadIdx.x;
  constexpr bool TWO = G::NBUF == 2;
  T *B0 = (T *)smem_raw, *B1 = (T *)(smem_raw + G::BUF), *B2 = (T *)(smem_raw + (G::NBUF - 1) * G::BUF);
  C2<T> *Wt = (C2<T> *)(smem_raw + G::NBUF * G::BUF), *Qx = Wt + N, *Qy = Qx + N;
  load_tables<T, N, PX, PY, FIX_NTH>(ax, ay, Wt, Qx, Qy);
  const Barrier bar;
  const int y0 = r * G::ROWS;
  T *const rows = TWO ? B1 : B2;  // the x^-1 output rows that store_cells reads
  for (int k = blockIdx.x / C; k < g.nz; k += gridDim.x / C) {
    if constexpr (std::is_same_v<Out, OutHaloAdd>) {  // the rows this CTA adds to, on their way to L2
      const double *span = out.p + out.g.pidx(0, y0 + 1, k + 1);
      const unsigned bytes = (unsigned)(sizeof(double) * G::ROWS * (N + 2)) & ~15u;
      if (tid == 0 && ((uintptr_t)span & 15) == 0) prefetch_l2(span, bytes);
    }
    const T *Sp = S + (long)k * N * N + r * G::COLS;
    if constexpr (std::is_same_v<T, float>) {  // the column block: 16-byte copies, all in flight together
      static_assert(G::COLS % 4 == 0, "column block rows must be whole 16-byte chunks");
      constexpr int Q = G::COLS / 4;
      for (int i = tid; i < N * Q; i += FIX_NTH) {
        const unsigned rw = i / Q, c = i % Q;
        cp_async16(B0 + rw * G::COLS + 4 * c, Sp + (long)rw * N + 4 * c);
      }
      cp_async_wait_all();
    } else {
      for (int i = tid; i < N * G::COLS; i += FIX_NTH) {
        const unsigned u = i;
        B0[i] = Sp[(u / G::COLS) * N + u % G::COLS];
      }
    }
    __syncthreads();
    if constexpr (TWO) {
      // y^-1: columns in B0 -> stage B1 -> columns back in B0 (read by the first stage)
      fix::inverse<T, N, PY, G::BY, FIX_NTH>(B0, 1, G::COLS, B0, 1, G::COLS, (C2<T> *)B1, (C2<T> *)B0, Wt, Qy,
                                              tid, bar);
      cluster.sync();  // every CTA's column block is complete
      gather_rows<T, N, C, FIX_NTH>(cluster, B0, B1, r);
      cluster.sync();  // every CTA has read the blocks
      // x^-1: rows in B1 (pitch P) -> stage B0 -> rows back in B1
      fix::inverse<T, N, PX, G::BX, FIX_NTH>(B1, G::P, 1, B1, G::P, 1, (C2<T> *)B0, (C2<T> *)B1, Wt, Qx, tid, bar);
    } else {
      // y^-1: columns in B0 -> stages in B1/B0 -> columns in B2
      fix::inverse<T, N, PY, G::BY, FIX_NTH>(B0, 1, G::COLS, B2, 1, G::COLS, (C2<T> *)B1, (C2<T> *)B0, Wt, Qy,
                                              tid, bar);
      cluster.sync();  // every CTA's column block is complete
      gather_rows<T, N, C, FIX_NTH>(cluster, B2, B0, r);
      cluster.sync();  // every CTA has read the blocks
      // x^-1: rows in B0 -> stages in B1/B0 -> rows in B2 (pitch P)
      fix::inverse<T, N, PX, G::BX, FIX_NTH>(B0, G::P, 1, B2, G::P, 1, (C2<T> *)B1, (C2<T> *)B0, Wt, Qx, tid, bar);
    }
    __syncthreads();
    store_cells<T>(
        out, G::ROWS * N,
        [&](int idx, int &x, int &y, int &kk) -> bool {
          const unsigned u = idx;
          x = (int)(u % N);
          y = y0 + (int)(u / N);
          kk = k;
          return true;
        },
        [&](int idx) {
          const unsigned u = idx;
          return rows[u + u / N];
        });
    __syncthreads();
  }
}

// Raises the kernel's dynamic shared-memory limit once per device.
int prepare(const void *kernel, size_t smem, int C) {
  static std::mutex mu;
  static std::set<std::pair<const void *, int>> done;
  std::lock_guard<std::mutex> lk(mu);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  if (done.count({kernel, dev})) return 0;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return -1;
  if (C > 8 && cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
    return -1;
  done.insert({kernel, dev});
  return 0;
}

template <typename K, typename... Args>
cudaError_t cluster_start(K kernel, size_t smem, int clusters, int C, int nth, cudaStream_t st, Args... args) {
  if (prepare((const void *)kernel, smem, C)) return cudaErrorInvalidValue;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(clusters * C));
  cfg.blockDim = dim3((unsigned)nth);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)C;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

bool kind_ok(int p) { return p == BC_PP || p == BC_NN; }


template <int N, typename F> cudaError_t with_kinds(int px, int py, F &&f) {
  if (px == BC_PP && py == BC_PP) return f(std::integral_constant<int, BC_PP>(), std::integral_constant<int, BC_PP>());
  if (px == BC_PP && py == BC_NN) return f(std::integral_constant<int, BC_PP>(), std::integral_constant<int, BC_NN>());
  if (px == BC_NN && py == BC_PP) return f(std::integral_constant<int, BC_NN>(), std::integral_constant<int, BC_PP>());
  if (px == BC_NN && py == BC_NN) return f(std::integral_constant<int, BC_NN>(), std::integral_constant<int, BC_NN>());
  return cudaErrorInvalidValue;
}

template <int N>
cudaError_t fwd_n(const AxisPlan &ax, const AxisPlan &ay, const InF32 &in, float *S, const Geo &g, double *nrm,
                  cudaStream_t st) {
  using Cf = FixCfg<N>;
  using G = FixGeo<float, N, Cf::C>;
  return with_kinds<N>(ax.pair, ay.pair, [&](auto px, auto py) {
    return cluster_start(k_xyfwd_fix<float, N, Cf::C, Cf::NTH, decltype(px)::value, decltype(py)::value, InF32>,
                         G::SMEM, g.nz, Cf::C, Cf::NTH, st, ax, ay, in, S, g, nrm);
  });
}

template <int N, typename Out>
cudaError_t inv_n(const AxisPlan &ax, const AxisPlan &ay, const float *S, const Out &out, const Geo &g,
                  cudaStream_t st) {
  using Cf = FixCfg<N>;
  using G = FixGeo<float, N, Cf::C>;
  return with_kinds<N>(ax.pair, ay.pair, [&](auto px, auto py) {
    return cluster_start(k_xyinv_fix<float, N, Cf::C, Cf::NTH, decltype(px)::value, decltype(py)::value, Out>,
                         G::SMEM, g.nz, Cf::C, Cf::NTH, st, ax, ay, S, out, g);
  });
}

// Co-resident clusters of the (N, PP, PP) inverse kernel: 0 when a cluster
// of the required size cannot be placed on this device.
template <int N> int capacity_n() {
  using Cf = FixCfg<N>;
  using G = FixGeo<float, N, Cf::C>;
  auto kernel = k_xyinv_fix<float, N, Cf::C, Cf::NTH, BC_PP, BC_PP, OutHalo>;
  if (prepare((const void *)kernel, G::SMEM, Cf::C)) return 0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)Cf::C);
  cfg.blockDim = dim3((unsigned)Cf::NTH);
  cfg.dynamicSmemBytes = G::SMEM;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)Cf::C;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, kernel, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

}  // namespace

bool fixed_supported(int nx, int ny, int C, int px, int py) {
  if (const char *e = getenv("FLUTAS_GB300_FIXED")) {  // 0 disables the fixed-size kernels (A/B timing)
    if (atoi(e) == 0) return false;
  }
  if (nx != ny || !kind_ok(px) || !kind_ok(py)) return false;
  return (nx == 256 && C == FixCfg<256>::C) || (nx == 512 && C == FixCfg<512>::C);
}

int fixed_cluster_size(int nx, int ny, int px, int py) {
  if (nx != ny || !kind_ok(px) || !kind_ok(py)) return 0;
  if (nx == 256) return capacity_n<256>() > 0 ? FixCfg<256>::C : 0;
  if (nx == 512) return capacity_n<512>() > 0 ? FixCfg<512>::C : 0;
  return 0;
}

cudaError_t xyfwd_fixed(const AxisPlan &ax, const AxisPlan &ay, const InF32 &in, float *S, const Geo &g,
                        double *nrm, int C, cudaStream_t st, bool *handled) {
  *handled = fixed_supported(g.nx, g.ny, C, ax.pair, ay.pair);
  if (!*handled) return cudaSuccess;
  return g.nx == 256 ? fwd_n<256>(ax, ay, in, S, g, nrm, st) : fwd_n<512>(ax, ay, in, S, g, nrm, st);
}
cudaError_t xyinv_fixed(const AxisPlan &ax, const AxisPlan &ay, const float *S, const OutHalo &out, const Geo &g,
                        int C, cudaStream_t st, bool *handled) {
  *handled = fixed_supported(g.nx, g.ny, C, ax.pair, ay.pair);
  if (!*handled) return cudaSuccess;
  return g.nx == 256 ? inv_n<256>(ax, ay, S, out, g, st) : inv_n<512>(ax, ay, S, out, g, st);
}
cudaError_t xyinv_fixed(const AxisPlan &ax, const AxisPlan &ay, const float *S, const OutHaloAdd &out, const Geo &g,
                        int C, cudaStream_t st, bool *handled) {
  *handled = fixed_supported(g.nx, g.ny, C, ax.pair, ay.pair);
  if (!*handled) return cudaSuccess;
  return g.nx == 256 ? inv_n<256>(ax, ay, S, out, g, st) : inv_n<512>(ax, ay, S, out, g, st);
}

}  // namespace fg
