// kernels.cuh -- sm_103a kernels of the FluTAS pressure-projection path.
//
//   x / y transform passes  : src/solver_cpu.f90:59,65,83,89 (FFTW r2r along x, y)
//   z tridiagonal solve      : src/solver_cpu.f90:71-77, gaussel 117-145,
//                              gaussel_periodic 147-185, dgtsv_homebrewed 187-223
//   fillps                   : src/fillps.f90:50-57
//   correc                   : src/correc.f90:57-60
//   boundp / set_bc          : src/bound.f90:146-646 (nh_p = 1, single domain)
//   updt_rhs_b               : src/bound.f90:829-944
//   chkdiv                   : src/chkdiv.f90:37-63
//   pres_tw_src              : src/source.f90:247-309 (constant-coefficient branch)
//   face-centred / odd DCT-IV: src/fft.f90:233-291 (extended-FFT kinds, fft_ext.cuh)
//
// Layouts (Fortran column-major, x fastest):
//   p-like fields  (0:nx+1, 0:ny+1, 0:nz+1)        double
//   velocities     (1-h:nx+h, 1-h:ny+h, 1-h:nz+h)   double, h = nh_u
//   spectral S     (nx, ny, nz) no halo             T (double or float)
#pragma once
#include <type_traits>
#include "fft_engine.cuh"
#include "fft_ext.cuh"
#include "bits.cuh"
#include "ghosts.cuh"

namespace fg {

// ------------------------------------------------------------------ indexing
struct Geo {
  int nx, ny, nz;
  int h;  // velocity halo nh_u
  FG_HD long pidx(int i, int j, int k) const {  // Fortran (i,j,k), halo 1
    return (long)i + (long)(nx + 2) * ((long)j + (long)(ny + 2) * (long)k);
  }
  FG_HD long uidx(int i, int j, int k) const {  // Fortran (i,j,k), halo h
    return (long)(i - 1 + h) + (long)(nx + 2 * h) * ((long)(j - 1 + h) + (long)(ny + 2 * h) * (long)(k - 1 + h));
  }
  FG_HD long sidx(int i0, int j0, int k0) const {  // 0-based, no halo
    return (long)i0 + (long)nx * ((long)j0 + (long)ny * (long)k0);
  }
};

// Cell loop of the stencil kernels: i along threads, j and k along grid y / z
// (no 64-bit division per cell).  Launch with grid_cells().
template <typename F> __device__ __forceinline__ void for_cells(const Geo &g, F &&f) {
  for (int k0 = blockIdx.z; k0 < g.nz; k0 += gridDim.z)
    for (int j0 = blockIdx.y; j0 < g.ny; j0 += gridDim.y)
      for (int i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 < g.nx; i0 += gridDim.x * blockDim.x) f(i0, j0, k0);
}
inline dim3 grid_cells(const Geo &g, int threads = 256) {
  int gx = (g.nx + threads - 1) / threads;
  return dim3(gx, g.ny < 65535 ? g.ny : 65535, g.nz < 65535 ? g.nz : 65535);
}

// Asynchronous global -> shared copies (no register staging: every copy a
// thread has issued is in flight at once) and an L2 prefetch of a contiguous
// span.  Copies of 4 and 8 bytes go through L1 (.ca), 16-byte ones bypass it.
template <int B> __device__ __forceinline__ void cp_async(void *dst, const void *src) {
  static_assert(B == 4 || B == 8 || B == 16, "cp.async copies 4, 8 or 16 bytes");
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  const size_t g = __cvta_generic_to_global(src);
  if constexpr (B == 16) asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(g) : "memory");
  else asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(d), "l"(g), "n"(B) : "memory");
}
__device__ __forceinline__ void cp_async4(void *dst, const void *src) { cp_async<4>(dst, src); }
__device__ __forceinline__ void cp_async16(void *dst, const void *src) { cp_async<16>(dst, src); }
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int PENDING> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(PENDING) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
// bytes: a multiple of 16 from a 16-byte aligned address (the caller checks)
__device__ __forceinline__ void prefetch_l2(const void *p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(__cvta_generic_to_global(p)), "r"(bytes)
               : "memory");
}

// Reciprocal in FP64: FP32 seed refined by two Newton-Raphson steps
// y <- y (2 - x y); each step squares the relative error (2^-22 -> 2^-44 -> ~1 ulp).
// The seed's conversions run on the integer ALUs (bits.cuh), so the FP64 pipe
// issues only the four Newton instructions.  Valid for arguments whose
// magnitude lies in FP32's normal range.
__device__ __forceinline__ double rcp64(double x) {
  double y = f64_of(__frcp_rn(f32_of(x)));
  y = y * fma(-x, y, 2.0);
  y = y * fma(-x, y, 2.0);
  return y;
}
// True when |x| lies in FP32's normal range (exponent bits only: no FP64 instruction).
__device__ __forceinline__ bool f32_range(double x) {
  const unsigned e = (hi_word(x) >> 20) & 0x7ffu;
  return e > 897u && e < 1150u;
}

// Value of an FP64 RHS in the arithmetic type of a pass, and the FP32 value
// used for the norms (integer-ALU conversions, bits.cuh).
template <typename T> __device__ __forceinline__ T to_pass(double v);
template <> __device__ __forceinline__ float to_pass<float>(double v) { return f32_of(v); }
template <> __device__ __forceinline__ double to_pass<double>(double v) { return v; }
__device__ __forceinline__ void to_pass_into(float &o, double v) { o = f32_of(v); }
__device__ __forceinline__ void to_pass_into(float &o, float v) { o = v; }
__device__ __forceinline__ void to_pass_into(double &o, double v) { o = v; }
__device__ __forceinline__ void to_pass_into(double &o, float v) { o = f64_of(v); }
__device__ __forceinline__ void to_pass_into(dd &o, double v) { o = dd_of(v); }
__device__ __forceinline__ void to_pass_into(dd &o, dd v) { o = v; }
// Storage <-> arithmetic of the z sweeps: the FP64 solver keeps its spectrum as
// double-float pairs (its transforms' type) and sweeps in FP64.
__device__ __forceinline__ double z_load(const dd &v) { return double_of(v); }
__device__ __forceinline__ double z_load(const double &v) { return v; }
__device__ __forceinline__ float z_load(const float &v) { return v; }
__device__ __forceinline__ void z_store(dd &o, double v) { o = dd_of(v); }
__device__ __forceinline__ void z_store(double &o, double v) { o = v; }
__device__ __forceinline__ void z_store(float &o, float v) { o = v; }
__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(double v) { return f32_of(v); }
__device__ __forceinline__ float to_f32(dd v) { return v.h; }

// CTAs per SM the transform kernels are compiled for: two (at most 128
// registers a thread) for FP32 and double-float, one for FP64.
template <typename T> constexpr int xf_minb() { return std::is_same<T, double>::value ? 1 : 2; }

// ------------------------------------------------------- forward input modes
// All take 0-based interior coordinates (i0,j0,k0) and return the RHS value.
struct InHalo {  // p(1:nx,1:ny,1:nz) of a halo-1 array
  static constexpr const char *tag = "halo";
  static constexpr const char *keep_tag = "keep-halo";
  const double *p;
  Geo g;
  __device__ double operator()(int i0, int j0, int k0) const { return p[g.pidx(i0 + 1, j0 + 1, k0 + 1)]; }
  __device__ void keep(int, int, int, double) const {}
};

struct InF32 {  // contiguous (nx,ny,nz) FP32 array (a RHS already evaluated by k_stencil_pass)
  static constexpr const char *tag = "f32";
  const float *f;
  Geo g;
  __device__ float operator()(int i0, int j0, int k0) const { return f[g.sidx(i0, j0, k0)]; }
  __device__ void keep(int, int, int, float) const {}
};

struct InPlain {  // contiguous (nx,ny,nz) FP64 array
  static constexpr const char *tag = "plain";
  const double *f;
  Geo g;
  __device__ double operator()(int i0, int j0, int k0) const { return f[g.sidx(i0, j0, k0)]; }
  __device__ void keep(int, int, int, double) const {}
};

struct InPlainDD {  // contiguous (nx,ny,nz) double-float array (the FP64 solver's spectrum)
  static constexpr const char *tag = "plain";
  const dd *f;
  Geo g;
  __device__ dd operator()(int i0, int j0, int k0) const { return f[g.sidx(i0, j0, k0)]; }
  __device__ void keep(int, int, int, dd) const {}
};

// fillps (src/fillps.f90:50-57) + optional updt_rhs_b (src/bound.f90:829-944).
// The factors dti*dzfi(k)*rho0, dti*dyi*rho0, dti*dxi*rho0 are folded (FP64
// instructions are the scarce resource on this GPU).
struct InFillps {
  static constexpr const char *tag = "fillps";
  static constexpr const char *keep_tag = "keep-fillps";
  const double *u, *v, *w;
  const double *cz;  // cz[k] = dti*dzfi(k)*rho0 for k = 1..nz (index k)
  double cy, cx;     // dti*dyi*rho0, dti*dxi*rho0
  const double *rhsbx, *rhsby, *rhsbz;  // nullable
  int q1, q2, q3;
  Geo g;
  __device__ double operator()(int i0, int j0, int k0) const {
    const int i = i0 + 1, j = j0 + 1, k = k0 + 1;
    const long c = g.uidx(i, j, k);
    const long sy = g.nx + 2 * g.h, sz = (long)(g.nx + 2 * g.h) * (g.ny + 2 * g.h);
    double val = fma(w[c] - w[c - sz], cz[k], fma(v[c] - v[c - sy], cy, (u[c] - u[c - 1]) * cx));
    if (rhsbx) {
      const int nx = g.nx, ny = g.ny, nz = g.nz;
      if (i == 1) val += rhsbx[(j - 1) + (long)ny * (k - 1)];
      if (i == nx - q1) val += rhsbx[(j - 1) + (long)ny * (k - 1) + (long)ny * nz];
      if (j == 1) val += rhsby[(i - 1) + (long)nx * (k - 1)];
      if (j == ny - q2) val += rhsby[(i - 1) + (long)nx * (k - 1) + (long)nx * nz];
      if (k == 1) val += rhsbz[(i - 1) + (long)nx * (j - 1)];
      if (k == nz - q3) val += rhsbz[(i - 1) + (long)nx * (j - 1) + (long)nx * ny];
    }
    return val;
  }
  __device__ void keep(int, int, int, double) const {}
};

// FP64 residual r = f - A x of the cell-centred 7-point operator that the
// solver inverts (ghost rules of src/initsolver.f90:188-246 tridmatrix and the
// x/y eigenvalues: P wrap, N p0=p1, D p0=-p1).  f and x are halo-1 arrays.
struct InResidual {
  static constexpr const char *tag = "residual";
  const double *f, *x;
  const double *zc;  // per level k (0-based): [3k] czm = dzfi*dzci(k-1), [3k+1] czp = dzfi*dzci(k), [3k+2] cc
  double dxi2, dyi2;
  char bc[6];
  Geo g;
  __device__ double ghost(char b, double pc, double pw) const { return b == 'P' ? pw : (b == 'N' ? pc : -pc); }
  __device__ double operator()(int i0, int j0, int k0) const {
    const int i = i0 + 1, j = j0 + 1, k = k0 + 1, nx = g.nx, ny = g.ny, nz = g.nz;
    const long c = g.pidx(i, j, k);
    const long sx = 1, sy = nx + 2, sz = (long)(nx + 2) * (ny + 2);
    const double pc = x[c];
    double pw, pe, ps, pn, pb, pt;
    if (i > 1 && i < nx && j > 1 && j < ny && k > 1 && k < nz) {
      pw = x[c - sx]; pe = x[c + sx]; ps = x[c - sy]; pn = x[c + sy]; pb = x[c - sz]; pt = x[c + sz];
    } else {
      pw = i > 1 ? x[c - sx] : ghost(bc[0], pc, x[g.pidx(nx, j, k)]);
      pe = i < nx ? x[c + sx] : ghost(bc[1], pc, x[g.pidx(1, j, k)]);
      ps = j > 1 ? x[c - sy] : ghost(bc[2], pc, x[g.pidx(i, ny, k)]);
      pn = j < ny ? x[c + sy] : ghost(bc[3], pc, x[g.pidx(i, 1, k)]);
      pb = k > 1 ? x[c - sz] : ghost(bc[4], pc, x[g.pidx(i, j, nz)]);
      pt = k < nz ? x[c + sz] : ghost(bc[5], pc, x[g.pidx(i, j, 1)]);
    }
    const double czm = zc[3 * k0], czp = zc[3 * k0 + 1], cc = zc[3 * k0 + 2];
    // f - A x accumulated into f: two adds and five FMAs (FP64 is the bound)
    double r = fma(-cc, pc, f[c]);
    r = fma(-dxi2, pe + pw, r);
    r = fma(-dyi2, pn + ps, r);
    r = fma(-czm, pb, r);
    return fma(-czp, pt, r);
  }
  __device__ void keep(int, int, int, double) const {}
};

// Wrapper: evaluates the inner RHS functor and keeps an FP64 copy of it in the
// interior of a halo-1 array (the RHS the mixed-precision residual needs).
// The loaders call keep() after the evaluations of a batch of cells.
template <typename Inner> struct InKeep {
  static constexpr const char *tag = Inner::keep_tag;
  Inner inner;
  double *kept;
  Geo g;  // halo-1 geometry of kept
  __device__ double operator()(int i0, int j0, int k0) const { return inner(i0, j0, k0); }
  __device__ void keep(int i0, int j0, int k0, double v) const { kept[g.pidx(i0 + 1, j0 + 1, k0 + 1)] = v; }
};

// ------------------------------------------------------ inverse output modes
struct OutHalo {  // p(i,j,k) = v * scale   (scale applied in the arithmetic type of the pass)
  static constexpr const char *tag = "halo";
  double *p;
  double scale;
  Geo g;
  __device__ void operator()(int i0, int j0, int k0, double v) const { p[g.pidx(i0 + 1, j0 + 1, k0 + 1)] = v * scale; }
  __device__ void operator()(int i0, int j0, int k0, float v) const {
    p[g.pidx(i0 + 1, j0 + 1, k0 + 1)] = f64_of(v * f32_of(scale));
  }
  __device__ void operator()(int i0, int j0, int k0, dd v) const { p[g.pidx(i0 + 1, j0 + 1, k0 + 1)] = double_of(v) * scale; }
  __device__ double pre(int, int, int) const { return 0.0; }
  __device__ void put(int i0, int j0, int k0, double, double v) const { (*this)(i0, j0, k0, v); }
  __device__ void put(int i0, int j0, int k0, double, float v) const { (*this)(i0, j0, k0, v); }
  __device__ void put(int i0, int j0, int k0, double, dd v) const { (*this)(i0, j0, k0, v); }
};
struct OutPlain {  // the contiguous (nx,ny,nz) spectral array itself (an in-place inverse pass)
  static constexpr const char *tag = "plain";
  double *s;
  Geo g;
  __device__ void operator()(int i0, int j0, int k0, double v) const { s[g.sidx(i0, j0, k0)] = v; }
  __device__ double pre(int, int, int) const { return 0.0; }
  __device__ void put(int i0, int j0, int k0, double, double v) const { (*this)(i0, j0, k0, v); }
};
struct OutHaloAdd {  // p(i,j,k) += v * scale  (iterative-refinement update, accumulated in FP64)
  static constexpr const char *tag = "haloadd";
  double *p;
  double scale;
  Geo g;
  __device__ void operator()(int i0, int j0, int k0, double v) const { p[g.pidx(i0 + 1, j0 + 1, k0 + 1)] += v * scale; }
  __device__ void operator()(int i0, int j0, int k0, float v) const {
    p[g.pidx(i0 + 1, j0 + 1, k0 + 1)] += f64_of(v * f32_of(scale));
  }
  __device__ double pre(int i0, int j0, int k0) const { return p[g.pidx(i0 + 1, j0 + 1, k0 + 1)]; }
  __device__ void put(int i0, int j0, int k0, double old, double v) const {
    p[g.pidx(i0 + 1, j0 + 1, k0 + 1)] = old + v * scale;
  }
  __device__ void put(int i0, int j0, int k0, double old, float v) const {
    p[g.pidx(i0 + 1, j0 + 1, k0 + 1)] = old + f64_of(v * f32_of(scale));
  }
};

// ---------------------------------------------------------------------------
// Batched global loads and stores of the transform kernels.  Each thread
// evaluates BATCH_U cells before it stores any of them, so that the loads of
// BATCH_U cells are in flight together: a store between two evaluations would
// keep the compiler from hoisting the later loads (it cannot prove that they do
// not alias the store).  coord(idx, x, y, k) maps a slab index to 0-based
// interior coordinates and returns false for padding entries.
// ---------------------------------------------------------------------------
constexpr int BATCH_U = 4;

template <typename T, typename In, typename Coord, typename Dst>
__device__ __forceinline__ void load_cells(const In &in, int tot, const Coord &coord, const Dst &dst, float &ss) {
  const int tid = threadIdx.x, nth = blockDim.x;
  using V = decltype(in(0, 0, 0));  // double (FP64 functors) or float (InF32)
  for (int b = tid; b < tot; b += BATCH_U * nth) {
    V v[BATCH_U];
    int xs[BATCH_U], ys[BATCH_U], ks[BATCH_U];
    bool ok[BATCH_U];
#pragma unroll
    for (int u = 0; u < BATCH_U; u++) {
      const int idx = b + u * nth;
      ok[u] = idx < tot && coord(idx, xs[u], ys[u], ks[u]);
      v[u] = ok[u] ? in(xs[u], ys[u], ks[u]) : (V)0;
    }
#pragma unroll
    for (int u = 0; u < BATCH_U; u++) {
      const int idx = b + u * nth;
      if (idx < tot) {
        if (ok[u]) in.keep(xs[u], ys[u], ks[u], v[u]);
        T t;
        to_pass_into(t, v[u]);
        const float f = to_f32(t);
        ss = fmaf(f, f, ss);
        dst(idx, t);
      }
    }
  }
}

template <typename T, typename Out, typename Coord, typename Src>
__device__ __forceinline__ void store_cells(const Out &out, int tot, const Coord &coord, const Src &src) {
  const int tid = threadIdx.x, nth = blockDim.x;
  for (int b = tid; b < tot; b += BATCH_U * nth) {
    double old[BATCH_U];
    int xs[BATCH_U], ys[BATCH_U], ks[BATCH_U];
    bool ok[BATCH_U];
#pragma unroll
    for (int u = 0; u < BATCH_U; u++) {
      const int idx = b + u * nth;
      ok[u] = idx < tot && coord(idx, xs[u], ys[u], ks[u]);
      old[u] = ok[u] ? out.pre(xs[u], ys[u], ks[u]) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < BATCH_U; u++) {
      const int idx = b + u * nth;
      if (ok[u]) out.put(xs[u], ys[u], ks[u], old[u], (T)src(idx));
    }
  }
}

// ---------------------------------------------------------------- smem sizes
template <typename T> FG_HD size_t align_up(size_t b) { return (b + 255) & ~(size_t)255; }

// Row-batch geometry for the x pass: M rows (even) of length nx, pitch P.
// The FP32 transform kernels are held to 128 registers (two 256-thread CTAs
// per SM, no spills); the FP64 ones keep up to 255 (they spill at 128).
FG_HD int xpitch(int nx) { return nx + 1; }

// ===========================================================================
// x pass (forward): rows -> spectral rows.  One CTA handles M rows at a time.
// ===========================================================================
template <typename T>
struct StoreRowsS {  // store into S rows: line l of this batch -> global row row0+l
  T *S;
  long row0, rows;
  int nx;
  __device__ void pair(int c, int t, T v0, T v1) {
    const long r0 = row0 + 2 * c;
    if (r0 < rows) S[r0 * nx + t] = v0;
    if (r0 + 1 < rows) S[(r0 + 1) * nx + t] = v1;
  }
  __device__ void single(int c, int t, T v) {
    const long r = row0 + c;
    if (r < rows) S[r * nx + t] = v;
  }
};

template <typename T>
struct StorePlaneReal {  // write real plane (row-major y*pitch + x)
  T *R;
  int pitch, rowbase;  // line l = row rowbase + l for x lines
  __device__ void pair(int c, int t, T v0, T v1) {
    R[(2 * c) * pitch + t] = v0;
    R[(2 * c + 1) * pitch + t] = v1;
  }
  __device__ void single(int c, int t, T v) { R[c * pitch + t] = v; }
};

// Block sum of v, added atomically to *acc (all threads of the block call it).
__device__ __forceinline__ void block_sum_add(double v, double *acc) {
  __shared__ double part[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) part[wid] = v;
  __syncthreads();
  if (wid == 0) {
    v = lane < (int)(blockDim.x >> 5) ? part[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) atomicAdd(acc, v);
  }
}

// Stencil pass ahead of a transform: evaluates an FP64 RHS functor (fillps,
// or the residual f - A x) per cell, optionally keeps the FP64 value (halo-1
// array `keep`) and writes the value in the transform's type into `s32` (no
// halo, x fastest: the input of the transform, which may run in place; FP32
// values truncated), and adds the
// FP32 sum of squares of the FP32 values to *nrm (as the fused norms of the
// transform passes).  With keep = s32 = nullptr it is the norm-only check.
// Four cells per thread are evaluated before any is stored.
template <typename In, typename TO, typename IDX = int>
__global__ void __launch_bounds__(256) k_stencil_pass(In in, Geo g, double *keep, TO *s32, double *nrm) {
  // IDX = int while nx*ny*nz < 2^31 (shift/multiply divisions), long long beyond
  const IDX tot = (IDX)g.nx * g.ny * g.nz;
  const FastDiv fx(g.nx), fy(g.ny);
  float ss = 0.0f;
  for (IDX b = (IDX)blockIdx.x * blockDim.x * 4 + threadIdx.x; b < tot; b += (IDX)gridDim.x * blockDim.x * 4) {
    double v[4];
    int xs[4], ys[4], ks[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const IDX idx = b + (IDX)u * blockDim.x;
      int row;
      if constexpr (sizeof(IDX) == 4) {
        row = fx.div((int)idx);
        xs[u] = (int)idx - row * g.nx;
      } else {
        const IDX r = idx / g.nx;  // rows stay below 2^31 (ny*nz)
        row = (int)r;
        xs[u] = (int)(idx - r * g.nx);
      }
      const int k = fy.div(row);
      ks[u] = k;
      ys[u] = row - k * g.ny;
      v[u] = idx < tot ? in(xs[u], ys[u], ks[u]) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const IDX idx = b + (IDX)u * blockDim.x;
      const float f = f32_of(v[u]);
      ss = fmaf(f, f, ss);
      if (idx < tot) {
        if (keep) keep[g.pidx(xs[u] + 1, ys[u] + 1, ks[u] + 1)] = v[u];
        if (s32) {
          TO o;
          to_pass_into(o, v[u]);  // the FP32 value for FP32 transforms, the FP64 value itself otherwise
          s32[idx] = o;
        }
      }
    }
  }
  if (nrm) block_sum_add((double)ss, nrm);
}


// One tile of the x pass: M rows starting at global row row0 (row = j + ny*k).
// smem: M*P reals + M*nx reals.  Accumulates the squares of the inputs in ss.
template <typename T, typename In>
__device__ __forceinline__ void xfwd_tile(const AxisPlan &ax, const In &in, T *S, const Geo &g, int M, long row0,
                                          unsigned char *smem, float &ss) {
  const int nx = g.nx, P = xpitch(nx);
  T *A = (T *)smem;
  C2<T> *C1 = (C2<T> *)(smem + align_up<T>(sizeof(T) * (size_t)M * P));
  C2<T> *C2b = (C2<T> *)A;  // ping-pong partner aliases the input rows
  const long rows = (long)g.ny * g.nz;
  const int tid = threadIdx.x, nth = blockDim.x;
  const int B = cbatch(ax.pair, M);
  {
    const FastDiv fnx(nx), fny(g.ny);
    const int r0 = (int)row0, nrows = (int)rows;  // ny*nz < 2^31
    load_cells<T>(
        in, M * nx,
        [&](int idx, int &x, int &y, int &k) -> bool {
          const int m = fnx.div(idx), r = r0 + m;
          x = idx - m * nx;
          k = fny.div(r);
          y = r - k * g.ny;
          return r < nrows;
        },
        [&](int idx, T t) { A[idx + fnx.div(idx)] = t; }, ss);
  }
  __syncthreads();
  pre_fwd<T>(ax, A, P, 1, M, C1, B, tid, nth);
  __syncthreads();
  C2<T> *cur = C1, *nxt = C2b;
  int Ns = 1;
  for (int s = 0; s < ax.nst; s++) {
    stage_dispatch<T, false>(ax.radix[s], cur, nxt, ax.N, B, B, Ns, (const C2<T> *)ax.W, tid, nth);
    Ns *= ax.radix[s];
    C2<T> *t = cur; cur = nxt; nxt = t;
    __syncthreads();
  }
  StoreRowsS<T> st{S, row0, rows, nx};
  post_fwd<T>(ax, cur, B, M, st, tid, nth);
  __syncthreads();
}

template <typename T, typename In>
__global__ void __launch_bounds__(256, xf_minb<T>()) k_xfwd(AxisPlan ax, In in, T *S, Geo g, int M, double *nrm) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const long rows = (long)g.ny * g.nz;
  float ss = 0.0f;  // sum of squares for convergence checks (FP32 per thread)
  for (long row0 = (long)blockIdx.x * M; row0 < rows; row0 += (long)gridDim.x * M)
    xfwd_tile<T, In>(ax, in, S, g, M, row0, smem_raw, ss);
  if (nrm) block_sum_add((double)ss, nrm);
}

// x pass (inverse): spectral rows -> output functor, times normfft

template <typename T, typename Out>
__device__ __forceinline__ void xinv_tile(const AxisPlan &ax, const T *S, const Out &out, const Geo &g, int M,
                                          long row0, unsigned char *smem) {
  const int nx = g.nx, P = xpitch(nx);
  T *A = (T *)smem;
  C2<T> *C1 = (C2<T> *)(smem + align_up<T>(sizeof(T) * (size_t)M * P));
  C2<T> *C2b = (C2<T> *)A;
  const long rows = (long)g.ny * g.nz;
  const int tid = threadIdx.x, nth = blockDim.x;
  const int B = cbatch(ax.pair, M);
  const bool inv = fft_inverse(ax.pair, true);
  for (int idx = tid; idx < M * nx; idx += nth) {
    const int m = idx / nx, x = idx % nx;
    const long r = row0 + m;
    A[m * P + x] = r < rows ? S[r * nx + x] : (T)0;
  }
  __syncthreads();
  pre_bwd<T>(ax, A, P, 1, M, C1, B, tid, nth);
  __syncthreads();
  C2<T> *cur = C1, *nxt = C2b;
  int Ns = 1;
  for (int s = 0; s < ax.nst; s++) {
    if (inv) stage_dispatch<T, true>(ax.radix[s], cur, nxt, ax.N, B, B, Ns, (const C2<T> *)ax.W, tid, nth);
    else stage_dispatch<T, false>(ax.radix[s], cur, nxt, ax.N, B, B, Ns, (const C2<T> *)ax.W, tid, nth);
    Ns *= ax.radix[s];
    C2<T> *t = cur; cur = nxt; nxt = t;
    __syncthreads();
  }
  // real rows into the free buffer, then the batched epilogue
  T *R = (cur == C1) ? A : (T *)C1;
  const int PR = (cur == C1) ? P : nx;
  StorePlaneReal<T> sr{R, PR, 0};
  post_bwd<T>(ax, cur, B, M, sr, tid, nth);
  __syncthreads();
  {
    const FastDiv fnx(nx), fny(g.ny);
    const int r0 = (int)row0, nrows = (int)rows;
    store_cells<T>(
        out, M * nx,
        [&](int idx, int &x, int &y, int &k) -> bool {
          const int m = fnx.div(idx), r = r0 + m;
          x = idx - m * nx;
          k = fny.div(r);
          y = r - k * g.ny;
          return r < nrows;
        },
        [&](int idx) { const int m = fnx.div(idx); return R[m * PR + (idx - m * nx)]; });
  }
  __syncthreads();
}

template <typename T, typename Out>
__global__ void __launch_bounds__(256, xf_minb<T>()) k_xinv(AxisPlan ax, const T *S, Out out, Geo g, int M) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const long rows = (long)g.ny * g.nz;
  for (long row0 = (long)blockIdx.x * M; row0 < rows; row0 += (long)gridDim.x * M)
    xinv_tile<T, Out>(ax, S, out, g, M, row0, smem_raw);
}

// ===========================================================================
// y pass: a tile of W columns (all ny rows) of one z-plane.  S -> S.
// ===========================================================================
template <typename T>
struct StoreColsS {  // line l of the tile = column x0+l; position t = row y
  T *S;
  long plane_off;
  int nx, x0, W;
  __device__ void pair(int c, int t, T v0, T v1) {
    const int x = x0 + 2 * c;
    T *dst = S + plane_off + (long)t * nx + x;
    if (2 * c + 1 < W) { dst[0] = v0; dst[1] = v1; }
    else if (2 * c < W) dst[0] = v0;
  }
  __device__ void single(int c, int t, T v) {
    if (c < W) S[plane_off + (long)t * nx + x0 + c] = v;
  }
};

// One tile of the y pass: columns [x0, x0+W) of plane k, all ny rows.
template <typename T, bool BACKWARD>
__device__ __forceinline__ void ypass_tile(const AxisPlan &ay, T *S, const Geo &g, int W, long tile,
                                           unsigned char *smem) {
  const int ny = g.ny, nx = g.nx;
  T *A = (T *)smem;  // ny rows x W
  C2<T> *C1 = (C2<T> *)(smem + align_up<T>(sizeof(T) * (size_t)W * ny));
  C2<T> *C2b = (C2<T> *)A;
  const int tid = threadIdx.x, nth = blockDim.x;
  const int tiles_x = (nx + W - 1) / W;
  const int B = cbatch(ay.pair, W);
  const bool inv = fft_inverse(ay.pair, BACKWARD);
  const int tx = (int)(tile % tiles_x), k = (int)(tile / tiles_x);
  const int x0 = tx * W, Wv = min(W, nx - x0);
  const long off = (long)k * nx * ny;
  for (int idx = tid; idx < W * ny; idx += nth) {
    const int y = idx / W, xx = idx % W;
    A[idx] = xx < Wv ? S[off + (long)y * nx + x0 + xx] : (T)0;
  }
  __syncthreads();
  if (BACKWARD) pre_bwd<T>(ay, A, 1, W, W, C1, B, tid, nth);
  else pre_fwd<T>(ay, A, 1, W, W, C1, B, tid, nth);
  __syncthreads();
  C2<T> *cur = C1, *nxt = C2b;
  int Ns = 1;
  for (int s = 0; s < ay.nst; s++) {
    if (inv) stage_dispatch<T, true>(ay.radix[s], cur, nxt, ay.N, B, B, Ns, (const C2<T> *)ay.W, tid, nth);
    else stage_dispatch<T, false>(ay.radix[s], cur, nxt, ay.N, B, B, Ns, (const C2<T> *)ay.W, tid, nth);
    Ns *= ay.radix[s];
    C2<T> *t = cur; cur = nxt; nxt = t;
    __syncthreads();
  }
  StoreColsS<T> st{S, off, nx, x0, Wv};
  if (BACKWARD) post_bwd<T>(ay, cur, B, W, st, tid, nth);
  else post_fwd<T>(ay, cur, B, W, st, tid, nth);
  __syncthreads();
}

template <typename T, bool BACKWARD>
__global__ void __launch_bounds__(256, xf_minb<T>()) k_ypass(AxisPlan ay, T *S, Geo g, int W) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const long ntiles = (long)((g.nx + W - 1) / W) * g.nz;
  for (long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) ypass_tile<T, BACKWARD>(ay, S, g, W, tile, smem_raw);
}

// ===========================================================================
// Fused x+y plane pass (one CTA owns a whole z-plane in shared memory).
// Forward: In -> x transform -> y transform -> S.
// Inverse: S -> y^-1 -> x^-1 -> Out.
// Shared memory: two buffers of nx*ny reals (plus row padding of the first).
// ===========================================================================
template <typename T>
struct StorePlaneRealCols {  // columns as lines: line l = column l, position t = row
  T *R;
  int pitch;
  __device__ void pair(int c, int t, T v0, T v1) {
    R[t * pitch + 2 * c] = v0;
    R[t * pitch + 2 * c + 1] = v1;
  }
  __device__ void single(int c, int t, T v) { R[t * pitch + c] = v; }
};

template <typename T, bool INV>
__device__ __forceinline__ C2<T> *run_stages(const AxisPlan &ap, C2<T> *cur, C2<T> *nxt, int B, int tid, int nth) {
  int Ns = 1;
  for (int s = 0; s < ap.nst; s++) {
    stage_dispatch<T, INV>(ap.radix[s], cur, nxt, ap.N, B, B, Ns, (const C2<T> *)ap.W, tid, nth);
    Ns *= ap.radix[s];
    C2<T> *t = cur; cur = nxt; nxt = t;
    __syncthreads();
  }
  return cur;
}

// Both transforms of one z-plane k in one CTA's shared memory (ny x P + nx*ny
// reals); accumulates the squares of the inputs in ss.
template <typename T, typename In>
__device__ __forceinline__ void xyfwd_plane_tile(const AxisPlan &ax, const AxisPlan &ay, const In &in, T *S,
                                                 const Geo &g, int k, unsigned char *smem, float &ss) {
  const int nx = g.nx, ny = g.ny, P = xpitch(nx);
  T *A = (T *)smem;  // ny x P
  T *Bu = (T *)(smem + align_up<T>(sizeof(T) * (size_t)ny * P));  // nx*ny reals
  const int tid = threadIdx.x, nth = blockDim.x;
  const FastDiv fnx(nx);
  load_cells<T>(
      in, nx * ny,
      [&](int idx, int &x, int &y, int &kk) -> bool {
        y = fnx.div(idx);
        x = idx - y * nx;
        kk = k;
        return true;
      },
      [&](int idx, T t) { A[idx + fnx.div(idx)] = t; }, ss);
  __syncthreads();
  // ---- x transform: lines = rows of A
  const int Bx = cbatch(ax.pair, ny);
  pre_fwd<T>(ax, A, P, 1, ny, (C2<T> *)Bu, Bx, tid, nth);
  __syncthreads();
  C2<T> *fin = run_stages<T, false>(ax, (C2<T> *)Bu, (C2<T> *)A, Bx, tid, nth);
  T *G = (fin == (C2<T> *)Bu) ? A : Bu;   // free buffer for the real x-spectrum
  const int gp = (G == A) ? P : nx;
  StorePlaneReal<T> sx{G, gp, 0};
  post_fwd<T>(ax, fin, Bx, ny, sx, tid, nth);
  __syncthreads();
  // ---- y transform: lines = columns of G
  const int By = cbatch(ay.pair, nx);
  C2<T> *F = (C2<T> *)(G == A ? Bu : A);
  pre_fwd<T>(ay, G, 1, gp, nx, F, By, tid, nth);
  __syncthreads();
  C2<T> *fy = run_stages<T, false>(ay, F, (C2<T> *)G, By, tid, nth);
  StoreColsS<T> st{S, (long)k * nx * ny, nx, 0, nx};
  post_fwd<T>(ay, fy, By, nx, st, tid, nth);
  __syncthreads();
}

template <typename T, typename In>
__global__ void __launch_bounds__(512) k_xyfwd_plane(AxisPlan ax, AxisPlan ay, In in, T *S, Geo g, double *nrm) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float ss = 0.0f;  // sum of squares for convergence checks (FP32 per thread)
  for (int k = blockIdx.x; k < g.nz; k += gridDim.x) xyfwd_plane_tile<T, In>(ax, ay, in, S, g, k, smem_raw, ss);
  if (nrm) block_sum_add((double)ss, nrm);
}

// Both inverse transforms of one z-plane k in one CTA's shared memory.
template <typename T, typename Out>
__device__ __forceinline__ void xyinv_plane_tile(const AxisPlan &ax, const AxisPlan &ay, const T *S, const Out &out,
                                                 const Geo &g, int k, unsigned char *smem) {
  const int nx = g.nx, ny = g.ny, P = xpitch(nx);
  T *A = (T *)smem;
  T *Bu = (T *)(smem + align_up<T>(sizeof(T) * (size_t)ny * P));
  const int tid = threadIdx.x, nth = blockDim.x;
  const bool invx = fft_inverse(ax.pair, true), invy = fft_inverse(ay.pair, true);
  const T *Sp = S + (long)k * nx * ny;
  for (int idx = tid; idx < nx * ny; idx += nth) {
    const int y = idx / nx, x = idx % nx;
    A[y * P + x] = Sp[idx];
  }
  __syncthreads();
  // ---- y^-1: lines = columns of A
  const int By = cbatch(ay.pair, nx);
  pre_bwd<T>(ay, A, 1, P, nx, (C2<T> *)Bu, By, tid, nth);
  __syncthreads();
  C2<T> *fy = invy ? run_stages<T, true>(ay, (C2<T> *)Bu, (C2<T> *)A, By, tid, nth)
                   : run_stages<T, false>(ay, (C2<T> *)Bu, (C2<T> *)A, By, tid, nth);
  T *G = (fy == (C2<T> *)Bu) ? A : Bu;
  const int gp = (G == A) ? P : nx;
  StorePlaneRealCols<T> sy{G, gp};
  post_bwd<T>(ay, fy, By, nx, sy, tid, nth);
  __syncthreads();
  // ---- x^-1: lines = rows of G
  const int Bx = cbatch(ax.pair, ny);
  C2<T> *F = (C2<T> *)(G == A ? Bu : A);
  pre_bwd<T>(ax, G, gp, 1, ny, F, Bx, tid, nth);
  __syncthreads();
  C2<T> *fx = invx ? run_stages<T, true>(ax, F, (C2<T> *)G, Bx, tid, nth)
                   : run_stages<T, false>(ax, F, (C2<T> *)G, Bx, tid, nth);
  // real plane into the free buffer, then the batched epilogue
  T *R = (fx == F) ? G : (T *)F;
  const int PR = (R == A) ? P : nx;
  StorePlaneReal<T> sr{R, PR, 0};
  post_bwd<T>(ax, fx, Bx, ny, sr, tid, nth);
  __syncthreads();
  const FastDiv fnx(nx);
  store_cells<T>(
      out, nx * ny,
      [&](int idx, int &x, int &y, int &kk) -> bool {
        y = fnx.div(idx);
        x = idx - y * nx;
        kk = k;
        return true;
      },
      [&](int idx) { const int y = fnx.div(idx); return R[y * PR + (idx - y * nx)]; });
  __syncthreads();
}

template <typename T, typename Out>
__global__ void __launch_bounds__(512) k_xyinv_plane(AxisPlan ax, AxisPlan ay, const T *S, Out out, Geo g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  for (int k = blockIdx.x; k < g.nz; k += gridDim.x) xyinv_plane_tile<T, Out>(ax, ay, S, out, g, k, smem_raw);
}

// ===========================================================================
// z solve: Thomas per (kx,ky) column (src/solver_cpu.f90:117-223).
// A CTA stages TC consecutive columns (all nz levels) in shared memory.
// Columns are indexed q = kx + nx*ky; element (q,k) at S[q + nx*ny*k].
// ===========================================================================
struct ZArgs {
  const double *a, *b, *c;   // tridmatrix coefficients (nz), FP64
  const void *at, *bt, *ct;  // the same, rounded to the arithmetic type of the kernel
  const double *lam;         // lambdaxy (nx*ny)
  int nq;                    // nx*ny columns
  int nz;                    // full nz
  int nn;                    // nz - q   (solver_cpu.f90:71-72)
  int periodic;              // bcz == 'PP'
  int pin;                   // 1: the singular (lam == 0) column of an N/P z problem is pinned
  int *nonfinite;            // nullable: set to 1 when a column's solution is not finite
};

// A non-finite value anywhere in a column (or in the z-plane transforms that
// fed it) reaches the column's level-0 solution through the forward
// elimination and the back substitution: checking that one value per column
// flags a NaN/Inf input of the solve.
template <typename T> __device__ __forceinline__ void flag_nonfinite(const ZArgs &za, T x0) {
  if (za.nonfinite && !isfinite((double)x0)) atomicOr(za.nonfinite, 1);
}

// Thomas on a column in shared memory (stride ts), in place; d scratch (stride ts).
// T is the arithmetic type.  Follows dgtsv_homebrewed step by step.
template <typename T, typename St>
__device__ __forceinline__ void thomas_col(int n, const double *a, const double *b, const double *c,
                                           double lam, St *p, St *d, int ts, bool pin_last) {
  T z = (T)1 / (T)(b[0] + lam);
  d[0] = (St)((T)c[0] * z);
  p[0] = (St)((T)p[0] * z);
  for (int l = 1; l < n - 1; l++) {
    z = (T)1 / ((T)(b[l] + lam) - (T)a[l] * (T)d[(l - 1) * ts]);
    d[l * ts] = (St)((T)c[l] * z);
    p[l * ts] = (St)(((T)p[l * ts] - (T)a[l] * (T)p[(l - 1) * ts]) * z);
  }
  T zl = (T)(b[n - 1] + lam) - (T)a[n - 1] * (T)d[(n - 2) * ts];
  if (zl != (T)0 && !pin_last) p[(n - 1) * ts] = (St)(((T)p[(n - 1) * ts] - (T)a[n - 1] * (T)p[(n - 2) * ts]) / zl);
  else p[(n - 1) * ts] = (St)0;
  for (int l = n - 2; l >= 0; l--) p[l * ts] = (St)((T)p[l * ts] - (T)d[l * ts] * (T)p[(l + 1) * ts]);
}

template <typename T, typename ST = T>
__global__ void __launch_bounds__(128) k_zsolve(ZArgs za, ST *S) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int TC = blockDim.x, nz = za.nz, tid = threadIdx.x;
  T *col = (T *)smem_raw;        // nz x TC
  T *dsc = col + (long)nz * TC;  // nz x TC
  T *p2 = dsc + (long)nz * TC;   // nz x TC (periodic only)
  const long plane = za.nq;
  for (long q0 = (long)blockIdx.x * TC; q0 < za.nq; q0 += (long)gridDim.x * TC) {
    const int tcv = (int)min((long)TC, za.nq - q0);
    for (int idx = tid; idx < nz * TC; idx += TC) {
      const int k = idx / TC, t = idx % TC;
      if (t < tcv) col[idx] = z_load(S[q0 + t + plane * k]);
    }
    __syncthreads();
    if (tid < tcv) {
      const long q = q0 + tid;
      const double lam = za.lam[q];
      T *pc = col + tid, *dc = dsc + tid;
      const int n = za.nn;
      if (!za.periodic) {
        const bool pin = za.pin && lam == 0.0;
        thomas_col<T, T>(n, za.a, za.b, za.c, lam, pc, dc, TC, pin);
      } else {
        // gaussel_periodic (solver_cpu.f90:147-185)
        T *p2c = p2 + tid;
        for (int k = 0; k < n; k++) p2c[k * TC] = (T)0;
        p2c[0] = (T)(-za.a[0]);
        p2c[(n - 2) * TC] = (T)(-za.c[n - 2]);
        thomas_col<T, T>(n - 1, za.a, za.b, za.c, lam, pc, dc, TC, false);
        thomas_col<T, T>(n - 1, za.a, za.b, za.c, lam, p2c, dc, TC, false);
        const T num = (T)pc[(n - 1) * TC] - (T)za.c[n - 1] * (T)pc[0] - (T)za.a[n - 1] * (T)pc[(n - 2) * TC];
        const T den = (T)(za.b[n - 1] + lam) + (T)za.c[n - 1] * (T)p2c[0] + (T)za.a[n - 1] * (T)p2c[(n - 2) * TC];
        const bool pin = (za.pin && lam == 0.0) || den == (T)0;
        const T pn = pin ? (T)0 : num / den;
        pc[(n - 1) * TC] = pn;
        for (int k = 0; k < n - 1; k++) pc[k * TC] = (T)pc[k * TC] + (T)p2c[k * TC] * pn;
      }
      flag_nonfinite(za, (T)pc[0]);
    }
    __syncthreads();
    for (int idx = tid; idx < nz * TC; idx += TC) {
      const int k = idx / TC, t = idx % TC;
      if (t < tcv) z_store(S[q0 + t + plane * k], col[idx]);
    }
    __syncthreads();
  }
}

// ===========================================================================
// Stencil kernels (drop-in entry points).  One thread per interior cell.
// ===========================================================================
#ifndef FG_NO_PLAIN_KERNELS
__global__ void k_fillps(InFillps in, double *p) {
  const Geo &g = in.g;
  for_cells(g, [&](int i0, int j0, int k0) { p[g.pidx(i0 + 1, j0 + 1, k0 + 1)] = in(i0, j0, k0); });
}
#endif

struct CorrecArgs {
  const double *p, *dzci;  // dzci offset: dzci[k] = dzci(k)
  double *u, *v, *w;
  double factori, factorj, dt, rho0i;
  Geo g;
};
#ifndef FG_NO_PLAIN_KERNELS
__global__ void k_correc(CorrecArgs a) {
  // src/correc.f90:57-60
  const Geo &g = a.g;
  for_cells(g, [&](int i0, int j0, int k0) {
    const int i = i0 + 1, j = j0 + 1, k = k0 + 1;
    const double pc = a.p[g.pidx(i, j, k)];
    const long ui = g.uidx(i, j, k);
    a.u[ui] = a.u[ui] - a.factori * (a.p[g.pidx(i + 1, j, k)] - pc) * a.rho0i;
    a.v[ui] = a.v[ui] - a.factorj * (a.p[g.pidx(i, j + 1, k)] - pc) * a.rho0i;
    a.w[ui] = a.w[ui] - a.dt * a.dzci[k] * (a.p[g.pidx(i, j, k + 1)] - pc) * a.rho0i;
  });
}
#endif

// boundp for one direction: set_bc (src/bound.f90:227-646), centred, nh_p = 1.
struct BoundArgs {
  double *p;
  Geo g;
  int idir;           // 1,2,3
  char ctype0, ctype1;
  double f0, s0, f1, s1;  // ghost = f + s * inner
};
#ifndef FG_NO_PLAIN_KERNELS
__global__ void k_boundp_dir(BoundArgs a) {
  const Geo &g = a.g;
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  long n1, n2;
  if (a.idir == 1) { n1 = ny + 2; n2 = nz + 2; }
  else if (a.idir == 2) { n1 = nx + 2; n2 = nz + 2; }
  else { n1 = nx + 2; n2 = ny + 2; }
  const long N = n1 * n2;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < N; t += (long)gridDim.x * blockDim.x) {
    const int s = (int)(t % n1), r = (int)(t / n1);
    long lo, lo_in, hi, hi_in, lo_wrap, hi_wrap;
    if (a.idir == 1) {
      lo = g.pidx(0, s, r); lo_in = g.pidx(1, s, r); hi = g.pidx(nx + 1, s, r); hi_in = g.pidx(nx, s, r);
    } else if (a.idir == 2) {
      lo = g.pidx(s, 0, r); lo_in = g.pidx(s, 1, r); hi = g.pidx(s, ny + 1, r); hi_in = g.pidx(s, ny, r);
    } else {
      lo = g.pidx(s, r, 0); lo_in = g.pidx(s, r, 1); hi = g.pidx(s, r, nz + 1); hi_in = g.pidx(s, r, nz);
    }
    lo_wrap = hi_in; hi_wrap = lo_in;  // periodic copies: p(0)=p(n), p(n+1)=p(1)
    double plo, phi;
    if (a.ctype0 == 'P') plo = a.p[lo_wrap]; else plo = a.f0 + a.s0 * a.p[lo_in];
    if (a.ctype1 == 'P') phi = a.p[hi_wrap]; else phi = a.f1 + a.s1 * a.p[hi_in];
    a.p[lo] = plo;
    a.p[hi] = phi;
  }
}
#endif

// divergence check: per-block partial (sum, max) in double
struct DivArgs {
  const double *u, *v, *w, *dzfi;  // dzfi[k] = dzfi(k)
  double dxi, dyi;
  Geo g;
};
#ifndef FG_NO_PLAIN_KERNELS
__global__ void k_chkdiv(DivArgs a, double *partial) {
  const Geo &g = a.g;
  double tot = 0.0, mx = 0.0;
  for_cells(g, [&](int i0, int j0, int k0) {
    const int i = i0 + 1, j = j0 + 1, k = k0 + 1;
    const double div = (a.w[g.uidx(i, j, k)] - a.w[g.uidx(i, j, k - 1)]) * a.dzfi[k] +
                       (a.v[g.uidx(i, j, k)] - a.v[g.uidx(i, j - 1, k)]) * a.dyi +
                       (a.u[g.uidx(i, j, k)] - a.u[g.uidx(i - 1, j, k)]) * a.dxi;
    tot += div;
    mx = fmax(mx, fabs(div));
  });
  __shared__ double s_tot[32], s_mx[32];
  for (int o = 16; o > 0; o >>= 1) {
    tot += __shfl_down_sync(0xffffffffu, tot, o);
    mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { s_tot[wid] = tot; s_mx[wid] = mx; }
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    tot = lane < nw ? s_tot[lane] : 0.0;
    mx = lane < nw ? s_mx[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      tot += __shfl_down_sync(0xffffffffu, tot, o);
      mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    }
    const long bid = blockIdx.x + (long)gridDim.x * (blockIdx.y + (long)gridDim.y * blockIdx.z);
    if (lane == 0) { partial[2 * bid] = tot; partial[2 * bid + 1] = mx; }
  }
}
#endif

}  // namespace fg

namespace fg {

// updt_rhs_b (src/bound.f90:829-944) for one direction: add rhs planes.
struct RhsbArgs {
  double *p;
  const double *rhs;  // (n1, n2, 0:1)
  Geo g;
  int idir, q;
};
#ifndef FG_NO_PLAIN_KERNELS
__global__ void k_updt_rhs_b_dir(RhsbArgs a) {
  const Geo &g = a.g;
  int n1, n2;
  if (a.idir == 1) { n1 = g.ny; n2 = g.nz; }
  else if (a.idir == 2) { n1 = g.nx; n2 = g.nz; }
  else { n1 = g.nx; n2 = g.ny; }
  const long N = (long)n1 * n2;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < N; t += (long)gridDim.x * blockDim.x) {
    const int s = (int)(t % n1) + 1, r = (int)(t / n1) + 1;
    long lo, hi;
    if (a.idir == 1) { lo = g.pidx(1, s, r); hi = g.pidx(g.nx - a.q, s, r); }
    else if (a.idir == 2) { lo = g.pidx(s, 1, r); hi = g.pidx(s, g.ny - a.q, r); }
    else { lo = g.pidx(s, r, 1); hi = g.pidx(s, r, g.nz - a.q); }
    a.p[lo] += a.rhs[t];
    a.p[hi] += a.rhs[t + N];
  }
}
#endif

// pres_tw_src (src/source.f90:247-309), _CONSTANT_COEFFS_POISSON branch.
// With f1 = 1 + f2, dp = p(+) - p, dq = pold(+) - pold and t = dp - dq, the
// increment f_t12*[-dp*dli/rho0 - (1/rho_f - 1/rho0)*(f1*dp - f2*dq)*dli]
// equals f_t12*dli*[(f2/rho0)*t - (1/rho_f)*(dp + f2*t)]; 1/rho_f = 2/(rho+rho(+)).
struct PresTwArgs {
  const double *p, *pold, *rho;
  double *u, *v, *w;
  const double *zA, *zB;  // per level k: f_t12*dzci(k)*f2/rho0 and 2*f_t12*dzci(k)
  double xA, xB, yA, yB;  // the same with dxi, dyi
  double f2;
  float xA32, xB32, yA32, yB32, f2_32;  // FP32 copies for the mixed path
  int fp32;               // 1: increment evaluated in FP32 from FP64 differences (mixed path)
  Geo g;
};
// FP32 increment (mixed path) from the differences of p and of pold across a
// face (dp, dq: FP32 roundings of differences that cancel, formed without
// rounding the operands first); the rest of the Dodd-Ferrante increment
// (relative error ~1e-7 of a term that is itself small against u) in FP32;
// the update u += delta stays FP64.
__device__ __forceinline__ double df_incr32(float dp, float dq, float rs, float A, float B, float f2) {
  const float t = dp - dq;
  const float dg = fmaf(f2, t, dp);
  return f64_of(fmaf(A, t, -B * (__fdividef(1.0f, rs) * dg)));  // SFU reciprocal (rs: a sum of densities)
}
// p, pold and rho at one cell.
struct DfPoint {
  double p, q, r;
};
// The six differences come from exact FP32 splits of p and pold (split32):
// only the three updates use the FP64 pipe.  A cell whose twelve values are not
// all nonzero and inside the split's range (2^-103 <= |v| < 2^128) takes FP64
// differences and the general conversions instead.  zA, zB: the level's z
// factors in FP32.
__device__ __forceinline__ void df_cell32(const PresTwArgs &a, float zA, float zB, const DfPoint &c, const DfPoint &x,
                                          const DfPoint &y, const DfPoint &z, double &u, double &v, double &w) {
  float r0, rx, ry, rz, dpx, dpy, dpz, dqx, dqy, dqz;
  if (split_range(c.p) & split_range(c.q) & split_range(c.r) & split_range(x.p) & split_range(x.q) &
      split_range(x.r) & split_range(y.p) & split_range(y.q) & split_range(y.r) & split_range(z.p) &
      split_range(z.q) & split_range(z.r)) {
    r0 = f32_in(c.r);
    rx = f32_in(x.r) + r0; ry = f32_in(y.r) + r0; rz = f32_in(z.r) + r0;
    float h0, l0, h, l;
    split32_in(c.p, h0, l0);
    split32_in(x.p, h, l); dpx = diff32(h, l, h0, l0);
    split32_in(y.p, h, l); dpy = diff32(h, l, h0, l0);
    split32_in(z.p, h, l); dpz = diff32(h, l, h0, l0);
    split32_in(c.q, h0, l0);
    split32_in(x.q, h, l); dqx = diff32(h, l, h0, l0);
    split32_in(y.q, h, l); dqy = diff32(h, l, h0, l0);
    split32_in(z.q, h, l); dqz = diff32(h, l, h0, l0);
  } else {
    r0 = f32_of(c.r);
    rx = f32_of(x.r) + r0; ry = f32_of(y.r) + r0; rz = f32_of(z.r) + r0;
    dpx = f32_of(x.p - c.p); dpy = f32_of(y.p - c.p); dpz = f32_of(z.p - c.p);
    dqx = f32_of(x.q - c.q); dqy = f32_of(y.q - c.q); dqz = f32_of(z.q - c.q);
  }
  u += df_incr32(dpx, dqx, rx, a.xA32, a.xB32, a.f2_32);
  v += df_incr32(dpy, dqy, ry, a.yA32, a.yB32, a.f2_32);
  w += df_incr32(dpz, dqz, rz, zA, zB, a.f2_32);
}
// FP64 path: the differences of p and pold across a face in FP64 (exact when
// they cancel), the rest of the increment in double-float arithmetic (dd.cuh:
// about 2^-47 of its terms), the update u += increment in FP64 (two additions:
// the increment's two parts).  Four FP64 instructions a component instead of
// the eleven of an FP64 evaluation (FP64 is the scarce pipe of this part).
__device__ __forceinline__ dd dd_rcp(dd b) {  // 1/b: FP32 seed, one double-float Newton step
  const float y = __frcp_rn(b.h);
  const dd e = dd(1.0f, 0.0f) - b * dd(y, 0.0f);
  return dd_fast_two_sum(y, y * e.h);
}
__device__ __forceinline__ double df_incr_dd(double dp, double dq, dd rs, dd A, dd B, dd f2) {
  const dd p = dd_of(dp), t = p - dd_of(dq);
  const dd dg = f2 * t + p;
  const dd r = A * t - B * (dd_rcp(rs) * dg);
  return f64_of(r.h) + f64_of(r.l);
}
__device__ __forceinline__ void df_cell64(const PresTwArgs &a, dd zA, dd zB, const DfPoint &c, const DfPoint &x,
                                          const DfPoint &y, const DfPoint &z, double &u, double &v, double &w) {
  const dd f2 = dd_of(a.f2), rc = dd_of(c.r);
  u += df_incr_dd(x.p - c.p, x.q - c.q, dd_of(x.r) + rc, dd_of(a.xA), dd_of(a.xB), f2);
  v += df_incr_dd(y.p - c.p, y.q - c.q, dd_of(y.r) + rc, dd_of(a.yA), dd_of(a.yB), f2);
  w += df_incr_dd(z.p - c.p, z.q - c.q, dd_of(z.r) + rc, zA, zB, f2);
}

// One thread per (i, j) column and PRESTW_KZ consecutive levels: the z
// neighbour of a level is the centre of the next (12 loads a cell, not 17),
// and the next level's loads are issued before this level's stores.
constexpr int PRESTW_KZ = 16, PRESTW_NT = 128;
inline dim3 presw_grid(const Geo &g) {
  return dim3((g.nx + PRESTW_NT - 1) / PRESTW_NT, g.ny < 65535 ? g.ny : 65535, (g.nz + PRESTW_KZ - 1) / PRESTW_KZ);
}
#ifndef FG_NO_PLAIN_KERNELS
__global__ void __launch_bounds__(PRESTW_NT) k_pres_tw_src(PresTwArgs a) {
  const Geo &g = a.g;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int kb = blockIdx.z * PRESTW_KZ + 1, ke = min(kb + PRESTW_KZ - 1, g.nz);
  __shared__ float zab[2][PRESTW_KZ];  // the block's z factors in FP32 (mixed path)
  static_assert(PRESTW_NT >= 2 * PRESTW_KZ, "one thread per z factor");
  if (a.fp32 && threadIdx.x < 2 * PRESTW_KZ) {
    const int q = threadIdx.x % PRESTW_KZ, half = threadIdx.x / PRESTW_KZ;
    if (kb + q <= g.nz) zab[half][q] = f32_of((half ? a.zB : a.zA)[kb + q]);
  }
  __syncthreads();
  if (i > g.nx) return;
  const long sy = g.nx + 2, sz = sy * (g.ny + 2), usz = (long)(g.nx + 2 * g.h) * (g.ny + 2 * g.h);
  const double *__restrict__ P = a.p, *__restrict__ Q = a.pold, *__restrict__ R = a.rho;
  double *__restrict__ U = a.u, *__restrict__ V = a.v, *__restrict__ W = a.w;
  auto at = [&](long o) { return DfPoint{P[o], Q[o], R[o]}; };
  for (int j = blockIdx.y + 1; j <= g.ny; j += gridDim.y) {
    long c = g.pidx(i, j, kb), ui = g.uidx(i, j, kb);
    DfPoint cen = at(c), x = at(c + 1), y = at(c + sy), z = at(c + sz);
    double u = U[ui], v = V[ui], w = W[ui];
    for (int k = kb; k <= ke; k++) {
      DfPoint xn = x, yn = y, zn = z;
      double un = u, vn = v, wn = w;
      if (k < ke) {
        xn = at(c + sz + 1); yn = at(c + sz + sy); zn = at(c + 2 * sz);
        un = U[ui + usz]; vn = V[ui + usz]; wn = W[ui + usz];
      }
      if (a.fp32) df_cell32(a, zab[0][k - kb], zab[1][k - kb], cen, x, y, z, u, v, w);
      else df_cell64(a, dd_of(a.zA[k]), dd_of(a.zB[k]), cen, x, y, z, u, v, w);
      U[ui] = u; V[ui] = v; W[ui] = w;
      cen = z; x = xn; y = yn; z = zn;
      u = un; v = vn; w = wn;
      c += sz; ui += usz;
    }
  }
}
#endif

// outflow (src/bound.f90:649-773): the velocity normal to an outflow boundary
// from zero divergence of the adjacent cells.  idir = +-1, +-2, +-3 (sign:
// high or low side).  One thread per (face point, layer q); the high side starts
// at the last interior face and runs q = 0..nh_u, the low side writes the
// ghosts q = 0..nh_u-1, as the reference does.  Rounded as written (no FMA), so
// the values are bit-identical to the reference expression.
struct OutflowArgs {
  double *u, *v, *w;
  const double *dzf;  // dzf[k], k in 1-nh_d..nz+nh_d
  double dx, dy, dxi, dyi;
  int nx, ny, nz, h, idir;
};
#ifndef FG_NO_PLAIN_KERNELS
__global__ void k_outflow(OutflowArgs a) {
  const int ad = a.idir < 0 ? -a.idir : a.idir;
  const bool hi = a.idir > 0;
  const int nq = hi ? a.h + 1 : a.h;  // layers q = 0..qmin+1 (high) or 0..qmin (low), qmin = h - 1
  const int na = ad == 1 ? a.ny : a.nx, nb = ad == 3 ? a.ny : a.nz;
  const long tot = (long)na * nb * nq;
  const long HX = a.nx + 2 * a.h, HY = a.ny + 2 * a.h;
  auto at = [&](int i, int j, int k) { return (long)(i - 1 + a.h) + HX * ((long)(j - 1 + a.h) + HY * (long)(k - 1 + a.h)); };
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (long)gridDim.x * blockDim.x) {
    const int q = (int)(t % nq), ab = (int)(t / nq), p1 = ab % na + 1, p2 = ab / na + 1;
    if (ad == 1) {
      const int j = p1, k = p2, i = hi ? a.nx + q : 1 + q;  // i: the face whose neighbours give the divergence
      const double s = __dadd_rn(__dmul_rn(__dsub_rn(a.v[at(i, j, k)], a.v[at(i, j - 1, k)]), a.dyi),
                                 __dmul_rn(__dsub_rn(a.w[at(i, j, k)], a.w[at(i, j, k - 1)]), 1.0 / a.dzf[k]));
      if (hi) a.u[at(i, j, k)] = __dsub_rn(a.u[at(a.nx - 1 - q, j, k)], __dmul_rn(a.dx, s));
      else a.u[at(-q, j, k)] = __dadd_rn(a.u[at(1 + q, j, k)], __dmul_rn(a.dx, s));
    } else if (ad == 2) {
      const int i = p1, k = p2, j = hi ? a.ny + q : 1 + q;
      const double s = __dadd_rn(__dmul_rn(__dsub_rn(a.u[at(i, j, k)], a.u[at(i - 1, j, k)]), a.dxi),
                                 __dmul_rn(__dsub_rn(a.w[at(i, j, k)], a.w[at(i, j, k - 1)]), 1.0 / a.dzf[k]));
      if (hi) a.v[at(i, j, k)] = __dsub_rn(a.v[at(i, a.ny - 1 - q, k)], __dmul_rn(a.dy, s));
      else a.v[at(i, -q, k)] = __dadd_rn(a.v[at(i, 1 + q, k)], __dmul_rn(a.dy, s));
    } else {
      const int i = p1, j = p2, k = hi ? a.nz + q : 1 + q;
      const double s = __dadd_rn(__dmul_rn(__dsub_rn(a.u[at(i, j, k)], a.u[at(i - 1, j, k)]), a.dxi),
                                 __dmul_rn(__dsub_rn(a.v[at(i, j, k)], a.v[at(i, j - 1, k)]), a.dyi));
      if (hi) a.w[at(i, j, k)] = __dsub_rn(a.w[at(i, j, a.nz - 1 - q)], __dmul_rn(a.dzf[k], s));
      else a.w[at(i, j, -q)] = __dadd_rn(a.w[at(i, j, 1 + q)], __dmul_rn(a.dzf[-q], s));
    }
  }
}
#endif

// update_property (src/vof.f90:240-271): prop = vof*prop12(1) + (1-vof)*prop12(2)
// on the interior of halo-1 arrays, rounded as written (no contraction into an
// FMA), so the result is bit-identical to the reference expression.
#ifndef FG_NO_PLAIN_KERNELS
__global__ void k_update_property(const double *vof, double *prop, double p1, double p2, Geo g) {
  for_cells(g, [&](int i0, int j0, int k0) {
    const long c = g.pidx(i0 + 1, j0 + 1, k0 + 1);
    const double f = vof[c];
    prop[c] = __dadd_rn(__dmul_rn(f, p1), __dmul_rn(__dsub_rn(1.0, f), p2));
  });
}
#endif

// correc with the pressure increment phi, fused with p = p + phi
// (src/correc.f90:57-60 and the update of src/apps/two_phase_inc_isot/main__two_phase_inc_isot.f90:698-714).
struct CorrecAddArgs {
  const double *phi;
  const double *cz;  // cz[k] = dt*rho0i*dzci(k) (index k)
  double *u, *v, *w, *p;
  double *pold;      // non-null: pold = p before the update (the app's `pold = p`, interior cells)
  double cx, cy;     // dt*dxi*rho0i, dt*dyi*rho0i
  Geo g;
};
#ifndef FG_NO_PLAIN_KERNELS
__global__ void k_correc_padd(CorrecAddArgs a) {
  const Geo &g = a.g;
  for_cells(g, [&](int i0, int j0, int k0) {
    const int i = i0 + 1, j = j0 + 1, k = k0 + 1;
    const long pc = g.pidx(i, j, k);
    const double ph = a.phi[pc];
    const long ui = g.uidx(i, j, k);
    a.u[ui] = fma(-a.cx, a.phi[pc + 1] - ph, a.u[ui]);
    a.v[ui] = fma(-a.cy, a.phi[pc + (g.nx + 2)] - ph, a.v[ui]);
    a.w[ui] = fma(-a.cz[k], a.phi[pc + (long)(g.nx + 2) * (g.ny + 2)] - ph, a.w[ui]);
    const double p0 = a.p[pc];
    if (a.pold) a.pold[pc] = p0;
    a.p[pc] = p0 + ph;
  });
}
#endif

// The last convergence check of a mixed projection fused with the correction
// it leads to: ||f - A x||^2 (as k_stencil_pass) and, in the same pass,
// correc with phi = x and p = p + x (k_correc_padd's arithmetic).  Both halves
// are bound by the FP64 pipe and read the same x; one pass saves the other's
// memory traffic and launch.  The caller applies it when the measured
// contraction predicts convergence and tops the correction up if the check
// fails after all (correc and the p update are linear in phi).
template <typename IDX = int>
__global__ void __launch_bounds__(256) k_resnorm_correc(InResidual R, CorrecAddArgs a, double *nrm) {
  const Geo &g = a.g;  // velocity halo h; R.g: halo-1 geometry of x and f
  const IDX tot = (IDX)g.nx * g.ny * g.nz;
  const FastDiv fx(g.nx), fy(g.ny);
  const long plane = (long)(g.nx + 2) * (g.ny + 2);
  float ss = 0.0f;
  for (IDX b = (IDX)blockIdx.x * blockDim.x * 2 + threadIdx.x; b < tot; b += (IDX)gridDim.x * blockDim.x * 2) {
    double v[2];
    int xs[2], ys[2], ks[2];
#pragma unroll
    for (int u = 0; u < 2; u++) {
      const IDX idx = b + (IDX)u * blockDim.x;
      int row;
      if constexpr (sizeof(IDX) == 4) {
        row = fx.div((int)idx);
        xs[u] = (int)idx - row * g.nx;
      } else {
        const IDX r = idx / g.nx;
        row = (int)r;
        xs[u] = (int)(idx - r * g.nx);
      }
      ks[u] = fy.div(row);
      ys[u] = row - ks[u] * g.ny;
      v[u] = idx < tot ? R(xs[u], ys[u], ks[u]) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 2; u++) {
      const IDX idx = b + (IDX)u * blockDim.x;
      const float f = f32_of(v[u]);
      ss = fmaf(f, f, ss);
      if (idx < tot) {
        const int i = xs[u] + 1, j = ys[u] + 1, k = ks[u] + 1;
        const long pc = g.pidx(i, j, k), ui = g.uidx(i, j, k);
        const double ph = a.phi[pc];
        if (a.u) a.u[ui] = fma(-a.cx, a.phi[pc + 1] - ph, a.u[ui]);  // null: applied before (k_correc_u)
        a.v[ui] = fma(-a.cy, a.phi[pc + (g.nx + 2)] - ph, a.v[ui]);
        a.w[ui] = fma(-a.cz[k], a.phi[pc + plane] - ph, a.w[ui]);
        const double p0 = a.p[pc];
        if (a.pold) a.pold[pc] = p0;
        a.p[pc] = p0 + ph;
      }
    }
  }
  block_sum_add((double)ss, nrm);
}

// The u part of correc alone (the same expression as k_resnorm_correc's), so
// that u's ghost cells and its copy to the host can start while the rest of
// the correction runs.
#ifndef FG_NO_PLAIN_KERNELS
__global__ void k_correc_u(CorrecAddArgs a) {
  const Geo &g = a.g;
  for_cells(g, [&](int i0, int j0, int k0) {
    const int i = i0 + 1, j = j0 + 1, k = k0 + 1;
    const long pc = g.pidx(i, j, k), ui = g.uidx(i, j, k);
    a.u[ui] = fma(-a.cx, a.phi[pc + 1] - a.phi[pc], a.u[ui]);
  });
}
#endif

// d = x - s on a whole halo-1 array (the correction still to apply after a
// fused check that did not end the solve).
#ifndef FG_NO_PLAIN_KERNELS
__global__ void k_sub(const double *x, const double *s, double *d, long n) {
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) d[t] = x[t] - s[t];
}
#endif


}  // namespace fg

namespace fg {


}  // namespace fg

namespace fg {

// ===========================================================================
// Streaming z solve (non-periodic z): one thread per (kx,ky) column, columns
// coalesced across the warp, z levels processed in chunks of CH with the next
// chunk prefetched into registers.  The forward sweep of dgtsv_homebrewed
// (src/solver_cpu.f90:187-223) writes its eliminated values y_k back into S
// (the line stays in L2 until the backward sweep overwrites it with x_k);
// the elimination factors d_k are not stored: the backward sweep recomputes
// them chunk by chunk from d at the chunk start, kept in shared memory.
// ===========================================================================
// 1/x: the SFU reciprocal in FP32 (the FP32 solve is refined in FP64), a
// correctly rounded division in FP64.
__device__ __forceinline__ float zrcp(float x) { return __fdividef(1.0f, x); }
// FP64 pivots: Newton-Raphson reciprocal (rcp64) inside FP32's normal range,
// an IEEE division outside it.
__device__ __forceinline__ double zrcp(double x) { return f32_range(x) ? rcp64(x) : 1.0 / x; }

// Coefficients of one z level, staged in shared memory once per CTA so that a
// level costs one 16- (FP32) or 32-byte (FP64) broadcast load.
template <typename T> struct alignas(4 * sizeof(T)) ZCoef {
  T a, b, c, pad;
};
template <typename T, int CH> FG_HD size_t zstream_smem(int nn, int nt) {
  return sizeof(ZCoef<T>) * (size_t)nn + sizeof(T) * (size_t)nt * (size_t)((nn + CH - 1) / CH);
}

// Chunks whose levels all lie below n - 1 (every chunk but the last) run
// without per-level predicates; the last one takes the general path (the last
// level divides, and a pinned singular column ends in zero).  Level 0 needs no
// case of its own: its pivot b + lam - a*0 is b + lam exactly (a is finite).
template <typename T, int CH, typename ST = T>
__global__ void __launch_bounds__(128) k_zstream(ZArgs za, ST *__restrict__ S, long q_begin, long q_end) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int n = za.nn;
  ZCoef<T> *co = (ZCoef<T> *)smem_raw;  // [n]
  T *chk = (T *)(co + n);               // [nch][nt]: d_{k0-1} of each chunk
  for (int k = tid; k < n; k += nt)
    co[k] = ZCoef<T>{((const T *)za.at)[k], ((const T *)za.bt)[k], ((const T *)za.ct)[k], (T)0};
  __syncthreads();
  const long q = q_begin + (long)blockIdx.x * nt + tid;
  if (q >= q_end) return;  // no block-wide barrier below
  const long plane = za.nq;
  const double lam64 = za.lam[q];
  const bool pin = za.pin && lam64 == 0.0;
  const T lam = (T)lam64;
  ST *col = S + q;
  const int nch = (n + CH - 1) / CH;
  // ---- forward elimination
  T r[CH], rn[CH];
#pragma unroll
  for (int i = 0; i < CH; i++) r[i] = i < n ? z_load(col[(long)i * plane]) : (T)0;
  T dprev = (T)0, yprev = (T)0;
  for (int m = 0; m < nch; m++) {
    const int k0 = m * CH;
    ST *p = col + (long)k0 * plane;
    {
      const ST *pn = p + (long)CH * plane;
#pragma unroll
      for (int i = 0; i < CH; i++) rn[i] = k0 + CH + i < n ? z_load(pn[(long)i * plane]) : (T)0;
    }
    chk[m * nt + tid] = dprev;
    if (k0 + CH < n) {
#pragma unroll
      for (int i = 0; i < CH; i++) {
        const ZCoef<T> cf = co[k0 + i];
        const T z = zrcp(fma(-cf.a, dprev, cf.b + lam));
        const T y = fma(-cf.a, yprev, r[i]) * z;
        dprev = cf.c * z;
        z_store(*p, y);
        p += plane;
        yprev = y;
      }
    } else {
#pragma unroll
      for (int i = 0; i < CH; i++) {
        const int k = k0 + i;
        if (k < n) {
          const ZCoef<T> cf = co[k];
          const T piv = fma(-cf.a, dprev, cf.b + lam);
          T y, d;
          if (k < n - 1) {
            const T z = zrcp(piv);
            d = cf.c * z;
            y = fma(-cf.a, yprev, r[i]) * z;
          } else {
            y = (piv != (T)0 && !pin) ? fma(-cf.a, yprev, r[i]) / piv : (T)0;
            d = (T)0;
          }
          z_store(*p, y);
          p += plane;
          dprev = d;
          yprev = y;
        }
      }
    }
#pragma unroll
    for (int i = 0; i < CH; i++) r[i] = rn[i];
  }
  // ---- back substitution, chunks from the top
  T xnext = (T)0;
  {
    const int k0 = (nch - 1) * CH;
#pragma unroll
    for (int i = 0; i < CH; i++) r[i] = k0 + i < n ? z_load(col[(long)(k0 + i) * plane]) : (T)0;
  }
  for (int m = nch - 1; m >= 0; m--) {
    const int k0 = m * CH;
    if (m > 0) {
      const ST *pp = col + (long)(k0 - CH) * plane;
#pragma unroll
      for (int i = 0; i < CH; i++) rn[i] = z_load(pp[(long)i * plane]);
    }
    T dd[CH];
    T dp = chk[m * nt + tid];
    if (k0 + CH < n) {
#pragma unroll
      for (int i = 0; i < CH; i++) {
        const ZCoef<T> cf = co[k0 + i];
        const T z = zrcp(fma(-cf.a, dp, cf.b + lam));
        dd[i] = cf.c * z;
        dp = dd[i];
      }
      ST *p = col + (long)(k0 + CH - 1) * plane;
#pragma unroll
      for (int i = CH - 1; i >= 0; i--) {
        const T x = fma(-dd[i], xnext, r[i]);
        z_store(*p, x);
        p -= plane;
        xnext = x;
      }
    } else {
#pragma unroll
      for (int i = 0; i < CH; i++) {
        const int k = k0 + i;
        if (k < n - 1) {
          const ZCoef<T> cf = co[k];
          const T z = zrcp(fma(-cf.a, dp, cf.b + lam));
          dd[i] = cf.c * z;
          dp = dd[i];
        } else {
          dd[i] = (T)0;
        }
      }
#pragma unroll
      for (int i = CH - 1; i >= 0; i--) {
        const int k = k0 + i;
        if (k < n) {
          const T x = (k == n - 1) ? r[i] : fma(-dd[i], xnext, r[i]);
          z_store(col[(long)k * plane], x);
          xnext = x;
        }
      }
    }
#pragma unroll
    for (int i = 0; i < CH; i++) r[i] = rn[i];
  }
  flag_nonfinite(za, xnext);  // level 0
}

}  // namespace fg

namespace fg {

// One direction of bounduvw (src/bound.f90:17-144): both ends, all three
// velocity components; one thread per face point, ghost layers in order.
struct SetBc3Args {
  double *f[3];
  int nx, ny, nz, h, idir;
  BcSide side[3][2];  // [component][ibound]
};
#ifndef FG_NO_PLAIN_KERNELS
__global__ void k_set_bc3(SetBc3Args s) {
  const int n = s.idir == 1 ? s.nx : (s.idir == 2 ? s.ny : s.nz);
  const int na = s.idir == 1 ? s.ny : s.nx, nb = s.idir == 3 ? s.ny : s.nz;
  const long HX = s.nx + 2 * s.h, HY = s.ny + 2 * s.h;
  const long wa = na + 2 * s.h, wb = nb + 2 * s.h;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < wa * wb; t += (long)gridDim.x * blockDim.x) {
    const int a = (int)(t % wa) + 1 - s.h, b = (int)(t / wa) + 1 - s.h;
    auto at = [&](int tt) -> long {
      int i, j, k;
      if (s.idir == 1) { i = tt; j = a; k = b; }
      else if (s.idir == 2) { i = a; j = tt; k = b; }
      else { i = a; j = b; k = tt; }
      return (long)(i - 1 + s.h) + HX * ((long)(j - 1 + s.h) + HY * (long)(k - 1 + s.h));
    };
    for (int ib = 0; ib < 2; ib++)
      for (int c = 0; c < 3; c++) {
        double *p = s.f[c];
        const BcSide &sd = s.side[c][ib];
        for (int q = 0; q < s.h; q++) {
          const double f = sd.factor[q];
          if (sd.ctype == 'P') {
            p[at(0 - q)] = p[at(n - q)];
            p[at(n + 1 + q)] = p[at(1 + q)];
          } else if (sd.centered) {
            if (ib == 0) p[at(0 - q)] = f + sd.sgn * p[at(1 + q)];
            else p[at(n + 1 + q)] = f + sd.sgn * p[at(n - q)];
          } else if (sd.ctype == 'D') {
            if (ib == 0) p[at(0 - q)] = f;
            else { p[at(n + q)] = f; p[at(n + 1 + q)] = p[at(n - 1 - q)]; }
          } else {
            if (ib == 0) p[at(0 - q)] = 1.0 * f + p[at(1 + q)];
            else { p[at(n + q)] = 1.0 * f + p[at(n - 1 - q)]; p[at(n + 1 + q)] = 2.0 * f + p[at(n - 1 - q)]; }
          }
        }
      }
  }
}
#endif

}  // namespace fg

namespace fg {

// Ghost cells of boundp / bounduvw in one launch: one thread per written cell,
// each field's value from the composition of set_bc's maps (ghosts.cuh).
#ifndef FG_NO_PLAIN_KERNELS
// k_ghosts over the written cells of a range of z planes (GhostSegs).
template <int NC> __global__ void k_ghosts_seg(const __grid_constant__ GhostArgs<NC> a, GhostSegs s) {
  for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < s.total; q += (long)gridDim.x * blockDim.x) {
    const long t = ghost_seg_cell(s, q);
    int ip[3];
    ghost_cell(a, t, ip);
    const long o = ghost_index(a, ip);
#pragma unroll
    for (int c = 0; c < NC; c++) {
      double v;
      if (ghost_value(a, c, ip, &v)) a.f[c][o] = v;
    }
  }
}
template <int NC> __global__ void k_ghosts(const __grid_constant__ GhostArgs<NC> a, long count) {  // maps read in place
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < count; t += (long)gridDim.x * blockDim.x) {
    int ip[3];
    ghost_cell(a, t, ip);
    const long o = ghost_index(a, ip);
#pragma unroll
    for (int c = 0; c < NC; c++) {
      double v;
      if (ghost_value(a, c, ip, &v)) a.f[c][o] = v;
    }
  }
}
#endif
}  // namespace fg

namespace fg {
// out[k] = s * in[k] for k in [0, n): folded z factors (e.g. dti*rho0*dzfi(k)),
// up to four vectors in one launch (one block each).
struct ScaleJobs {
  const double *in[4];
  double s[4];
  double *out[4];
  int n[4];
  int count = 0;
  void add(const double *i, double sc, double *o, int len) {
    in[count] = i; s[count] = sc; out[count] = o; n[count] = len;
    count++;
  }
};
#ifndef FG_NO_PLAIN_KERNELS
__global__ void k_scale_vecs(ScaleJobs j) {
  const int b = blockIdx.x;
  for (int k = threadIdx.x; k < j.n[b]; k += blockDim.x) j.out[b][k] = j.s[b] * j.in[b][k];
}
#endif
}  // namespace fg

namespace fg {

// ===========================================================================
// Batched solves: many independent grids of different sizes and BCs.
// Each pass is one persistent kernel that drains a (grid, tile) work queue
// (an atomic counter over the concatenated tiles of all grids).  Grids that
// have converged are skipped.  The pass sequence is captured in a CUDA graph.
// ===========================================================================
struct BatchGrid {
  Geo g;                 // halo-1 geometry
  AxisPlan ax, ay;       // FP32 transform plans
  ZArgs za;              // FP32 z coefficients (at/bt/ct), lambda, pin, periodic
  double *x, *f;         // FP64 halo arrays: solution (RHS on entry), RHS copy
  float *S, *S2;         // spectral array, periodic-z scratch (nullable)
  const double *zres;    // residual coefficients, 3 per level
  double dxi2, dyi2, normfft;
  char bc[6];
  int M, W;              // x-pass rows per tile, y-pass columns per tile
  int plane;             // 1: both transforms of a z-plane in one CTA (kb_xyfwd_plane / kb_xyinv_plane)
  double *nrm;           // [0] ||f||^2, [1] ||r||^2 of the current check
  int *active;           // 1 while the grid still refines
};

// Work queue of one pass over the grids that still refine: slot s of the
// compacted list is grid ids[s]; prefix[s] is the running total of tiles of
// slots < s (nslots + 1 entries).  kb_compact rebuilds the list after every
// convergence update, so a pass over converged grids has no items at all.
// Tile kinds of the batched passes: x tiles, y tiles, z tiles, plane items of
// small planes (several CTAs a SM), plane items of large planes.
constexpr int BATCH_KINDS = 5;
struct BatchQueue {
  const BatchGrid *grids;
  const long *prefix;
  const int *ids;
  const int *nslots;
  int *counter;          // work counter of this pass (zeroed before the pass)
};

__device__ __forceinline__ int batch_find(const long *prefix, int ng, long item) {
  int lo = 0, hi = ng;  // prefix[lo] <= item < prefix[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (prefix[mid] <= item) lo = mid; else hi = mid;
  }
  return lo;
}

// Fetch the next work item for the whole block (thread 0 takes it, all read it).
__device__ __forceinline__ long batch_next(int *counter) {
  __shared__ long s_item;
  __syncthreads();
  if (threadIdx.x == 0) s_item = (long)atomicAdd(counter, 1);
  __syncthreads();
  return s_item;
}

// First pass (mode 0: RHS = x, keep f = x) or residual pass (mode 1: r = f - A x).
#ifndef FG_NO_PLAIN_KERNELS
__global__ void __launch_bounds__(256) kb_xfwd(BatchQueue q, int mode) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ns = *q.nslots;
  const long total = q.prefix[ns];
  for (long item = batch_next(q.counter); item < total; item = batch_next(q.counter)) {
    const int slot = batch_find(q.prefix, ns, item);
    const BatchGrid &G = q.grids[q.ids[slot]];
    if (!*G.active) continue;
    const long row0 = (item - q.prefix[slot]) * G.M;
    float ss = 0.0f;
    if (mode == 0) {
      InKeep<InHalo> in{InHalo{G.x, G.g}, G.f, G.g};
      xfwd_tile<float, InKeep<InHalo>>(G.ax, in, G.S, G.g, G.M, row0, smem_raw, ss);
    } else {
      InResidual in;
      in.f = G.f; in.x = G.x; in.zc = G.zres; in.dxi2 = G.dxi2; in.dyi2 = G.dyi2;
      for (int t = 0; t < 6; t++) in.bc[t] = G.bc[t];
      in.g = G.g;
      xfwd_tile<float, InResidual>(G.ax, in, G.S, G.g, G.M, row0, smem_raw, ss);
    }
    block_sum_add((double)ss, G.nrm + (mode == 0 ? 0 : 1));
  }
}
#endif

// Grids whose planes fit one CTA: both transforms of a plane per item (the
// x and y pass kernels carry no items for them).  mode 0: first pass (RHS =
// x, keep f), mode 1: residual pass.
#ifndef FG_NO_PLAIN_KERNELS
template <int NT>  // threads a CTA: 256 for small planes (two CTAs a SM), 512 for large ones (one)
__global__ void __launch_bounds__(NT) kb_xyfwd_plane(BatchQueue q, int mode) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ns = *q.nslots;
  const long total = q.prefix[ns];
  for (long item = batch_next(q.counter); item < total; item = batch_next(q.counter)) {
    const int slot = batch_find(q.prefix, ns, item);
    const BatchGrid &G = q.grids[q.ids[slot]];
    if (!*G.active) continue;
    const int k = (int)(item - q.prefix[slot]);
    float ss = 0.0f;
    if (mode == 0) {
      InKeep<InHalo> in{InHalo{G.x, G.g}, G.f, G.g};
      xyfwd_plane_tile<float, InKeep<InHalo>>(G.ax, G.ay, in, G.S, G.g, k, smem_raw, ss);
    } else {
      InResidual in;
      in.f = G.f; in.x = G.x; in.zc = G.zres; in.dxi2 = G.dxi2; in.dyi2 = G.dyi2;
      for (int t = 0; t < 6; t++) in.bc[t] = G.bc[t];
      in.g = G.g;
      xyfwd_plane_tile<float, InResidual>(G.ax, G.ay, in, G.S, G.g, k, smem_raw, ss);
    }
    block_sum_add((double)ss, G.nrm + (mode == 0 ? 0 : 1));
  }
}
// mode 0: x = e * normfft; mode 1: x += e * normfft
template <int NT>
__global__ void __launch_bounds__(NT) kb_xyinv_plane(BatchQueue q, int mode) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ns = *q.nslots;
  const long total = q.prefix[ns];
  for (long item = batch_next(q.counter); item < total; item = batch_next(q.counter)) {
    const int slot = batch_find(q.prefix, ns, item);
    const BatchGrid &G = q.grids[q.ids[slot]];
    if (!*G.active) continue;
    const int k = (int)(item - q.prefix[slot]);
    if (mode == 0) xyinv_plane_tile<float, OutHalo>(G.ax, G.ay, G.S, OutHalo{G.x, G.normfft, G.g}, G.g, k, smem_raw);
    else xyinv_plane_tile<float, OutHaloAdd>(G.ax, G.ay, G.S, OutHaloAdd{G.x, G.normfft, G.g}, G.g, k, smem_raw);
  }
}
#endif

template <bool BACKWARD>
__global__ void __launch_bounds__(256) kb_ypass(BatchQueue q) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ns = *q.nslots;
  const long total = q.prefix[ns];
  for (long item = batch_next(q.counter); item < total; item = batch_next(q.counter)) {
    const int slot = batch_find(q.prefix, ns, item);
    const BatchGrid &G = q.grids[q.ids[slot]];
    if (!*G.active) continue;
    ypass_tile<float, BACKWARD>(G.ay, G.S, G.g, G.W, item - q.prefix[slot], smem_raw);
  }
}

// mode 0: x = e * normfft; mode 1: x += e * normfft
#ifndef FG_NO_PLAIN_KERNELS
__global__ void __launch_bounds__(256, 2) kb_xinv(BatchQueue q, int mode) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ns = *q.nslots;
  const long total = q.prefix[ns];
  for (long item = batch_next(q.counter); item < total; item = batch_next(q.counter)) {
    const int slot = batch_find(q.prefix, ns, item);
    const BatchGrid &G = q.grids[q.ids[slot]];
    if (!*G.active) continue;
    const long row0 = (item - q.prefix[slot]) * G.M;
    if (mode == 0) xinv_tile<float, OutHalo>(G.ax, G.S, OutHalo{G.x, G.normfft, G.g}, G.g, G.M, row0, smem_raw);
    else xinv_tile<float, OutHaloAdd>(G.ax, G.S, OutHaloAdd{G.x, G.normfft, G.g}, G.g, G.M, row0, smem_raw);
  }
}
#endif

// z solve of one column per thread (FP32).  Non-periodic: the forward sweep
// writes the eliminated values into S, the backward sweep recomputes the
// elimination factors from per-chunk checkpoints kept in shared memory
// (chk[nchunk][blockDim]).  Periodic: the spike solution of gaussel_periodic
// (src/solver_cpu.f90:147-185) goes through S2 and a third sweep combines.
template <int CH>
static __device__ void zcol_f32(const ZArgs &za, float *S, float *S2, long q, bool act, float *chk) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const long plane = za.nq;
  const double lam64 = act ? za.lam[q] : 1.0;
  const bool pin = za.pin && lam64 == 0.0;
  const float lam = (float)lam64;
  const float *ca = (const float *)za.at, *cb = (const float *)za.bt, *cc = (const float *)za.ct;
  float *col = S + (act ? q : 0);
  float *col2 = S2 ? S2 + (act ? q : 0) : nullptr;
  const bool per = za.periodic != 0;
  const int n = per ? za.nn - 1 : za.nn;  // system solved by elimination
  const int nch = (n + CH - 1) / CH;
  // forward
  float dprev = 0.f, yprev = 0.f, y2prev = 0.f;
  for (int m = 0; m < nch; m++) {
    const int k0 = m * CH;
    chk[m * nt + tid] = dprev;
    float r[CH];
#pragma unroll
    for (int i = 0; i < CH; i++) r[i] = (act && k0 + i < n) ? col[(long)(k0 + i) * plane] : 0.f;
#pragma unroll
    for (int i = 0; i < CH; i++) {
      const int k = k0 + i;
      if (k < n) {
        const float bb = cb[k] + lam, ak = ca[k];
        const float piv = k == 0 ? bb : fmaf(-ak, dprev, bb);
        float y, d = 0.f;
        if (k < n - 1 || per) {
          const float z = __fdividef(1.0f, piv);
          d = cc[k] * z;
          y = (k == 0 ? r[i] : fmaf(-ak, yprev, r[i])) * z;
          if (per) {
            // spike RHS: -a(1) at the first level, -c(n-1) at the last of the n-1 system
            float g = (k == 0 ? -ca[0] : 0.f) + (k == n - 1 ? -cc[n - 1] : 0.f);
            const float y2 = (k == 0 ? g : fmaf(-ak, y2prev, g)) * z;
            if (act) col2[(long)k * plane] = y2;
            y2prev = y2;
          }
        } else {
          y = (piv != 0.f && !pin) ? __fdividef(fmaf(-ak, yprev, r[i]), piv) : 0.f;
        }
        if (act) col[(long)k * plane] = y;
        dprev = d;
        yprev = y;
      }
    }
  }
  // backward
  float xnext = 0.f, x2next = 0.f;
  float x0 = 0.f, x20 = 0.f, xlast = 0.f, x2last = 0.f;
  for (int m = nch - 1; m >= 0; m--) {
    const int k0 = m * CH;
    float dd[CH];
    float dp = chk[m * nt + tid];
#pragma unroll
    for (int i = 0; i < CH; i++) {
      const int k = k0 + i;
      if (k < n - 1) {
        const float bb = cb[k] + lam;
        const float z = __fdividef(1.0f, k == 0 ? bb : fmaf(-ca[k], dp, bb));
        dd[i] = cc[k] * z;
        dp = dd[i];
      } else {
        dd[i] = 0.f;
      }
    }
#pragma unroll
    for (int i = CH - 1; i >= 0; i--) {
      const int k = k0 + i;
      if (k < n) {
        const float yk = act ? col[(long)k * plane] : 0.f;
        const float x = (k == n - 1) ? yk : fmaf(-dd[i], xnext, yk);
        if (act) col[(long)k * plane] = x;
        xnext = x;
        if (k == n - 1) xlast = x;
        if (k == 0) x0 = x;
        if (per) {
          const float y2k = act ? col2[(long)k * plane] : 0.f;
          const float x2 = (k == n - 1) ? y2k : fmaf(-dd[i], x2next, y2k);
          if (act) col2[(long)k * plane] = x2;
          x2next = x2;
          if (k == n - 1) x2last = x2;
          if (k == 0) x20 = x2;
        }
      }
    }
  }
  if (per && act) {
    const int nn = za.nn;
    const float rn = col[(long)(nn - 1) * plane];
    const float num = rn - cc[nn - 1] * x0 - ca[nn - 1] * xlast;
    const float den = (cb[nn - 1] + lam) + cc[nn - 1] * x20 + ca[nn - 1] * x2last;
    const float pn = ((za.pin && lam64 == 0.0) || den == 0.f) ? 0.f : num / den;
    col[(long)(nn - 1) * plane] = pn;
    for (int k = 0; k < nn - 1; k++) col[(long)k * plane] = fmaf(col2[(long)k * plane], pn, col[(long)k * plane]);
  }
}

#ifndef FG_NO_PLAIN_KERNELS
__global__ void __launch_bounds__(128) kb_z(BatchQueue q) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *chk = (float *)smem_raw;
  const int ns = *q.nslots;
  const long total = q.prefix[ns];
  for (long item = batch_next(q.counter); item < total; item = batch_next(q.counter)) {
    const int slot = batch_find(q.prefix, ns, item);
    const BatchGrid &G = q.grids[q.ids[slot]];
    if (!*G.active) continue;
    const long qcol = (item - q.prefix[slot]) * blockDim.x + threadIdx.x;
    zcol_f32<16>(G.za, G.S, G.S2, qcol, qcol < G.za.nq, chk);
  }
}
#endif

// ===========================================================================
// The whole batched refinement as one persistent kernel.  One work queue runs
// over every (pass, grid, tile) item of the solve in pass order: the first
// solve (x, y, z, y^-1, x^-1), then per refinement iteration the residual x
// pass and, for the grids still above tol, the next correction.  An item waits
// for the previous pass of its own grid only (a per-(pass, grid) count of the
// finished tiles), so the passes of different grids overlap: small grids run
// their z sweeps while large ones still transform.  A grid that has reached
// tol skips its later passes: the first item of such a pass moves the queue
// past the grid's other tiles of it (atomicMax) and counts them finished, so a
// skipped pass costs about one item, not one per tile.  Items leave the queue in
// order and every earlier item belongs to a running block, so a wait always
// ends; it is still bounded: past the limit the kernel records the failure,
// raises the abort flag every block checks, and returns.  Selected with
// FLUTAS_GB300_BATCH_PERSISTENT=1: the default form (one work-queue kernel per
// pass, kb_xfwd ... kb_xinv) measured faster from 8 to 512 grids, because here
// the compute warps wait at each item's barrier while warp 0 resolves the next
// item through dependent L2 round trips.
// ===========================================================================
enum BatchPass : int { PB_XF0 = 0, PB_Y = 1, PB_Z = 2, PB_YI = 3, PB_XI0 = 4, PB_XR = 5, PB_XI1 = 6 };

struct PersistArgs {
  const BatchGrid *grids;
  int ng;
  const long *prefix;  // 3 x (ng+1) running totals of the x tiles, y tiles, z tiles (blockDim columns) of the grids
  const int *ptype;    // per pass: BatchPass
  const int *piter;    // per pass: refinement iteration (0: the first solve)
  const long *poff;    // npass + 1: first queue item of each pass
  const int *pstart;   // npass * ng + 1: first queue item of (pass p, grid g) at p * ng + g
  int *pass_done;      // npass: finished tiles of each pass over all grids
  int npass;
  int chunk;           // consecutive items a block takes from the queue at once
  int *counter;        // queue position (zeroed before the launch)
  int *done;           // npass x ng: finished tiles of (pass, grid)
  int *err;            // [0]: a wait gave up; [1]: abort flag
  double *nrm;         // per grid, stride entries: [0] ||f||^2, [it] ||r||^2 after it FP32 solves
  int stride;          // max_iter + 1
  double tol;
  int max_iter;
  long spin_limit;     // polls of a dependency wait before it gives up
  unsigned long long *stats;  // items worked, tiles skipped, waits that polled, polls, ns per pass type (or null)
};

__host__ __device__ inline int pass_kind(int type) {  // 0: x tiles, 1: y tiles, 2: z tiles
  return (type == PB_Y || type == PB_YI) ? 1 : (type == PB_Z ? 2 : 0);
}

#ifndef FG_NO_PLAIN_KERNELS
__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Largest i in [0, n) with A[i] <= key, for A non-decreasing and A[0] <= key:
// a 32-way search by one warp (every lane calls it), two dependent loads for
// up to 1024 entries.
__device__ __forceinline__ int warp_find32(const int *A, int n, int key) {
  const int lane = threadIdx.x & 31;
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int step = (hi - lo + 31) >> 5;
    const int idx = lo + lane * step;
    const unsigned m = __ballot_sync(0xffffffffu, idx < hi && A[idx] <= key);
    lo += (31 - __clz(m)) * step;
    hi = min(lo + step, hi);
  }
  return lo;
}

__device__ __forceinline__ int ld_acquire_gpu(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_gpu_add(int *p, int v) {
  asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Two CTAs a SM (128 registers a thread; one CTA at up to 255 registers measured slower:
// 270 against 175 ms for 512 grids in an earlier form of the kernel).
__global__ void __launch_bounds__(256, 2) kb_persist(PersistArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int kMaxPass = 5 + 5 * 32;
  __shared__ int s_ptype[kMaxPass], s_piter[kMaxPass];
  __shared__ int s_p, s_g, s_go, s_count;  // s_go 1: work, 0: skip (grid converged), -1: abort or end
  __shared__ long s_tile;
  for (int i = threadIdx.x; i < a.npass; i += blockDim.x) {
    s_ptype[i] = a.ptype[i];
    s_piter[i] = a.piter[i];
  }
  const int total = a.pstart[(long)a.npass * a.ng];
  const int npair = a.npass * a.ng;
  const int lane = threadIdx.x & 31;
  const bool w0 = threadIdx.x < 32;
  // Warp 0 schedules.  The queue hands out chunks of `chunk` consecutive items;
  // lane 0 takes the next chunk while the block works on the current one, so
  // the queue's round trip hides behind the tiles.  Every item depends on
  // lower-numbered items only, and a block finishes its items in order, so the
  // lowest unfinished item is always some block's current one and can run.
  const int K = a.chunk;
  int cur = 0, cend = 0, nxt = (w0 && lane == 0) ? atomicAdd(a.counter, K) : 0;
  bool want = false;  // the next chunk is to be taken
  // The (pass, grid) pair of the last item, its queue range [qs, qe) and the
  // decision for it: later items of the same pair reuse all three.
  int q = 0, qs = 0, qe = 0, qgo = 1;
  // Every pass <= acq_upto had finished over all grids when an acquire of this
  // block saw it: items whose previous pass is among them need no wait and no
  // acquire (all they read was final then; tiles of one pass read and write
  // disjoint data).  Fewer acquires also keep the tables in L1.
  int acq_upto = -1;
  unsigned long long n_work = 0, n_skip = 0, n_wait = 0, n_poll = 0, t_sched = 0;
  __syncthreads();
  for (;;) {
    if (w0) {
      const unsigned long long ts = a.stats ? globaltimer_ns() : 0;
      if (cur >= cend) {
        cur = nxt;
        cend = nxt + K;
        want = true;
      }
      const int item = __shfl_sync(0xffffffffu, cur, 0);
      cur++;
      int go = -1, count = 1;
      if (item < total) {
        if (item >= qe) {  // a new pair: find it, wait for its grid's previous pass, decide
          {  // one scan of the next 32 pairs, a search of the rest when it is further
            const int idx = q + lane;
            const int v = idx <= npair ? a.pstart[idx] : INT_MAX;
            const unsigned m = __ballot_sync(0xffffffffu, v <= item);
            if (m != 0xffffffffu) q += 31 - __clz(m);
            else q += 31 + warp_find32(a.pstart + q + 31, npair - q - 31, item);
          }
          qs = a.pstart[q];
          qe = a.pstart[q + 1];
          const int p = q / a.ng, g = q - p * a.ng;
          const int type = s_ptype[p], it = s_piter[p];
          qgo = 1;
          if (p > 0 && acq_upto < p - 1 && lane == 0) {  // the previous pass of this grid, every tile of it
            const int qp = q - a.ng;
            const int need = a.pstart[qp + 1] - a.pstart[qp];
            const int need_all = (int)(a.poff[p] - a.poff[p - 1]);
            const int *d = a.done + qp, *dall = a.pass_done + (p - 1);
            long spins = 0;
            for (;;) {  // acquire: the finished tiles' writes are visible from here on
              const int c = ld_acquire_gpu(d), call = ld_acquire_gpu(dall);
              if (call >= need_all) acq_upto = p - 1;
              if (c >= need) break;
              if (((volatile int *)a.err)[1] || ++spins > a.spin_limit) {
                atomicExch(a.err, 1);
                atomicExch(a.err + 1, 1);
                qgo = -1;
                break;
              }
              __nanosleep(64);
            }
            n_wait += spins > 0;
            n_poll += spins;
          }
          qgo = __shfl_sync(0xffffffffu, qgo, 0);
          __syncwarp();
          // converged after iteration j <= jmax: lane j-1 looks at ||r_j||^2 / ||f||^2
          const int jmax = type == PB_XR ? it - 1 : it;
          if (qgo == 1 && jmax >= 1) {
            const double *nr = a.nrm + (long)g * a.stride;
            bool conv = false;
            if (lane < jmax) {
              const double f2 = __ldcg(nr), r2 = __ldcg(nr + lane + 1);
              const double rel = f2 > 0.0 ? sqrt(r2 / f2) : sqrt(r2);
              conv = !(rel > a.tol);  // NaN stops the grid too
            }
            conv = __any_sync(0xffffffffu, conv);
            if (conv || (type != PB_XR && it >= a.max_iter)) qgo = 0;
          }
          if (qgo == 0 && lane == 0) {
            // The grid is done: move the queue past the rest of its tiles of this pass
            // and count the ones no block has taken yet as finished.
            const int old = atomicMax(a.counter, qe);
            if (old < qe) count += qe - old;
          }
        }
        go = qgo;
        if (lane == 0) {
          if (go == 0) n_skip += count;
          else if (go == 1) n_work++;
          if (go >= 0 && want) {
            nxt = atomicAdd(a.counter, K);
            want = false;
          }
        }
      }
      if (lane == 0) {
        const int p = q / a.ng;
        s_p = p; s_g = q - p * a.ng; s_tile = item - qs; s_go = go; s_count = count;
        if (a.stats) t_sched += globaltimer_ns() - ts;
      }
    }
    __syncthreads();
    const int go = s_go, p = s_p, g = s_g;
    const long tile = s_tile;
    if (go < 0) break;
    const int type = s_ptype[p], it = s_piter[p];
    const unsigned long long t0 = a.stats ? globaltimer_ns() : 0;
    if (go) {
      const BatchGrid &G = a.grids[g];
      double *nr = a.nrm + (long)g * a.stride;
      float ss = 0.0f;
      switch (type) {
        case PB_XF0: {
          InKeep<InHalo> in{InHalo{G.x, G.g}, G.f, G.g};
          xfwd_tile<float, InKeep<InHalo>>(G.ax, in, G.S, G.g, G.M, tile * G.M, smem_raw, ss);
          block_sum_add((double)ss, nr);
          break;
        }
        case PB_XR: {
          InResidual in;
          in.f = G.f; in.x = G.x; in.zc = G.zres; in.dxi2 = G.dxi2; in.dyi2 = G.dyi2;
          for (int t = 0; t < 6; t++) in.bc[t] = G.bc[t];
          in.g = G.g;
          xfwd_tile<float, InResidual>(G.ax, in, G.S, G.g, G.M, tile * G.M, smem_raw, ss);
          block_sum_add((double)ss, nr + it);
          break;
        }
        case PB_Y: ypass_tile<float, false>(G.ay, G.S, G.g, G.W, tile, smem_raw); break;
        case PB_YI: ypass_tile<float, true>(G.ay, G.S, G.g, G.W, tile, smem_raw); break;
        case PB_Z: {
          const long qcol = tile * blockDim.x + threadIdx.x;
          zcol_f32<16>(G.za, G.S, G.S2, qcol, qcol < G.za.nq, (float *)smem_raw);
          break;
        }
        case PB_XI0:
          xinv_tile<float, OutHalo>(G.ax, G.S, OutHalo{G.x, G.normfft, G.g}, G.g, G.M, tile * G.M, smem_raw);
          break;
        default:
          xinv_tile<float, OutHaloAdd>(G.ax, G.S, OutHaloAdd{G.x, G.normfft, G.g}, G.g, G.M, tile * G.M, smem_raw);
          break;
      }
    }
    __syncthreads();  // every thread's writes of this tile precede the count
    if (threadIdx.x == 0) {
      // release, cumulative over the block's writes that the barrier ordered before it
      red_release_gpu_add(a.done + (long)p * a.ng + g, s_count);
      red_release_gpu_add(a.pass_done + p, s_count);
      if (a.stats && go) atomicAdd(a.stats + 4 + type, globaltimer_ns() - t0);  // ns per pass type
    }
  }
  if (threadIdx.x == 0 && a.stats) {
    atomicAdd(a.stats + 0, n_work);
    atomicAdd(a.stats + 1, n_skip);
    atomicAdd(a.stats + 2, n_wait);
    atomicAdd(a.stats + 3, n_poll);
    atomicAdd(a.stats + 11, t_sched);
  }
}

// relres and FP32 solves of every grid from the norms the persistent kernel left.
__global__ void kb_finalize(PersistArgs a, double *relres, int *iters) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < a.ng; g += gridDim.x * blockDim.x) {
    const double *n = a.nrm + (long)g * a.stride;
    const double f2 = n[0];
    double rel = 0.0;
    int j = 1;
    for (; j <= a.max_iter; j++) {
      rel = f2 > 0.0 ? sqrt(n[j] / f2) : sqrt(n[j]);
      if (!(rel > a.tol) || j == a.max_iter) break;
    }
    relres[g] = rel;
    iters[g] = j;
  }
}
#endif

// Per-grid convergence after a residual pass: relres[g], active[g], iters[g].
#ifndef FG_NO_PLAIN_KERNELS
__global__ void kb_update(BatchGrid *grids, int ng, double tol, int it, int max_iter, double *relres, int *iters) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
    BatchGrid &G = grids[g];
    if (!*G.active) continue;
    const double f2 = G.nrm[0], r2 = G.nrm[1];
    const double rel = f2 > 0.0 ? sqrt(r2 / f2) : sqrt(r2);
    relres[g] = rel;
    iters[g] = it;
    if (!(rel > tol) || it >= max_iter) *G.active = 0;  // NaN also stops
    G.nrm[1] = 0.0;
  }
}
#endif

#ifndef FG_NO_PLAIN_KERNELS
__global__ void kb_reset(BatchGrid *grids, int ng) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
    *grids[g].active = 1;
    grids[g].nrm[0] = 0.0;
    grids[g].nrm[1] = 0.0;
  }
}

// Compacted work lists (one block): the grids still active, in grid order,
// and for each of the BATCH_KINDS tile kinds (x tiles, y tiles, z tiles, plane
// items of two size classes) the running totals of their tiles.  full holds the per-grid running
// totals (BATCH_KINDS x (ng+1)), act receives the compacted ones, ids the
// slot -> grid map, nslots the count.
__global__ void __launch_bounds__(1024) kb_compact(const BatchGrid *grids, int ng, const long *full, long *act,
                                                   int *ids, int *nslots) {
  constexpr int NK = BATCH_KINDS + 1;
  __shared__ long wsum[NK][32];
  const int t = threadIdx.x, nt = blockDim.x, lane = t & 31, wid = t >> 5;
  const int chunk = (ng + nt - 1) / nt, g0 = t * chunk, g1 = min(ng, g0 + chunk);
  const long L = ng + 1;
  long c[NK] = {};  // active grids, then the tiles of each kind in this thread's range
  for (int g = g0; g < g1; g++)
    if (*grids[g].active) {
      c[0]++;
      for (int p = 0; p < BATCH_KINDS; p++) c[p + 1] += full[p * L + g + 1] - full[p * L + g];
    }
  long incl[NK];
#pragma unroll
  for (int k = 0; k < NK; k++) {  // exclusive scan over the block: warp scan, then over the warp totals
    long v = c[k];
    for (int o = 1; o < 32; o <<= 1) {
      const long u = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += u;
    }
    incl[k] = v;
    if (lane == 31) wsum[k][wid] = v;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NK; k++) {
      long v = lane < (nt >> 5) ? wsum[k][lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        const long u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
      }
      wsum[k][lane] = v;  // inclusive totals of warps 0..lane
    }
  }
  __syncthreads();
  long base[NK];
#pragma unroll
  for (int k = 0; k < NK; k++) base[k] = (wid ? wsum[k][wid - 1] : 0) + incl[k] - c[k];
  int slot = (int)base[0];
  long pos[BATCH_KINDS];
  for (int p = 0; p < BATCH_KINDS; p++) pos[p] = base[p + 1];
  for (int g = g0; g < g1; g++)
    if (*grids[g].active) {
      ids[slot] = g;
      for (int p = 0; p < BATCH_KINDS; p++) {
        act[p * L + slot] = pos[p];
        pos[p] += full[p * L + g + 1] - full[p * L + g];
      }
      slot++;
    }
  if (t == nt - 1) {  // the last thread ends the lists
    *nslots = slot;
    for (int p = 0; p < BATCH_KINDS; p++) act[p * L + slot] = pos[p];
  }
}
#endif

}  // namespace fg

#include <cooperative_groups.h>

namespace fg {

namespace cg = cooperative_groups;

// ===========================================================================
// Cluster plane passes: a z-plane too large for one CTA's shared memory is
// shared by a thread-block cluster of C CTAs.  CTA r transforms rows
// [r*ny/C, (r+1)*ny/C) along x, the cluster exchanges the x-spectrum through
// distributed shared memory so that CTA r holds columns [r*nx/C, (r+1)*nx/C)
// of every row, then transforms those along y.  The inverse runs the same in
// reverse order.  Shared memory per CTA: three buffers of (plane/C) values.
// ===========================================================================
template <typename T> struct ClusterPlane {
  int nx, ny, C;
  int rows, cols;       // ny/C, nx/C
  int P;                // row pitch of the slab buffer (nx + 1)
  size_t bufsz;         // bytes of one buffer (>= rows*P and >= ny*cols reals)
  __device__ ClusterPlane(int nx_, int ny_, int C_) : nx(nx_), ny(ny_), C(C_) {
    rows = ny / C;
    cols = nx / C;
    P = xpitch(nx);
    size_t a = (size_t)rows * P, b = (size_t)ny * cols;
    bufsz = align_up<T>(sizeof(T) * (a > b ? a : b));
  }
};

inline size_t cluster_plane_smem(int nx, int ny, int C, size_t tsize) {
  const size_t rows = ny / C, cols = nx / C, P = nx + 1;
  const size_t a = rows * P, b = (size_t)ny * cols;
  const size_t one = ((tsize * (a > b ? a : b)) + 255) & ~(size_t)255;
  return 3 * one;
}

template <typename T>
struct StoreColBlock {  // y-phase lines = columns of the local column block (row-major ny x cols)
  T *R;
  int pitch;
  __device__ void pair(int c, int t, T v0, T v1) {
    R[t * pitch + 2 * c] = v0;
    R[t * pitch + 2 * c + 1] = v1;
  }
  __device__ void single(int c, int t, T v) { R[t * pitch + c] = v; }
};

// Gathers through distributed shared memory, GATHER_U remote loads in flight
// per thread before the local stores of a batch.
constexpr int GATHER_U = 8;

// x-spectrum rows (slab of each CTA, pitch gp, in buffer `slab`) -> this CTA's
// column block (ny x cols, row-major) in `blk`.  Element idx of the block is row
// gl = idx / cols (= s*rows + lr: row lr of CTA s), column x0 + idx % cols.
template <typename T>
__device__ __forceinline__ void cluster_gather_cols(cg::cluster_group &cluster, const ClusterPlane<T> &cp, T *slab,
                                                    int gp, T *blk) {
  const int x0 = (int)cluster.block_rank() * cp.cols;
  const int tid = threadIdx.x, nth = blockDim.x, tot = cp.ny * cp.cols;
  const FastDiv fc(cp.cols), fr(cp.rows);
  for (int b = tid; b < tot; b += GATHER_U * nth) {
    T v[GATHER_U];
#pragma unroll
    for (int u = 0; u < GATHER_U; u++) {
      const int idx = b + u * nth;
      if (idx < tot) {
        const int gl = fc.div(idx), xc = idx - gl * cp.cols, s = fr.div(gl), lr = gl - s * cp.rows;
        v[u] = cluster.map_shared_rank(slab, s)[lr * gp + x0 + xc];
      }
    }
#pragma unroll
    for (int u = 0; u < GATHER_U; u++) {
      const int idx = b + u * nth;
      if (idx < tot) blk[idx] = v[u];
    }
  }
}

// this CTA's row slab (rows x nx, pitch P) from every CTA's column block (ny x
// cols).  Element idx of the slab is row lr = idx / nx, column xg = idx % nx,
// held by CTA s = xg / cols at (r*rows + lr, xg % cols).
template <typename T>
__device__ __forceinline__ void cluster_gather_rows(cg::cluster_group &cluster, const ClusterPlane<T> &cp, T *blk,
                                                    T *slab) {
  const int r = (int)cluster.block_rank();
  const int tid = threadIdx.x, nth = blockDim.x, tot = cp.rows * cp.nx;
  const FastDiv fn(cp.nx), fc(cp.cols);
  for (int b = tid; b < tot; b += GATHER_U * nth) {
    T v[GATHER_U];
#pragma unroll
    for (int u = 0; u < GATHER_U; u++) {
      const int idx = b + u * nth;
      if (idx < tot) {
        const int lr = fn.div(idx), xg = idx - lr * cp.nx, s = fc.div(xg), xc = xg - s * cp.cols;
        v[u] = cluster.map_shared_rank(blk, s)[(r * cp.rows + lr) * cp.cols + xc];
      }
    }
#pragma unroll
    for (int u = 0; u < GATHER_U; u++) {
      const int idx = b + u * nth;
      if (idx < tot) slab[idx + fn.div(idx)] = v[u];  // lr*P + xg with P = nx + 1
    }
  }
}

template <typename T, typename In>
__global__ void __launch_bounds__(256, xf_minb<T>()) k_xyfwd_cluster(AxisPlan ax, AxisPlan ay, In in, T *S, Geo g, double *nrm) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks();
  const int r = (int)cluster.block_rank();
  const ClusterPlane<T> cp(g.nx, g.ny, C);
  T *B0 = (T *)smem_raw;
  T *B1 = (T *)(smem_raw + cp.bufsz);
  T *B2 = (T *)(smem_raw + 2 * cp.bufsz);
  const int tid = threadIdx.x, nth = blockDim.x;
  const int nclusters = gridDim.x / C;
  const int cid = blockIdx.x / C;
  const FastDiv fnx(g.nx);
  float ss = 0.0f;
  for (int k = cid; k < g.nz; k += nclusters) {
    // ---- x transform of this CTA's rows
    const int y0 = r * cp.rows;
    load_cells<T>(
        in, cp.rows * g.nx,
        [&](int idx, int &x, int &y, int &kk) -> bool {
          const int ly = fnx.div(idx);
          x = idx - ly * g.nx;
          y = y0 + ly;
          kk = k;
          return true;
        },
        [&](int idx, T t) { B0[idx + fnx.div(idx)] = t; }, ss);
    __syncthreads();
    const int Bx = cbatch(ax.pair, cp.rows);
    pre_fwd<T>(ax, B0, cp.P, 1, cp.rows, (C2<T> *)B1, Bx, tid, nth);
    __syncthreads();
    C2<T> *fin = run_stages<T, false>(ax, (C2<T> *)B1, (C2<T> *)B0, Bx, tid, nth);
    T *G = (fin == (C2<T> *)B1) ? B0 : B1;  // real x-spectrum rows, pitch P
    StorePlaneReal<T> sx{G, cp.P, 0};
    post_fwd<T>(ax, fin, Bx, cp.rows, sx, tid, nth);
    cluster.sync();  // every slab complete
    cluster_gather_cols<T>(cluster, cp, G, cp.P, B2);
    cluster.sync();  // every CTA has read the slabs
    // ---- y transform of this CTA's columns (lines = columns of B2)
    const int By = cbatch(ay.pair, cp.cols);
    pre_fwd<T>(ay, B2, 1, cp.cols, cp.cols, (C2<T> *)B0, By, tid, nth);
    __syncthreads();
    C2<T> *fy = run_stages<T, false>(ay, (C2<T> *)B0, (C2<T> *)B1, By, tid, nth);
    StoreColsS<T> st{S, (long)k * g.nx * g.ny, g.nx, r * cp.cols, cp.cols};
    post_fwd<T>(ay, fy, By, cp.cols, st, tid, nth);
    __syncthreads();
  }
  if (nrm) block_sum_add((double)ss, nrm);
}

template <typename T, typename Out>
__global__ void __launch_bounds__(256, xf_minb<T>()) k_xyinv_cluster(AxisPlan ax, AxisPlan ay, const T *S, Out out, Geo g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks();
  const int r = (int)cluster.block_rank();
  const ClusterPlane<T> cp(g.nx, g.ny, C);
  T *B0 = (T *)smem_raw;
  T *B1 = (T *)(smem_raw + cp.bufsz);
  T *B2 = (T *)(smem_raw + 2 * cp.bufsz);
  const int tid = threadIdx.x, nth = blockDim.x;
  const bool invx = fft_inverse(ax.pair, true), invy = fft_inverse(ay.pair, true);
  const int nclusters = gridDim.x / C;
  const int cid = blockIdx.x / C;
  const FastDiv fnx(g.nx);
  for (int k = cid; k < g.nz; k += nclusters) {
    // ---- y^-1 of this CTA's columns
    const T *Sp = S + (long)k * g.nx * g.ny + r * cp.cols;
    for (int idx = tid; idx < g.ny * cp.cols; idx += nth) {
      const int y = idx / cp.cols, xc = idx % cp.cols;
      B0[idx] = Sp[(long)y * g.nx + xc];
    }
    __syncthreads();
    const int By = cbatch(ay.pair, cp.cols);
    pre_bwd<T>(ay, B0, 1, cp.cols, cp.cols, (C2<T> *)B1, By, tid, nth);
    __syncthreads();
    C2<T> *fy = invy ? run_stages<T, true>(ay, (C2<T> *)B1, (C2<T> *)B0, By, tid, nth)
                     : run_stages<T, false>(ay, (C2<T> *)B1, (C2<T> *)B0, By, tid, nth);
    StoreColBlock<T> sy{B2, cp.cols};
    post_bwd<T>(ay, fy, By, cp.cols, sy, tid, nth);
    cluster.sync();  // every column block complete
    cluster_gather_rows<T>(cluster, cp, B2, B0);
    cluster.sync();  // every CTA has read the blocks
    // ---- x^-1 of this CTA's rows (B0, pitch P)
    const int Bx = cbatch(ax.pair, cp.rows);
    pre_bwd<T>(ax, B0, cp.P, 1, cp.rows, (C2<T> *)B1, Bx, tid, nth);
    __syncthreads();
    C2<T> *fx = invx ? run_stages<T, true>(ax, (C2<T> *)B1, (C2<T> *)B0, Bx, tid, nth)
                     : run_stages<T, false>(ax, (C2<T> *)B1, (C2<T> *)B0, Bx, tid, nth);
    // real rows into B2 (free since the second cluster barrier), then the batched epilogue
    StorePlaneReal<T> sr{B2, cp.P, 0};
    post_bwd<T>(ax, fx, Bx, cp.rows, sr, tid, nth);
    __syncthreads();
    const int y0 = r * cp.rows;
    store_cells<T>(
        out, cp.rows * g.nx,
        [&](int idx, int &x, int &y, int &kk) -> bool {
          const int ly = fnx.div(idx);
          x = idx - ly * g.nx;
          y = y0 + ly;
          kk = k;
          return true;
        },
        [&](int idx) { return B2[idx + fnx.div(idx)]; });
    __syncthreads();
  }
}


// ===========================================================================
// Extended-FFT r2r pass (fft_ext.cuh): the face-centred kinds and the
// odd-length DCT-IV / DST-IV, in place on the spectral array S (nx, ny, nz),
// along x (axis 0: line = row j + ny*k) or y (axis 1: line = i + nx*k).  A tile
// of B lines: points staged in shared memory X (line-major), the complex DFT
// of length L in two ping-pong buffers, the read-out back into X (points the
// kind does not transform keep their value) and stored.  Global accesses are
// coalesced: x lines are read point-fastest, y lines line-fastest.
// ===========================================================================
template <typename T>
__global__ void __launch_bounds__(256) k_r2r_ext(ExtAxis ea, int kind, T *S, Geo g, int axis, int B) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = ea.n, L = ea.L;
  C2<T> *c1 = (C2<T> *)smem_raw, *c2 = c1 + (size_t)L * B;
  T *X = (T *)(c2 + (size_t)L * B);
  const long lines = axis == 0 ? (long)g.ny * g.nz : (long)g.nx * g.nz;
  const int tid = threadIdx.x, nth = blockDim.x;
  auto at = [&](long l, int j) -> long {  // S index of point j of line l
    if (axis == 0) return l * g.nx + j;
    const long k = l / g.nx, i = l - k * g.nx;
    return i + (long)g.nx * (j + (long)g.ny * k);
  };
  for (long l0 = (long)blockIdx.x * B; l0 < lines; l0 += (long)gridDim.x * B) {
    const int nb = (int)min((long)B, lines - l0);
    for (int idx = tid; idx < B * n; idx += nth) {
      int c, j;
      if (axis == 0) { c = idx / n; j = idx - c * n; }
      else { j = idx / B; c = idx - j * B; }
      X[c * n + j] = c < nb ? S[at(l0 + c, j)] : (T)0;
    }
    __syncthreads();
    ext_pre<T>(ea, kind, X, n, 1, B, c1, tid, nth);
    __syncthreads();
    C2<T> *cur = c1, *nxt = c2;
    int Ns = 1;
    for (int s = 0; s < ea.nst; s++) {
      stage_dispatch<T, false>(ea.radix[s], cur, nxt, L, B, B, Ns, (const C2<T> *)ea.W, tid, nth);
      Ns *= ea.radix[s];
      C2<T> *t = cur; cur = nxt; nxt = t;
      __syncthreads();
    }
    ext_post<T>(ea, kind, cur, B, X, n, 1, tid, nth);
    __syncthreads();
    for (int idx = tid; idx < B * n; idx += nth) {
      int c, j;
      if (axis == 0) { c = idx / n; j = idx - c * n; }
      else { j = idx / B; c = idx - j * B; }
      if (c < nb) S[at(l0 + c, j)] = X[c * n + j];
    }
    __syncthreads();
  }
}

// The spectral array written back into the interior of a halo array, times
// normfft (the last step of solver_cpu, src/solver_cpu.f90:93).
template <typename T>
__global__ void k_spec_out(const T *S, OutHalo out, Geo g) {
  const long tot = (long)g.nx * g.ny * g.nz;
  for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < tot; c += (long)gridDim.x * blockDim.x) {
    const long row = c / g.nx, k = row / g.ny;
    const int i0 = (int)(c - row * g.nx), j0 = (int)(row - k * g.ny);
    out(i0, j0, (int)k, S[c]);
  }
}

}  // namespace fg
