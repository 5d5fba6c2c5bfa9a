// emu.cu -- CPU execution of the transform passes of fft_engine.cuh.
//
// Test infrastructure: the pre/stage/post passes are __host__ __device__ and
// contain no barrier, so running each pass with (tid = 0, nth = 1) on the CPU
// executes exactly the arithmetic and indexing the kernels run on the GPU.
// Built as a host-only shared library (libflutas_emu.so) for the CPU tests.
#include <cstring>
#include <vector>

#include "axis_tables.cuh"
#include "bits.cuh"
#include "fft_engine.cuh"
#include "fft_fixed.cuh"
#include "ghosts.cuh"
#include "ptrcheck.h"

using namespace fg;

namespace {

template <typename T> struct HostStore {
  T *out;
  long ls, es;
  void pair(int c, int t, T v0, T v1) {
    out[(2L * c) * ls + t * es] = v0;
    out[(2L * c + 1) * ls + t * es] = v1;
  }
  void single(int c, int t, T v) { out[(long)c * ls + t * es] = v; }
};

template <typename T>
int run_lines(int pair, int n, int M, int backward, int cols, const double *in, double *out) {
  AxisPlan ap;
  std::vector<C2<T>> W, Q;
  if (fill_axis_tables<T>(n, pair, &ap, W, Q) != 0) return -2;
  ap.W = W.data();
  ap.Q = Q.data();
  const long ls = cols ? 1 : n, es = cols ? M : 1;
  std::vector<T> R((size_t)M * n), O((size_t)M * n, (T)0);
  for (long i = 0; i < (long)M * n; i++) R[i] = (T)in[i];
  const int B = cbatch(pair, M);
  std::vector<C2<T>> c1((size_t)B * ap.N + 1), c2((size_t)B * ap.N + 1);
  if (backward) pre_bwd<T>(ap, R.data(), ls, es, M, c1.data(), B, 0, 1);
  else pre_fwd<T>(ap, R.data(), ls, es, M, c1.data(), B, 0, 1);
  C2<T> *cur = c1.data(), *nxt = c2.data();
  const bool inv = fft_inverse(pair, backward != 0);
  int Ns = 1;
  for (int s = 0; s < ap.nst; s++) {
    if (inv) stage_dispatch<T, true>(ap.radix[s], cur, nxt, ap.N, B, B, Ns, W.data(), 0, 1);
    else stage_dispatch<T, false>(ap.radix[s], cur, nxt, ap.N, B, B, Ns, W.data(), 0, 1);
    Ns *= ap.radix[s];
    C2<T> *t = cur; cur = nxt; nxt = t;
  }
  HostStore<T> st{O.data(), ls, es};
  if (backward) post_bwd<T>(ap, cur, B, M, st, 0, 1);
  else post_fwd<T>(ap, cur, B, M, st, 0, 1);
  for (long i = 0; i < (long)M * n; i++) out[i] = (double)O[i];
  return 0;
}

}  // namespace

// Applies the r2r transform of BC pair `pair` (0 PP,1 NN,2 DD,3 ND,4 DN),
// forward or backward, to M lines of length n.  cols = 0: line l at
// in[l*n + t]; cols = 1: in[t*M + l] (the y-pass layout).  dbl selects FP64.
extern "C" __attribute__((visibility("default"))) int fg_emu_lines(int dbl, int pair, int n, int M, int backward,
                                                                   int cols, const double *in, double *out) {
  if (n < 1 || M < 1 || pair < 0 || pair > 4) return -1;
  if (dbl == 2) return run_lines<dd>(pair, n, M, backward, cols, in, out);  // double-float
  return dbl ? run_lines<double>(pair, n, M, backward, cols, in, out)
             : run_lines<float>(pair, n, M, backward, cols, in, out);
}

extern "C" __attribute__((visibility("default"))) int fg_emu_radix_plan(int N, int *radix) {
  return make_radix_plan(N, radix);
}

// The bit-operation conversions of bits.cuh, element by element.
extern "C" __attribute__((visibility("default"))) void fg_emu_f32_of(const double *x, float *y, long n) {
  for (long i = 0; i < n; i++) y[i] = f32_of(x[i]);
}
extern "C" __attribute__((visibility("default"))) void fg_emu_f64_of(const float *x, double *y, long n) {
  for (long i = 0; i < n; i++) y[i] = f64_of(x[i]);
}
extern "C" __attribute__((visibility("default"))) void fg_emu_split32(const double *x, float *h, float *l, int *ok,
                                                                       long n) {
  for (long i = 0; i < n; i++) {
    ok[i] = split_ok(x[i]) ? 1 : 0;
    split32(x[i], h[i], l[i]);
    if (split_range(x[i])) {  // the in-range forms agree with the general ones
      float h2, l2;
      split32_in(x[i], h2, l2);
      const float f = f32_in(x[i]);
      ok[i] |= (bits_of_float(h2) == bits_of_float(h[i]) && bits_of_float(l2) == bits_of_float(l[i]) &&
                bits_of_float(f) == bits_of_float(f32_of(x[i])))
                   ? 2
                   : 4;
    }
  }
}
// Ghost cells through the composed maps of ghosts.cuh (what k_ghosts runs);
// 1 when the maps do not compose (the library then runs the pass-by-pass kernels).
template <int NC> static int emu_ghosts(GhostArgs<NC> &a) {
  long count = 0;
  if (!ghosts_ready(a, &count)) return 1;
  for (long t = 0; t < count; t++) {  // a cell read is never a cell written: in place is exact
    int ip[3];
    ghost_cell(a, t, ip);
    const long o = ghost_index(a, ip);
    for (int c = 0; c < NC; c++) {
      double v;
      if (ghost_value(a, c, ip, &v)) a.f[c][o] = v;
    }
  }
  return 0;
}
extern "C" __attribute__((visibility("default"))) int fg_emu_boundp(const char *cbc, const int *n, const double *bc,
                                                                     const double *dl, double dzc0, double dzcn,
                                                                     double *p) {
  GhostArgs<1> a;
  a.f[0] = p;
  const double dr[3][2] = {{dl[0], dl[0]}, {dl[1], dl[1]}, {dzc0, dzcn}};
  boundp_maps(a, n, cbc, bc, dr);
  return emu_ghosts(a);
}
extern "C" __attribute__((visibility("default"))) int fg_emu_bounduvw(const char *cbc, const int *n, const double *bc,
                                                                       int nh_d, int h, const double *dl,
                                                                       const double *dzc, const double *dzf, double *u,
                                                                       double *v, double *w) {
  if (h < 1 || h > 4) return 2;
  BcSide sides[3][3][2];
  setbc_sides(cbc, bc, n[2], nh_d, h, dl, dzc, dzf, sides);
  GhostArgs<3> a;
  a.f[0] = u; a.f[1] = v; a.f[2] = w;
  a.n[0] = n[0]; a.n[1] = n[1]; a.n[2] = n[2]; a.h = h;
  for (int d = 0; d < 3; d++)
    for (int c = 0; c < 3; c++) setbc_maps(a.m[c][d], sides[d][c], n[d], h);
  return emu_ghosts(a);
}
// bounduvw slab by slab through the segments k_ghosts_seg runs (z-slabs of K
// interior planes, the ghost planes with the first and last slab).  Returns 1
// when the maps do not compose, 3 when the slabs' segments do not cover every
// written cell exactly once or hold a cell outside their planes.
extern "C" __attribute__((visibility("default"))) int fg_emu_bounduvw_slabs(const char *cbc, const int *n,
                                                                             const double *bc, int nh_d, int h,
                                                                             const double *dl, const double *dzc,
                                                                             const double *dzf, double *u, double *v,
                                                                             double *w, int K) {
  if (h < 1 || h > 4 || K < 1) return 2;
  BcSide sides[3][3][2];
  setbc_sides(cbc, bc, n[2], nh_d, h, dl, dzc, dzf, sides);
  GhostArgs<3> a;
  a.f[0] = u; a.f[1] = v; a.f[2] = w;
  a.n[0] = n[0]; a.n[1] = n[1]; a.n[2] = n[2]; a.h = h;
  for (int d = 0; d < 3; d++)
    for (int c = 0; c < 3; c++) setbc_maps(a.m[c][d], sides[d][c], n[d], h);
  long count = 0;
  if (!ghosts_ready(a, &count)) return 1;
  std::vector<int> seen(count, 0);
  const int nz = n[2], nslab = (nz + K - 1) / K;
  for (int sl = 0; sl < nslab; sl++) {
    const int ka = 1 + sl * K, kb = std::min(nz, ka + K - 1);
    const int e0 = sl == 0 ? 0 : ka + h - 1, e1 = sl == nslab - 1 ? nz + 2 * h : kb + h;
    const GhostSegs s = ghost_segs_of_planes(a, e0, e1);
    for (long q = 0; q < s.total; q++) {
      const long t = ghost_seg_cell(s, q);
      if (t < 0 || t >= count) return 3;
      seen[t]++;
      int ip[3];
      ghost_cell(a, t, ip);
      const int e = ip[2] - 1 + h;
      if (e < e0 || e >= e1) return 3;
      const long o = ghost_index(a, ip);
      for (int c = 0; c < 3; c++) {
        double val;
        if (ghost_value(a, c, ip, &val)) a.f[c][o] = val;
      }
    }
  }
  for (long t = 0; t < count; t++)
    if (seen[t] != 1) return 3;
  return 0;
}
extern "C" __attribute__((visibility("default"))) void fg_emu_diff32(const double *a, const double *b, float *d,
                                                                      long n) {
  for (long i = 0; i < n; i++) {
    float ha, la, hb, lb;
    split32(a[i], ha, la);
    split32(b[i], hb, lb);
    d[i] = diff32(ha, la, hb, lb);
  }
}

namespace {

template <typename T, int N, int PAIR, int M>
int run_fixed(int backward, const double *in, double *out, bool alias = false) {
  constexpr int B = M / 2;
  AxisPlan ap;
  std::vector<C2<T>> W, Q;
  if (fill_axis_tables<T>(N, PAIR, &ap, W, Q) != 0) return -1;
  std::vector<T> R((size_t)M * N), O((size_t)M * N, (T)0);
  for (size_t i = 0; i < R.size(); i++) R[i] = (T)in[i];
  std::vector<C2<T>> b0((size_t)B * N), b1((size_t)B * N);
  auto bar = [] {};
  if (alias) {
    // the two-buffer rotation of the N = 256 plane kernels (fixed.cu), two stages:
    // X holds the lines and is the second stage buffer; the forward split goes to Y
    // (the first stage buffer, read by the second stage), the inverse back into X
    static_assert(sizeof(C2<T>) * B == sizeof(T) * M, "a buffer holds the lines or the B complex lines");
    if (fix::Plan<N>::NST != 2) return -2;
    std::vector<C2<T>> X((size_t)B * N), Y((size_t)B * N);
    T *x = (T *)X.data(), *y = (T *)Y.data();
    for (size_t i = 0; i < R.size(); i++) x[i] = R[i];
    if (backward) {
      fix::inverse<T, N, PAIR, B, 1>(x, N, 1, x, N, 1, Y.data(), X.data(), W.data(), Q.data(), 0, bar);
      for (size_t i = 0; i < O.size(); i++) out[i] = (double)x[i];
    } else {
      HostStore<T> st{y, N, 1};
      fix::forward<T, N, PAIR, B, 1>(x, N, 1, Y.data(), X.data(), W.data(), Q.data(), st, 0, bar);
      for (size_t i = 0; i < O.size(); i++) out[i] = (double)y[i];
    }
    return 0;
  }
  if (backward) {
    fix::inverse<T, N, PAIR, B, 1>(R.data(), N, 1, O.data(), N, 1, b0.data(), b1.data(), W.data(), Q.data(), 0, bar);
  } else {
    HostStore<T> st{O.data(), N, 1};
    fix::forward<T, N, PAIR, B, 1>(R.data(), N, 1, b0.data(), b1.data(), W.data(), Q.data(), st, 0, bar);
  }
  for (size_t i = 0; i < O.size(); i++) out[i] = (double)O[i];
  return 0;
}

template <typename T, int N>
int fixed_pairs(int pair, int backward, const double *in, double *out, bool alias = false) {
  switch (pair) {
    case BC_PP: return run_fixed<T, N, BC_PP, 8>(backward, in, out, alias);
    case BC_NN: return run_fixed<T, N, BC_NN, 8>(backward, in, out, alias);
    case BC_DD: return run_fixed<T, N, BC_DD, 8>(backward, in, out, alias);
    default: return -1;
  }
}

}  // namespace

// The fixed-size passes (fft_fixed.cuh) on 8 real lines of length n (line l at
// in[l*n + t]), n in {32, 64, 256, 512}, kinds PP/NN/DD.
extern "C" __attribute__((visibility("default"))) int fg_emu_fixed(int dbl, int pair, int n, int backward,
                                                                   const double *in, double *out) {
#define FG_EMU_FIX(NN_)                                                                                  \
  if (n == NN_) return dbl ? fixed_pairs<double, NN_>(pair, backward, in, out) : fixed_pairs<float, NN_>(pair, backward, in, out);
  FG_EMU_FIX(32)
  FG_EMU_FIX(64)
  FG_EMU_FIX(256)
  FG_EMU_FIX(512)
#undef FG_EMU_FIX
  return -1;
}
// The same passes with the two-buffer rotation (n with two Stockham stages: 32, 64, 256).
extern "C" __attribute__((visibility("default"))) int fg_emu_fixed_alias(int dbl, int pair, int n, int backward,
                                                                         const double *in, double *out) {
#define FG_EMU_FIX(NN_)                                                                                  \
  if (n == NN_) return dbl ? fixed_pairs<double, NN_>(pair, backward, in, out, true)                  \
                           : fixed_pairs<float, NN_>(pair, backward, in, out, true);
  FG_EMU_FIX(32)
  FG_EMU_FIX(64)
  FG_EMU_FIX(256)
#undef FG_EMU_FIX
  return -1;
}

// The library's decision on where an array argument lives (ptrcheck.h).
extern "C" __attribute__((visibility("default"))) int fg_emu_classify_ptr(int attr_ok, int mem_type, int ptr_device,
                                                                         int cur_device) {
  return classify_ptr(attr_ok != 0, mem_type, ptr_device, cur_device);
}

// One extended-FFT r2r transform (fft_ext.cuh) of M lines of length n (line l
// at in[l*n + t]): the pre pass, the Stockham stages and the read-out, as the
// kernel runs them.  Points the kind does not transform are copied through.
template <typename T> static int run_ext(int kind, int n, int M, const double *in, double *out) {
  ExtAxis ea;
  std::vector<C2<T>> W, Qa, Qb;
  if (fill_ext_tables<T>(n, kind, kind, &ea, W, Qa, Qb) != 0) return -2;
  ea.W = W.data();
  ea.Qa = Qa.data();
  ea.Qb = Qb.data();
  std::vector<T> X((size_t)M * n), Y((size_t)M * n);
  for (long i = 0; i < (long)M * n; i++) X[i] = Y[i] = (T)in[i];
  std::vector<C2<T>> c1((size_t)M * ea.L), c2((size_t)M * ea.L);
  ext_pre<T>(ea, kind, X.data(), n, 1, M, c1.data(), 0, 1);
  C2<T> *cur = c1.data(), *nxt = c2.data();
  int Ns = 1;
  for (int s = 0; s < ea.nst; s++) {
    stage_dispatch<T, false>(ea.radix[s], cur, nxt, ea.L, M, M, Ns, W.data(), 0, 1);
    Ns *= ea.radix[s];
    C2<T> *t = cur; cur = nxt; nxt = t;
  }
  ext_post<T>(ea, kind, cur, M, Y.data(), n, 1, 0, 1);
  for (long i = 0; i < (long)M * n; i++) out[i] = (double)Y[i];
  return 0;
}

extern "C" __attribute__((visibility("default"))) int fg_emu_ext(int dbl, int kind, int n, int M, const double *in,
                                                                 double *out) {
  if (n < 2 || M < 1 || kind < EXT_DCT1 || kind > EXT_DST4) return -1;
  return dbl ? run_ext<double>(kind, n, M, in, out) : run_ext<float>(kind, n, M, in, out);
}
