// fft_fixed.cuh -- compile-time-sized r2r transforms of paired real lines.
//
// The same transforms as fft_engine.cuh (R2HC/HC2R for PP, Makhoul-reordered
// REDFT10/01 for NN, RODFT10/01 for DD: src/fft.f90:233-291), for a power-of-
// two length N, a batch of B complex lines (2B real lines) and a thread count
// NTH all known at compile time.  Every index is then a constant expression or
// a shift, and the r2r pre-pass is folded into the loads of the first
// Stockham stage (forward: packing and reordering of the real lines; inverse:
// recombination of the two spectra) and the inverse post-pass into the stores
// of the last stage.  A forward transform takes NST + 1 shared-memory passes
// (stages, then the Hermitian split), an inverse NST passes, against NST + 2
// for the run-time engine.
//
// Functions are __host__ __device__; the kernels pass __syncthreads() as the
// barrier between passes, the CPU emulator runs them with NTH = 1, tid = 0 and
// an empty barrier.
#pragma once
#include "fft_engine.cuh"

namespace fg {
namespace fix {

constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n / 2); }

// Balanced radix plan of N = 2^L: NST stages of at most radix 16.
template <int N> struct Plan {
  static constexpr int L = ilog2(N);
  static constexpr int NST = (L + 3) / 4;
  static constexpr int e(int s) { return L / NST + (s < L % NST ? 1 : 0); }
  static constexpr int R(int s) { return 1 << e(s); }
  static constexpr int NS(int s) { return s == 0 ? 1 : NS(s - 1) * R(s - 1); }
};

// Complex lines in shared memory: element (line c, index t) at Z[t*B + c].
template <typename T, int B> struct CLoad {
  const C2<T> *Z;
  FG_HD C2<T> operator()(int c, int t) const { return Z[t * B + c]; }
};
template <typename T, int B> struct CStore {
  C2<T> *Z;
  FG_HD void operator()(int c, int t, C2<T> v) const { Z[t * B + c] = v; }
};

// Forward pre-pass folded into the first stage: complex line c = real lines
// 2c (real part) and 2c+1 (imaginary part), reordered for NN/DD (Makhoul),
// with the DD sign flips.  Real element (line l, position t) at R[l*ls + t*es].
template <typename T, int N, int PAIR> struct RealPairLoad {
  const T *R;
  int ls, es;
  FG_HD C2<T> operator()(int c, int m) const {
    const int src = PAIR == BC_PP ? m : mperm(m, N);
    T x0 = R[(2 * c) * ls + src * es], x1 = R[(2 * c + 1) * ls + src * es];
    if (PAIR == BC_DD && (src & 1)) { x0 = -x0; x1 = -x1; }
    return mk<T>(x0, x1);
  }
};

// Inverse pre-pass folded into the first stage: the complex input of index k
// recombined from the two real spectra (halfcomplex for PP, pre-twiddled by
// conj(Q[k]) for NN/DD).
template <typename T, int N, int PAIR> struct SpecPairLoad {
  const T *R;
  int ls, es;
  const C2<T> *Q;
  FG_HD C2<T> operator()(int c, int k) const {
    const T *r0 = R + (2 * c) * ls, *r1 = R + (2 * c + 1) * ls;
    C2<T> V0, V1;
    if (PAIR == BC_PP) {
      if (k == 0 || 2 * k == N) {
        V0 = mk<T>(r0[k * es], (T)0);
        V1 = mk<T>(r1[k * es], (T)0);
      } else if (2 * k < N) {
        V0 = mk<T>(r0[k * es], r0[(N - k) * es]);
        V1 = mk<T>(r1[k * es], r1[(N - k) * es]);
      } else {
        V0 = mk<T>(r0[(N - k) * es], -r0[k * es]);
        V1 = mk<T>(r1[(N - k) * es], -r1[k * es]);
      }
    } else {
      T a0, b0, a1, b1;
      if (PAIR == BC_NN) {
        a0 = r0[k * es];
        a1 = r1[k * es];
        b0 = k > 0 ? r0[(N - k) * es] : (T)0;
        b1 = k > 0 ? r1[(N - k) * es] : (T)0;
      } else {  // DD: X~[k] = X[n-1-k]
        a0 = r0[(N - 1 - k) * es];
        a1 = r1[(N - 1 - k) * es];
        b0 = k > 0 ? r0[(k - 1) * es] : (T)0;
        b1 = k > 0 ? r1[(k - 1) * es] : (T)0;
      }
      const C2<T> q = Q[k];
      V0 = mk<T>(q.x * a0 - q.y * b0, -q.y * a0 - q.x * b0);
      V1 = mk<T>(q.x * a1 - q.y * b1, -q.y * a1 - q.x * b1);
    }
    return mk<T>(V0.x - V1.y, V0.y + V1.x);
  }
};

// Inverse post-pass folded into the last stage: real part -> line 2c, imaginary
// part -> line 2c+1, at the Makhoul position for NN/DD (DD sign flips).
template <typename T, int N, int PAIR> struct RealPairStore {
  T *R;
  int ls, es;
  FG_HD void operator()(int c, int m, C2<T> z) const {
    const int t = PAIR == BC_PP ? m : mperm(m, N);
    const T s = (PAIR == BC_DD && (t & 1)) ? (T)-1 : (T)1;
    R[(2 * c) * ls + t * es] = s * z.x;
    R[(2 * c + 1) * ls + t * es] = s * z.y;
  }
};

// One Stockham stage S of the N-point FFT over B lines.
template <typename T, int N, int S, int B, int NTH, bool INV, typename Ld, typename St>
FG_HD void stage(const Ld &ld, const St &st, const C2<T> *W, int tid) {
  using P = Plan<N>;
  constexpr int R = P::R(S), NS = P::NS(S), NR = N / R, TOT = B * NR, TWS = N / (NS * R);
  for (int bf = tid; bf < TOT; bf += NTH) {
    const int c = (int)((unsigned)bf % B), j = (int)((unsigned)bf / B), kk = (int)((unsigned)j % NS);
    C2<T> a[R];
#pragma unroll
    for (int r = 0; r < R; r++) a[r] = ld(c, j + r * NR);
    if constexpr (NS > 1) {
#pragma unroll
      for (int r = 1; r < R; r++) a[r] = cmul<T>(a[r], twid<T>(W, N, kk * r * TWS, INV));
    }
    dft_any<T, R, INV>(a, W, N);
    const int d0 = (j - kk) * R + kk;
#pragma unroll
    for (int r = 0; r < R; r++) st(c, d0 + r * NS, a[r]);
  }
}

// All stages: the first reads through ld0, the last writes through stl, the
// ones between ping-pong b0 -> b1 -> b0 ...  Returns nothing: the result is
// wherever stl put it.  bar() separates the passes.
template <typename T, int N, int B, int NTH, bool INV, int S = 0, typename Ld, typename StL, typename Bar>
FG_HD void stages(const Ld &ld, C2<T> *b0, C2<T> *b1, const StL &stl, const C2<T> *W, int tid, const Bar &bar) {
  constexpr int NST = Plan<N>::NST;
  if constexpr (S == NST - 1) {
    stage<T, N, S, B, NTH, INV>(ld, stl, W, tid);
  } else {
    CStore<T, B> st{b0};
    stage<T, N, S, B, NTH, INV>(ld, st, W, tid);
    bar();
    CLoad<T, B> nl{b0};
    stages<T, N, B, NTH, INV, S + 1>(nl, b1, b0, stl, W, tid, bar);
  }
}

// Forward Hermitian split (post-pass of R2HC / REDFT10 / RODFT10) of the B
// complex lines in F: st.pair(c, t, v0, v1) gets output position t of real
// lines 2c and 2c+1.
template <typename T, int N, int PAIR, int B, int NTH, typename Store>
FG_HD void post_fwd_pairs(const C2<T> *F, const C2<T> *Q, Store st, int tid) {
  constexpr int KMAX = PAIR == BC_PP ? N / 2 + 1 : N;
  constexpr int TOT = B * KMAX;
  for (int idx = tid; idx < TOT; idx += NTH) {
    const int c = (int)((unsigned)idx % B), k = (int)((unsigned)idx / B);
    const C2<T> Zk = F[k * B + c];
    const C2<T> Zm = F[(k ? N - k : 0) * B + c];
    const T h = (T)0.5;
    const C2<T> X0 = mk<T>(h * (Zk.x + Zm.x), h * (Zk.y - Zm.y));
    const C2<T> X1 = mk<T>(h * (Zk.y + Zm.y), h * (Zm.x - Zk.x));
    if (PAIR == BC_PP) {
      st.pair(c, k, X0.x, X1.x);
      if (k >= 1 && k <= (N - 1) / 2) st.pair(c, N - k, X0.y, X1.y);
    } else {
      const C2<T> q = Q[k];
      const T y0 = (T)2 * (X0.x * q.x - X0.y * q.y);
      const T y1 = (T)2 * (X1.x * q.x - X1.y * q.y);
      st.pair(c, PAIR == BC_NN ? k : N - 1 - k, y0, y1);
    }
  }
}

// Forward r2r of 2B real lines (R, strides ls/es) -> post-split through st.
// Buffers: b0, b1 hold B*N complex values each and differ from R (the first
// stage writes b0 while other threads still read R); st may write R.
template <typename T, int N, int PAIR, int B, int NTH, typename Store, typename Bar>
FG_HD void forward(const T *R, int ls, int es, C2<T> *b0, C2<T> *b1, const C2<T> *W, const C2<T> *Q,
                   Store st, int tid, const Bar &bar) {
  constexpr int NST = Plan<N>::NST;
  RealPairLoad<T, N, PAIR> ld{R, ls, es};
  // the last stage writes into b1 when NST is odd, b0 when even (ping-pong from b0)
  C2<T> *last = (NST % 2) ? b0 : b1;
  CStore<T, B> stl{last};
  stages<T, N, B, NTH, false>(ld, b0, b1, stl, W, tid, bar);
  bar();
  post_fwd_pairs<T, N, PAIR, B, NTH>(last, Q, st, tid);
}

// Inverse r2r of 2B real spectral lines (R) -> real lines (O): both through
// strides; b0, b1 as in forward.  The complex FFT runs in the inverse
// direction for every paired kind.
template <typename T, int N, int PAIR, int B, int NTH, typename Bar>
FG_HD void inverse(const T *R, int ls, int es, T *O, int ols, int oes, C2<T> *b0, C2<T> *b1, const C2<T> *W,
                   const C2<T> *Q, int tid, const Bar &bar) {
  SpecPairLoad<T, N, PAIR> ld{R, ls, es, Q};
  RealPairStore<T, N, PAIR> stl{O, ols, oes};
  stages<T, N, B, NTH, true>(ld, b0, b1, stl, W, tid, bar);
}

}  // namespace fix
}  // namespace fg
