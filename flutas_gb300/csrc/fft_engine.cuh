// fft_engine.cuh -- shared-memory Stockham FFT engine and the r2r pre/post
// passes for the x/y transforms of the FluTAS Poisson solver.
//
// The FluTAS solver (src/solver_cpu.f90:59-89) applies, per BC pair, FFTW's
// R2HC/HC2R (PP), REDFT10/01 (NN), RODFT10/01 (DD), REDFT11 (ND) and RODFT11
// (DN) along x and y (kind table: src/fft.f90:233-291).  Here every transform
// is built on a complex FFT:
//   PP, NN, DD : two real lines packed as one complex line of length n
//                (NN/DD through Makhoul's even/odd reordering, DD through the
//                DST<->DCT sign/reversal identities);
//   ND, DN     : one real line as a complex line of length n/2 (DCT-IV).
// Outputs are in FFTW's order (halfcomplex for R2HC), so the eigenvalues of
// src/initsolver.f90:122-186 apply unchanged.
//
// Every pass below is a __host__ __device__ function over (tid, nth) with no
// barrier inside: the kernels put __syncthreads() between passes, and the
// CPU emulator runs each pass over all tids in turn.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#ifndef FG_HD
#define FG_HD __host__ __device__ __forceinline__
#endif

#include "dd.cuh"

namespace fg {

// BC-pair codes (the x/y transform kind).
enum BcPair : int { BC_PP = 0, BC_NN = 1, BC_DD = 2, BC_ND = 3, BC_DN = 4 };

template <typename T> struct cplx_of;
template <> struct cplx_of<float> { using type = float2; };
template <> struct cplx_of<double> { using type = double2; };
struct dd2 {  // complex double-float (dd.cuh)
  dd x, y;
};
template <> struct cplx_of<dd> { using type = dd2; };
template <typename T> using C2 = typename cplx_of<T>::type;

template <typename T> FG_HD C2<T> mk(T x, T y) { C2<T> r; r.x = x; r.y = y; return r; }
template <typename T> FG_HD C2<T> cadd(C2<T> a, C2<T> b) { return mk<T>(a.x + b.x, a.y + b.y); }
template <typename T> FG_HD C2<T> csub(C2<T> a, C2<T> b) { return mk<T>(a.x - b.x, a.y - b.y); }
template <typename T> FG_HD C2<T> cmul(C2<T> a, C2<T> b) {
  return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename T> FG_HD C2<T> cmulc(C2<T> a, C2<T> b) {
  return mk<T>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
// multiply by -i (forward) or +i (inverse)
template <typename T, bool INV> FG_HD C2<T> rot90(C2<T> a) {
  return INV ? mk<T>(-a.y, a.x) : mk<T>(a.y, -a.x);
}

// Per-axis transform description (device pointers to twiddle tables of type T).
struct AxisPlan {
  int n;        // line length (number of cells along the axis)
  int pair;     // BcPair
  int N;        // complex FFT length: n (PP/NN/DD) or n/2 (ND/DN)
  int nst;      // number of Stockham stages
  int radix[12];
  const void *W;   // W_N^t = exp(-2 pi i t/N), t in [0,N)
  const void *Q;   // NN/DD: exp(-i pi k/(2n)), k in [0,n);
                   // ND/DN: [0,n/2) exp(-i pi (4j+1)/(4n)), then [n/2,n) exp(-i pi k/n)
};

// Makhoul reordering: v_m = x_perm(m).
FG_HD int mperm(int m, int n) { return m < (n + 1) / 2 ? 2 * m : 2 * (n - 1 - m) + 1; }

// Division by a runtime constant: shift/mask when it is a power of two.
struct FastDiv {
  int d, sh;
  bool p2;
  FG_HD explicit FastDiv(int d_) : d(d_), sh(0), p2((d_ & (d_ - 1)) == 0) {
    while ((1 << (sh + 1)) <= d_) sh++;
  }
  FG_HD int div(int x) const { return p2 ? (x >> sh) : x / d; }
  FG_HD int mod(int x) const { return p2 ? (x & (d - 1)) : x % d; }
};

// ---------------------------------------------------------------------------
// radix-R DFT kernels on registers (forward: exp(-2 pi i/R), INV: exp(+..)).
// ---------------------------------------------------------------------------
template <typename T, bool INV> FG_HD void dft2(C2<T> &a, C2<T> &b) {
  C2<T> t = a; a = cadd<T>(t, b); b = csub<T>(t, b);
}
template <typename T, bool INV> FG_HD void dft4(C2<T> &a0, C2<T> &a1, C2<T> &a2, C2<T> &a3) {
  C2<T> t0 = cadd<T>(a0, a2), t1 = csub<T>(a0, a2), t2 = cadd<T>(a1, a3);
  C2<T> t3 = rot90<T, INV>(csub<T>(a1, a3));
  a0 = cadd<T>(t0, t2); a2 = csub<T>(t0, t2); a1 = cadd<T>(t1, t3); a3 = csub<T>(t1, t3);
}

// exp(-/+ 2 pi i m / 16) constants
template <typename T> FG_HD C2<T> w16(int m, bool inv) {
  const T c1 = (T)0.92387953251128675613, s1 = (T)0.38268343236508977173, h = (T)0.70710678118654752440;
  T cs[5] = {(T)1, c1, h, s1, (T)0};
  m &= 15;
  // cos(2 pi m/16), sin(2 pi m/16) by octant symmetry
  int q = m >> 2, r = m & 3;
  T c, s;
  // angle = q*pi/2 + r*pi/8
  T cr = cs[r], sr = cs[4 - r];
  switch (q) {
    case 0: c = cr; s = sr; break;
    case 1: c = -sr; s = cr; break;
    case 2: c = -cr; s = -sr; break;
    default: c = sr; s = -cr; break;
  }
  return inv ? mk<T>(c, s) : mk<T>(c, -s);
}

template <typename T, bool INV> FG_HD void dft8(C2<T> *a) {
  // m = q + 2p (q<2, p<4); k = s + 4t
  dft4<T, INV>(a[0], a[2], a[4], a[6]);
  dft4<T, INV>(a[1], a[3], a[5], a[7]);
  // twiddle b1[s] *= W8^s
#pragma unroll
  for (int s = 1; s < 4; s++) a[1 + 2 * s] = cmul<T>(a[1 + 2 * s], w16<T>(2 * s, INV));
  C2<T> o[8];
#pragma unroll
  for (int s = 0; s < 4; s++) {
    C2<T> x0 = a[2 * s], x1 = a[1 + 2 * s];
    o[s] = cadd<T>(x0, x1);
    o[s + 4] = csub<T>(x0, x1);
  }
#pragma unroll
  for (int i = 0; i < 8; i++) a[i] = o[i];
}

template <typename T, bool INV> FG_HD void dft16(C2<T> *a) {
  // m = q + 4p ; k = s + 4t ; b_q = DFT4 over p of a[q+4p]
#pragma unroll
  for (int q = 0; q < 4; q++) dft4<T, INV>(a[q], a[q + 4], a[q + 8], a[q + 12]);
  // after dft4, a[q + 4s] holds b_q[s]; twiddle W16^{q s}
#pragma unroll
  for (int q = 1; q < 4; q++)
#pragma unroll
    for (int s = 1; s < 4; s++) a[q + 4 * s] = cmul<T>(a[q + 4 * s], w16<T>(q * s, INV));
  C2<T> o[16];
#pragma unroll
  for (int s = 0; s < 4; s++) {
    C2<T> x0 = a[0 + 4 * s], x1 = a[1 + 4 * s], x2 = a[2 + 4 * s], x3 = a[3 + 4 * s];
    dft4<T, INV>(x0, x1, x2, x3);
    o[s] = x0; o[s + 4] = x1; o[s + 8] = x2; o[s + 12] = x3;
  }
#pragma unroll
  for (int i = 0; i < 16; i++) a[i] = o[i];
}

// W_N^e for 0 <= e < N (every caller stays in range), conjugated for INV.
template <typename T> FG_HD C2<T> twid(const C2<T> *W, int N, int e, bool inv) {
  (void)N;
  const C2<T> w = W[e];
  return inv ? mk<T>(w.x, -w.y) : w;
}

// generic (odd) radix by direct summation; W is the length-N table, R | N
template <typename T, int R, bool INV> FG_HD void dftR(C2<T> *a, const C2<T> *W, int N) {
  C2<T> o[R];
  const int step = N / R;
#pragma unroll
  for (int q = 0; q < R; q++) {
    C2<T> acc = a[0];
#pragma unroll
    for (int r = 1; r < R; r++) acc = cadd<T>(acc, cmul<T>(a[r], twid<T>(W, N, ((r * q) % R) * step, INV)));
    o[q] = acc;
  }
#pragma unroll
  for (int q = 0; q < R; q++) a[q] = o[q];
}

// The same with the R roots of unity W_R^m (m < R) already in registers:
// R - 1 table loads per stage instead of R(R-1) per butterfly.
template <typename T, int R> FG_HD void dftR_w(C2<T> *a, const C2<T> *wr) {
  C2<T> o[R];
#pragma unroll
  for (int q = 0; q < R; q++) {
    C2<T> acc = a[0];
#pragma unroll
    for (int r = 1; r < R; r++) acc = cadd<T>(acc, cmul<T>(a[r], wr[(r * q) % R]));
    o[q] = acc;
  }
#pragma unroll
  for (int q = 0; q < R; q++) a[q] = o[q];
}

template <typename T, int R, bool INV> FG_HD void dft_any(C2<T> *a, const C2<T> *W, int N) {
  if constexpr (R == 2) dft2<T, INV>(a[0], a[1]);
  else if constexpr (R == 4) dft4<T, INV>(a[0], a[1], a[2], a[3]);
  else if constexpr (R == 8) dft8<T, INV>(a);
  else if constexpr (R == 16) dft16<T, INV>(a);
  else dftR<T, R, INV>(a, W, N);
}

// ---------------------------------------------------------------------------
// One Stockham stage over a batch of B complex lines of length N.
// Element (line c, index t) sits at buf[t*ldb + c]  (batch fastest).
// Ns = product of the radices of the previous stages.
// ---------------------------------------------------------------------------
template <typename T, int R, bool INV>
FG_HD void stage_pass(const C2<T> *in, C2<T> *out, int N, int B, int ldb, int Ns, const C2<T> *W,
                      int tid, int nth) {
  const int NR = N / R;
  const int total = B * NR;
  const int tws = N / (Ns * R);
  const FastDiv fb(B), fn(Ns);
  constexpr bool ODD = (R & (R - 1)) != 0;
  C2<T> wr[ODD ? R : 1];  // odd radices: W_R^m, loaded once per stage
  if constexpr (ODD) {
#pragma unroll
    for (int m = 0; m < R; m++) wr[m] = twid<T>(W, N, m * (N / R), INV);
  }
  for (int bf = tid; bf < total; bf += nth) {
    const int c = fb.mod(bf), j = fb.div(bf);
    const int kk = fn.mod(j);
    C2<T> a[R];
#pragma unroll
    for (int r = 0; r < R; r++) a[r] = in[(j + r * NR) * ldb + c];
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; r++) a[r] = cmul<T>(a[r], twid<T>(W, N, kk * r * tws, INV));
    }
    if constexpr (ODD) dftR_w<T, R>(a, wr);
    else dft_any<T, R, INV>(a, W, N);
    const int idxD = (j - kk) * R + kk;
#pragma unroll
    for (int r = 0; r < R; r++) out[(idxD + r * Ns) * ldb + c] = a[r];
  }
}

// A radix-R stage with rolled loops: each output of a butterfly summed directly
// from the R inputs (read from the buffer, twiddled on the fly).  Few registers;
// the double-float engine takes it for the large odd radices, whose unrolled
// butterflies would set the register count of every kernel they are part of.
template <typename T, bool INV>
FG_HD void stage_pass_rolled(int R, const C2<T> *in, C2<T> *out, int N, int B, int ldb, int Ns, const C2<T> *W,
                             int tid, int nth) {
  const int NR = N / R, total = B * NR, tws = N / (Ns * R), step = N / R;
  for (int bf = tid; bf < total; bf += nth) {
    const int c = bf % B, j = bf / B, kk = j % Ns, idxD = (j - kk) * R + kk;
    for (int q = 0; q < R; q++) {
      C2<T> acc = in[j * ldb + c];
      for (int r = 1; r < R; r++) {
        C2<T> a = in[(j + r * NR) * ldb + c];
        if (Ns > 1) a = cmul<T>(a, twid<T>(W, N, kk * r * tws, INV));
        acc = cadd<T>(acc, cmul<T>(a, twid<T>(W, N, ((r * q) % R) * step, INV)));
      }
      out[(idxD + q * Ns) * ldb + c] = acc;
    }
  }
}

template <typename T, bool INV>
FG_HD void stage_dispatch(int R, const C2<T> *in, C2<T> *out, int N, int B, int ldb, int Ns,
                          const C2<T> *W, int tid, int nth) {
  if constexpr (std::is_same<T, dd>::value) {
    if (R == 11 || R == 13) {
      stage_pass_rolled<T, INV>(R, in, out, N, B, ldb, Ns, W, tid, nth);
      return;
    }
  }
  switch (R) {
    case 2: stage_pass<T, 2, INV>(in, out, N, B, ldb, Ns, W, tid, nth); break;
    case 3: stage_pass<T, 3, INV>(in, out, N, B, ldb, Ns, W, tid, nth); break;
    case 4: stage_pass<T, 4, INV>(in, out, N, B, ldb, Ns, W, tid, nth); break;
    case 5: stage_pass<T, 5, INV>(in, out, N, B, ldb, Ns, W, tid, nth); break;
    case 7: stage_pass<T, 7, INV>(in, out, N, B, ldb, Ns, W, tid, nth); break;
    case 8: stage_pass<T, 8, INV>(in, out, N, B, ldb, Ns, W, tid, nth); break;
    case 11:
      if constexpr (!std::is_same<T, dd>::value) stage_pass<T, 11, INV>(in, out, N, B, ldb, Ns, W, tid, nth);
      break;
    case 13:
      if constexpr (!std::is_same<T, dd>::value) stage_pass<T, 13, INV>(in, out, N, B, ldb, Ns, W, tid, nth);
      break;
    case 16:  // double-float plans stop at radix 8 (fill_axis_tables): no radix-16 registers
      if constexpr (sizeof(T) == 4) stage_pass<T, 16, INV>(in, out, N, B, ldb, Ns, W, tid, nth);
      break;
    default: break;  // plans only contain the radices above
  }
}

// Radix plan for a length-N FFT: powers of two in balanced stages of at most
// 2^maxe (16 by default), then the odd factors 3,5,7,11,13.  Returns the
// number of stages, or -1 if N has another prime factor.
inline int make_radix_plan(int N, int *radix, int maxe = 4) {
  int e = 0, m = N;
  while (m % 2 == 0) { m /= 2; e++; }
  int ns = 0;
  if (e > 0) {
    int nst = (e + maxe - 1) / maxe;
    for (int s = 0; s < nst; s++) {
      int es = e / nst + (s < e % nst ? 1 : 0);
      radix[ns++] = 1 << es;
    }
  }
  const int odd[5] = {3, 5, 7, 11, 13};
  for (int i = 0; i < 5; i++)
    while (m % odd[i] == 0) { radix[ns++] = odd[i]; m /= odd[i]; }
  if (m != 1) return -1;
  if (ns == 0) radix[ns++] = 1;  // N == 1 (unused)
  return ns;
}

// ---------------------------------------------------------------------------
// r2r pre/post passes.  Real lines live in a strided real buffer:
//   element (line l, position t) at R[l*ls + t*es].
// Complex lines: element (line c, index t) at Cb[t*ldb + c].
// Paired kinds (PP/NN/DD): complex line c <-> real lines 2c, 2c+1 (B = M/2).
// DCT-IV kinds (ND/DN):    complex line c <-> real line c      (B = M).
// ---------------------------------------------------------------------------
FG_HD bool paired(int pair) { return pair <= BC_DD; }

// forward, real -> complex (before the FFT)
template <typename T>
FG_HD void pre_fwd(const AxisPlan &ap, const T *Rb, int ls, int es, int M, C2<T> *Cb, int ldb,
                   int tid, int nth) {
  const int n = ap.n;
  if (paired(ap.pair)) {
    const int B = M / 2, tot = B * n;
    const FastDiv fb(B);
    for (int idx = tid; idx < tot; idx += nth) {
      const int c = fb.mod(idx), m = fb.div(idx);
      const int src = ap.pair == BC_PP ? m : mperm(m, n);
      T x0 = Rb[(2 * c) * ls + src * es], x1 = Rb[(2 * c + 1) * ls + src * es];
      if (ap.pair == BC_DD && (src & 1)) { x0 = -x0; x1 = -x1; }
      Cb[m * ldb + c] = mk<T>(x0, x1);
    }
  } else {
    const int h = n / 2, tot = M * h;
    const C2<T> *Q = (const C2<T> *)ap.Q;
    const T sgn = (ap.pair == BC_DN && ((n - 1) & 1)) ? (T)-1 : (T)1;
    const FastDiv fm(M);
    for (int idx = tid; idx < tot; idx += nth) {
      const int c = fm.mod(idx), j = fm.div(idx);
      T xa = Rb[c * ls + (2L * j) * es];
      T xb = Rb[c * ls + (n - 1 - 2 * j) * es];
      if (ap.pair == BC_DN) xb = sgn * xb;  // (-1)^(n-1-2j) = (-1)^(n-1)
      Cb[j * ldb + c] = cmul<T>(mk<T>(xa, xb), Q[j]);
    }
  }
}

// Output functors: store(l, t, v) writes real value v of line l at position t.
// Paired forward post: positions come in (line 2c, line 2c+1) pairs.
template <typename T, typename Store>
FG_HD void post_fwd(const AxisPlan &ap, const C2<T> *F, int ldb, int M, Store &st, int tid,
                    int nth) {
  const int n = ap.n;
  if (paired(ap.pair)) {
    const int B = M / 2;
    const C2<T> *Q = (const C2<T> *)ap.Q;
    const int kmax = ap.pair == BC_PP ? n / 2 + 1 : n;
    const int tot = B * kmax;
    const FastDiv fb(B);
    for (int idx = tid; idx < tot; idx += nth) {
      const int c = fb.mod(idx), k = fb.div(idx);
      const C2<T> Zk = F[k * ldb + c];
      const C2<T> Zm = F[(k ? n - k : 0) * ldb + c];
      const T h = (T)0.5;
      C2<T> X0 = mk<T>(h * (Zk.x + Zm.x), h * (Zk.y - Zm.y));
      C2<T> X1 = mk<T>(h * (Zk.y + Zm.y), h * (Zm.x - Zk.x));
      if (ap.pair == BC_PP) {
        st.pair(c, k, X0.x, X1.x);
        if (k >= 1 && k <= (n - 1) / 2) st.pair(c, n - k, X0.y, X1.y);
      } else {
        const C2<T> q = Q[k];
        T y0 = (T)2 * (X0.x * q.x - X0.y * q.y);
        T y1 = (T)2 * (X1.x * q.x - X1.y * q.y);
        st.pair(c, ap.pair == BC_NN ? k : n - 1 - k, y0, y1);
      }
    }
  } else {
    const int h = n / 2, tot = M * h;
    const C2<T> *Q = (const C2<T> *)ap.Q + h;
    const FastDiv fm(M);
    for (int idx = tid; idx < tot; idx += nth) {
      const int c = fm.mod(idx), k = fm.div(idx);
      C2<T> u = cmul<T>(F[k * ldb + c], Q[k]);
      if (ap.pair == BC_ND) {
        st.single(c, 2 * k, (T)2 * u.x);
        st.single(c, n - 1 - 2 * k, (T)-2 * u.y);
      } else {
        st.single(c, n - 1 - 2 * k, (T)2 * u.x);
        st.single(c, 2 * k, (T)-2 * u.y);
      }
    }
  }
}

// backward, real spectral -> complex (before the inverse FFT)
template <typename T>
FG_HD void pre_bwd(const AxisPlan &ap, const T *Rb, int ls, int es, int M, C2<T> *Cb, int ldb,
                   int tid, int nth) {
  if (!paired(ap.pair)) { pre_fwd<T>(ap, Rb, ls, es, M, Cb, ldb, tid, nth); return; }
  const int n = ap.n, B = M / 2, tot = B * n;
  const C2<T> *Q = (const C2<T> *)ap.Q;
  const FastDiv fb(B);
  for (int idx = tid; idx < tot; idx += nth) {
    const int c = fb.mod(idx), k = fb.div(idx);
    const T *r0 = Rb + (2 * c) * ls, *r1 = Rb + (2 * c + 1) * ls;
    C2<T> V0, V1;
    if (ap.pair == BC_PP) {
      if (k == 0 || 2 * k == n) {
        V0 = mk<T>(r0[k * es], (T)0); V1 = mk<T>(r1[k * es], (T)0);
      } else if (2 * k < n) {
        V0 = mk<T>(r0[k * es], r0[(n - k) * es]); V1 = mk<T>(r1[k * es], r1[(n - k) * es]);
      } else {
        V0 = mk<T>(r0[(n - k) * es], -r0[k * es]); V1 = mk<T>(r1[(n - k) * es], -r1[k * es]);
      }
    } else {
      T a0, b0, a1, b1;
      if (ap.pair == BC_NN) {
        a0 = r0[k * es]; a1 = r1[k * es];
        b0 = k > 0 ? r0[(n - k) * es] : (T)0; b1 = k > 0 ? r1[(n - k) * es] : (T)0;
      } else {  // DD: X~[k] = X[n-1-k]
        a0 = r0[(n - 1 - k) * es]; a1 = r1[(n - 1 - k) * es];
        b0 = k > 0 ? r0[(k - 1) * es] : (T)0; b1 = k > 0 ? r1[(k - 1) * es] : (T)0;
      }
      const C2<T> q = Q[k];  // exp(-i pi k/2n); we need exp(+i ...) = conj
      // V = conj(q) * (a - i b)
      V0 = mk<T>(q.x * a0 - q.y * b0, -q.y * a0 - q.x * b0);
      V1 = mk<T>(q.x * a1 - q.y * b1, -q.y * a1 - q.x * b1);
    }
    Cb[k * ldb + c] = mk<T>(V0.x - V1.y, V0.y + V1.x);
  }
}

template <typename T, typename Store>
FG_HD void post_bwd(const AxisPlan &ap, const C2<T> *F, int ldb, int M, Store &st, int tid,
                    int nth) {
  if (!paired(ap.pair)) { post_fwd<T, Store>(ap, F, ldb, M, st, tid, nth); return; }
  const int n = ap.n, B = M / 2, tot = B * n;
  const FastDiv fb(B);
  for (int idx = tid; idx < tot; idx += nth) {
    const int c = fb.mod(idx), m = fb.div(idx);
    const C2<T> z = F[m * ldb + c];
    if (ap.pair == BC_PP) {
      st.pair(c, m, z.x, z.y);
    } else {
      const int t = mperm(m, n);
      const T s = (ap.pair == BC_DD && (t & 1)) ? (T)-1 : (T)1;
      st.pair(c, t, s * z.x, s * z.y);
    }
  }
}

// Which FFT direction a transform uses.
FG_HD bool fft_inverse(int pair, bool backward) { return backward && pair <= BC_DD; }

// Lines per complex line and complex batch for M real lines.
FG_HD int cbatch(int pair, int M) { return paired(pair) ? M / 2 : M; }

// Run all Stockham stages; returns the buffer holding the result (buf0 or buf1).
template <typename T, bool INV>
FG_HD C2<T> *stages_pass(const AxisPlan &ap, int s, C2<T> *cur, C2<T> *nxt, int B, int ldb, int Ns,
                         int tid, int nth) {
  stage_dispatch<T, INV>(ap.radix[s], cur, nxt, ap.N, B, ldb, Ns, (const C2<T> *)ap.W, tid, nth);
  return nxt;
}

}  // namespace fg
