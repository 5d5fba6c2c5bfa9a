// fft_ext.cuh -- r2r transforms through an extended complex FFT.
//
// The face-centred kinds of src/fft.f90:265-287 and the odd-length DCT-IV /
// DST-IV of the cell-centred ND/DN pairs are computed as one complex DFT of
// length L per real line, of a symmetric extension (or a pre-twiddled copy)
// of the line, followed by a twiddled read-out.  The complex DFT is the
// Stockham engine of fft_engine.cuh (stage_dispatch), so every radix plan of
// the paired kinds applies.  FFTW's definitions (unnormalised):
//
//   REDFT00 (n):    y_k = x_0 + (-1)^k x_{n-1} + 2 sum_{j=1}^{n-2} x_j cos(pi j k/(n-1))
//                   L = 2(n-1), even extension, y_k = Re Z_k
//   RODFT00 (N):    y_k = 2 sum_j x_j sin(pi (j+1)(k+1)/(N+1))
//                   L = 2(N+1), odd extension, y_k = -Im Z_{k+1}
//   RODFT10 (n):    y_k = 2 sum_j x_j sin(pi (2j+1)(k+1)/(2n))
//                   L = 2n, z = (x, -x reversed), y_k = Re(i e^{-i pi (k+1)/(2n)} Z_{k+1})
//   RODFT01 (n):    y_k = (-1)^k x_{n-1} + 2 sum_{j=0}^{n-2} x_j sin(pi (j+1)(2k+1)/(2n))
//                   L = 2n, z_m = c_m x_{m-1} e^{-i pi m/(2n)} (m = 1..n; c = 2, c_n = 1),
//                   y_k = -Im Z_k
//   REDFT11 (n):    y_k = 2 sum_j x_j cos(pi (2j+1)(2k+1)/(4n))
//                   L = 2n, z_j = x_j e^{-i pi j/(2n)} (j < n), y_k = 2 Re(e^{-i pi (2k+1)/(4n)} Z_k)
//   RODFT11 (n):    y_k = 2 sum_j x_j sin(pi (2j+1)(2k+1)/(4n))
//                   the same z, y_k = -2 Im(e^{-i pi (2k+1)/(4n)} Z_k)
//
// Z = DFT_L(z) with the forward sign.  One real line -> one complex line (no
// pairing: these kinds are the rare ones; the common kinds keep the paired
// engine).  Every function is __host__ __device__ over (tid, nth) with no
// barrier inside, as in fft_engine.cuh.
#pragma once
#include "fft_engine.cuh"

namespace fg {

enum ExtKind : int { EXT_NONE = 0, EXT_DCT1 = 1, EXT_DST1 = 2, EXT_DST2 = 3, EXT_DST3 = 4, EXT_DCT4 = 5, EXT_DST4 = 6 };

// Number of points a kind transforms on a line of n cells (RODFT00 of the
// face-centred DD pair leaves the last point, a boundary, untouched).
FG_HD int ext_points(int kind, int n) { return kind == EXT_DST1 ? n - 1 : n; }

// Extended DFT length.
FG_HD int ext_length(int kind, int n) {
  switch (kind) {
    case EXT_DCT1: return 2 * (n - 1);
    case EXT_DST1: return 2 * n;  // 2(N+1), N = n-1
    default: return 2 * n;
  }
}

struct ExtAxis {
  int n;          // cells along the axis
  int kf, kb;     // forward and backward kinds (ExtKind)
  int L;          // DFT length (both kinds of one axis share it)
  int nst;
  int radix[12];
  const void *W;   // W_L^t = exp(-2 pi i t/L), t < L
  const void *Qa;  // exp(-i pi m/(2n)), m = 0..n
  const void *Qb;  // exp(-i pi (2k+1)/(4n)), k < n
};

// z (L complex values of B lines, line c at buf[t*B + c]) from the real lines
// X (line c, point j at X[c*xs + j*xe]).
template <typename T>
FG_HD void ext_pre(const ExtAxis &ea, int kind, const T *X, int xs, int xe, int B, C2<T> *z, int tid, int nth) {
  const int n = ea.n, L = ea.L, tot = L * B;
  const C2<T> *Qa = (const C2<T> *)ea.Qa;
  for (int idx = tid; idx < tot; idx += nth) {
    const int c = idx % B, t = idx / B;
    const T *x = X + (long)c * xs;
    C2<T> v = mk<T>((T)0, (T)0);
    switch (kind) {
      case EXT_DCT1:  // even extension about 0 and n-1
        v.x = x[(t <= n - 1 ? t : L - t) * xe];
        break;
      case EXT_DST1: {  // odd extension of N = n-1 points: 0, x_0..x_{N-1}, 0, -x_{N-1}..-x_0
        const int N = n - 1;
        if (t >= 1 && t <= N) v.x = x[(t - 1) * xe];
        else if (t >= N + 2) v.x = -x[(L - t - 1) * xe];
        break;
      }
      case EXT_DST2:  // x, then -x reversed
        v.x = t < n ? x[t * xe] : -x[(L - 1 - t) * xe];
        break;
      case EXT_DST3:
        if (t >= 1 && t <= n) {
          const T cm = t < n ? (T)2 : (T)1;
          const T s = cm * x[(t - 1) * xe];
          v = mk<T>(s * Qa[t].x, s * Qa[t].y);
        }
        break;
      default:  // EXT_DCT4, EXT_DST4
        if (t < n) {
          const T s = x[t * xe];
          v = mk<T>(s * Qa[t].x, s * Qa[t].y);
        }
        break;
    }
    z[t * B + c] = v;
  }
}

// y (real lines Y, line c point k at Y[c*ys + k*ye]) from Z = DFT_L(z).
template <typename T>
FG_HD void ext_post(const ExtAxis &ea, int kind, const C2<T> *Z, int B, T *Y, int ys, int ye, int tid, int nth) {
  const int n = ea.n, np = ext_points(kind, n), tot = np * B;
  const C2<T> *Qa = (const C2<T> *)ea.Qa, *Qb = (const C2<T> *)ea.Qb;
  for (int idx = tid; idx < tot; idx += nth) {
    const int c = idx % B, k = idx / B;
    T y;
    switch (kind) {
      case EXT_DCT1: y = Z[k * B + c].x; break;
      case EXT_DST1: y = -Z[(k + 1) * B + c].y; break;
      case EXT_DST2: {  // Re(i conj(q) E) with q = e^{+i theta}: sin(theta) Re E - cos(theta) Im E
        const C2<T> e = Z[(k + 1) * B + c], q = Qa[k + 1];  // q = (cos, -sin)
        y = -q.y * e.x - q.x * e.y;
        break;
      }
      case EXT_DST3: y = -Z[k * B + c].y; break;
      case EXT_DCT4: {
        const C2<T> u = cmul<T>(Z[k * B + c], Qb[k]);
        y = (T)2 * u.x;
        break;
      }
      default: {  // EXT_DST4
        const C2<T> u = cmul<T>(Z[k * B + c], Qb[k]);
        y = (T)-2 * u.y;
        break;
      }
    }
    Y[(long)c * ys + k * ye] = y;
  }
}

}  // namespace fg
