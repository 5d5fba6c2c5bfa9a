// axis_tables.cuh -- host construction of the per-axis twiddle tables and
// radix plan (shared by the library and the CPU emulator used in tests).
#pragma once
#include <cmath>
#include <vector>

#include "fft_engine.cuh"
#include "fft_ext.cuh"

namespace fg {

// Fills ap (except the W/Q device pointers) and the host tables.
// Returns 0, or -1 if the size is not supported (odd n for ND/DN, prime > 13).
template <typename T>
inline int fill_axis_tables(int n, int pair, AxisPlan *ap, std::vector<C2<T>> &W, std::vector<C2<T>> &Q) {
  *ap = AxisPlan{};
  ap->n = n;
  ap->pair = pair;
  const bool pr = pair <= BC_DD;
  if (!pr && (n % 2)) return -1;
  ap->N = pr ? n : n / 2;
  // FP64 butterflies are capped at radix 8 (register pressure of 16 complex doubles)
  const int ns = ap->N == 1 ? 0 : make_radix_plan(ap->N, ap->radix, sizeof(T) == 8 ? 3 : 4);
  if (ns < 0) return -1;
  ap->nst = ns;
  const long double PI = 3.141592653589793238462643383279502884L;
  W.assign(ap->N, mk<T>(0, 0));
  Q.assign(n, mk<T>(0, 0));
  for (int t = 0; t < ap->N; t++) {
    const long double a = 2.0L * PI * t / ap->N;
    W[t] = mk<T>((T)(double)cosl(a), (T)(double)(-sinl(a)));
  }
  if (pr) {
    for (int k = 0; k < n; k++) {
      const long double a = PI * k / (2.0L * n);
      Q[k] = mk<T>((T)(double)cosl(a), (T)(double)(-sinl(a)));
    }
  } else {
    const int h = n / 2;
    for (int j = 0; j < h; j++) {
      const long double a = PI * (4.0L * j + 1.0L) / (4.0L * n);
      Q[j] = mk<T>((T)(double)cosl(a), (T)(double)(-sinl(a)));
    }
    for (int k = 0; k < h; k++) {
      const long double a = PI * k / (long double)n;
      Q[h + k] = mk<T>((T)(double)cosl(a), (T)(double)(-sinl(a)));
    }
  }
  return 0;
}

// Tables of an extended-FFT axis (fft_ext.cuh): kinds kf (forward) and kb
// (backward) on lines of n cells.  Returns -1 if the DFT length has a prime
// factor above 13.
template <typename T>
inline int fill_ext_tables(int n, int kf, int kb, ExtAxis *ea, std::vector<C2<T>> &W, std::vector<C2<T>> &Qa,
                           std::vector<C2<T>> &Qb) {
  *ea = ExtAxis{};
  ea->n = n;
  ea->kf = kf;
  ea->kb = kb;
  ea->L = ext_length(kf, n);
  if (ext_length(kb, n) != ea->L || ea->L < 2) return -1;
  const int ns = make_radix_plan(ea->L, ea->radix, sizeof(T) == 8 ? 3 : 4);
  if (ns < 0) return -1;
  ea->nst = ns;
  const long double PI = 3.141592653589793238462643383279502884L;
  W.assign(ea->L, mk<T>(0, 0));
  for (int t = 0; t < ea->L; t++) {
    const long double a = 2.0L * PI * t / ea->L;
    W[t] = mk<T>((T)(double)cosl(a), (T)(double)(-sinl(a)));
  }
  Qa.assign(n + 1, mk<T>(0, 0));
  for (int m = 0; m <= n; m++) {
    const long double a = PI * m / (2.0L * n);
    Qa[m] = mk<T>((T)(double)cosl(a), (T)(double)(-sinl(a)));
  }
  Qb.assign(n, mk<T>(0, 0));
  for (int k = 0; k < n; k++) {
    const long double a = PI * (2.0L * k + 1.0L) / (4.0L * n);
    Qb[k] = mk<T>((T)(double)cosl(a), (T)(double)(-sinl(a)));
  }
  return 0;
}

}  // namespace fg
