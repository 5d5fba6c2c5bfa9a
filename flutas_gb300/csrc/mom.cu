// mom.cu -- the momentum predictor on the device: rk (src/rk.f90:26-102) with
// momad_xyz_tw_cen (src/mom.f90:21-197), momad_xyz_tw_fll (199-386) or
// momad_xyz_sp (388-575), and cmpt_time_factors (src/rk.f90:104-135).
//
// rk computes the right-hand sides of all three momentum equations from the
// old velocities, then updates u = u + f_t1*dudt + f_t2*dudtrko and keeps
// dudt as the next step's dudtrko.  Here one kernel evaluates every cell's
// right-hand sides (FP64, the reference's expressions term by term) and writes
// the new velocities into a scratch field and dudt into dudtrko; a second one
// copies the new velocities into the interior (the halo stays, as in the
// reference, for bounduvw).  The new values cannot go straight into u: the
// neighbours' right-hand sides still read the old ones.
//
// The 3-D branches only (the reference's _TWOD build zeroes dudt; not built here).
#include "../../include/flutas_gb300.h"
#include "ptrcheck.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

void fg_set_error_text(const char *msg);  // flutas_gb300.cu
void fg_note_launches(unsigned n);        // flutas_gb300.cu

namespace {

int mfail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  fg_set_error_text(buf);
  return code;
}

#define MCK(call)                                                                                           \
  do {                                                                                                      \
    cudaError_t e_ = (call);                                                                                \
    if (e_ != cudaSuccess) return mfail(FLUTAS_ECUDA, "%s failed: %s", #call, cudaGetErrorString(e_));     \
  } while (0)

enum MomVariant { MOM_CEN = 0, MOM_FLL = 1, MOM_SP = 2 };

struct MomArgs {
  int nx, ny, nz, h;       // h = nh_u (velocity halo)
  double dxi, dyi, dzi;
  const double *dzci, *dzfi;  // already offset: dzci[k] is Fortran dzci(k)
  const double *u, *v, *w, *mu, *rho;
  double visc;             // mu_sp/rho_sp (single phase)
  double f1, f2;           // f_t1, f_t2
  double *un, *vn, *wn;    // new velocities, (nx,ny,nz)
  double *du0, *dv0, *dw0; // dudtrko etc. (nx,ny,nz): read, then overwritten with dudt
};

template <int VAR>
__device__ __forceinline__ void mom_cell(const MomArgs &a, int i, int j, int k, double &du, double &dv, double &dw) {
  const long UX = a.nx + 2 * a.h, UY = a.ny + 2 * a.h, PX = a.nx + 2, PY = a.ny + 2;
  auto ui = [&](int x, int y, int z) { return (long)(x - 1 + a.h) + UX * ((long)(y - 1 + a.h) + UY * (long)(z - 1 + a.h)); };
  auto pi = [&](int x, int y, int z) { return (long)x + PX * ((long)y + PY * (long)z); };
#define U(x, y, z) __ldg(a.u + ui(x, y, z))
#define V(x, y, z) __ldg(a.v + ui(x, y, z))
#define W(x, y, z) __ldg(a.w + ui(x, y, z))
#define MU(x, y, z) __ldg(a.mu + pi(x, y, z))
#define RHO(x, y, z) __ldg(a.rho + pi(x, y, z))
  const double dxi = a.dxi, dyi = a.dyi, dzi = a.dzi;
  const double zci = a.dzci[k], zcim = a.dzci[k - 1], zfi = a.dzfi[k], zfip = a.dzfi[k + 1];
  const int ip = i + 1, im = i - 1, jp = j + 1, jm = j - 1, kp = k + 1, km = k - 1;
  double adv_u, adv_v, adv_w;
  if constexpr (VAR != MOM_FLL) {
    // centred fluxes in divergence form (mom.f90:66-71, 110-115, 150-155)
    const double uuip = 0.25 * (U(ip, j, k) + U(i, j, k)) * (U(ip, j, k) + U(i, j, k));
    const double uuim = 0.25 * (U(im, j, k) + U(i, j, k)) * (U(im, j, k) + U(i, j, k));
    const double uvjp = 0.25 * (U(i, jp, k) + U(i, j, k)) * (V(ip, j, k) + V(i, j, k));
    const double uvjm = 0.25 * (U(i, jm, k) + U(i, j, k)) * (V(ip, jm, k) + V(i, jm, k));
    const double uwkp = 0.25 * (U(i, j, kp) + U(i, j, k)) * (W(ip, j, k) + W(i, j, k));
    const double uwkm = 0.25 * (U(i, j, km) + U(i, j, k)) * (W(ip, j, km) + W(i, j, km));
    adv_u = dxi * (-uuip + uuim) + dyi * (-uvjp + uvjm) + zfi * (-uwkp + uwkm);
    const double uvip = 0.25 * (U(i, j, k) + U(i, jp, k)) * (V(i, j, k) + V(ip, j, k));
    const double uvim = 0.25 * (U(im, j, k) + U(im, jp, k)) * (V(i, j, k) + V(im, j, k));
    const double vvjp = 0.25 * (V(i, j, k) + V(i, jp, k)) * (V(i, j, k) + V(i, jp, k));
    const double vvjm = 0.25 * (V(i, j, k) + V(i, jm, k)) * (V(i, j, k) + V(i, jm, k));
    const double wvkp = 0.25 * (W(i, j, k) + W(i, jp, k)) * (V(i, j, kp) + V(i, j, k));
    const double wvkm = 0.25 * (W(i, j, km) + W(i, jp, km)) * (V(i, j, km) + V(i, j, k));
    adv_v = dxi * (-uvip + uvim) + dyi * (-vvjp + vvjm) + zfi * (-wvkp + wvkm);
    const double uwip = 0.25 * (W(i, j, k) + W(ip, j, k)) * (U(i, j, k) + U(i, j, kp));
    const double uwim = 0.25 * (W(i, j, k) + W(im, j, k)) * (U(im, j, k) + U(im, j, kp));
    const double vwjp = 0.25 * (W(i, j, k) + W(i, jp, k)) * (V(i, j, k) + V(i, j, kp));
    const double vwjm = 0.25 * (W(i, j, k) + W(i, jm, k)) * (V(i, jm, k) + V(i, jm, kp));
    const double wwkp = 0.25 * (W(i, j, k) + W(i, j, kp)) * (W(i, j, k) + W(i, j, kp));
    const double wwkm = 0.25 * (W(i, j, k) + W(i, j, km)) * (W(i, j, k) + W(i, j, km));
    adv_w = dxi * (-uwip + uwim) + dyi * (-vwjp + vwjm) + zci * (-wwkp + wwkm);
  } else {
    // fourth-order gradient form with an upwind-biased fourth difference (mom.f90:231-290 etc.)
    auto g4 = [](double f1, double f2, double f3, double f4, double f5, double c, double dl) {
      return c * (f1 - 8.0 * f2 + 8.0 * f4 - f5) * (1.0 / 12.0) * dl +
             3.0 * fabs(c) * (f1 - 4.0 * f2 + 6.0 * f3 - 4.0 * f4 + f5) * (1.0 / 12.0) * dl;
    };
    double uc = U(i, j, k);
    double vc = 0.25 * (V(i, j, k) + V(ip, j, k) + V(i, jm, k) + V(ip, jm, k));
    double wc = 0.25 * (W(i, j, k) + W(ip, j, k) + W(i, j, km) + W(ip, j, km));
    adv_u = -(g4(U(i - 2, j, k), U(i - 1, j, k), U(i, j, k), U(i + 1, j, k), U(i + 2, j, k), uc, dxi) +
              g4(U(i, j - 2, k), U(i, j - 1, k), U(i, j, k), U(i, j + 1, k), U(i, j + 2, k), vc, dyi) +
              g4(U(i, j, k - 2), U(i, j, k - 1), U(i, j, k), U(i, j, k + 1), U(i, j, k + 2), wc, dzi));
    uc = 0.25 * (U(i, j, k) + U(i, jp, k) + U(im, j, k) + U(im, jp, k));
    vc = V(i, j, k);
    wc = 0.25 * (W(i, j, k) + W(i, jp, k) + W(i, j, km) + W(i, jp, km));
    adv_v = -(g4(V(i - 2, j, k), V(i - 1, j, k), V(i, j, k), V(i + 1, j, k), V(i + 2, j, k), uc, dxi) +
              g4(V(i, j - 2, k), V(i, j - 1, k), V(i, j, k), V(i, j + 1, k), V(i, j + 2, k), vc, dyi) +
              g4(V(i, j, k - 2), V(i, j, k - 1), V(i, j, k), V(i, j, k + 1), V(i, j, k + 2), wc, dzi));
    uc = 0.25 * (U(i, j, k) + U(i, j, kp) + U(im, j, k) + U(im, j, kp));
    vc = 0.25 * (V(i, j, k) + V(i, j, kp) + V(i, jm, k) + V(i, jm, kp));
    wc = W(i, j, k);
    adv_w = -(g4(W(i - 2, j, k), W(i - 1, j, k), W(i, j, k), W(i + 1, j, k), W(i + 2, j, k), uc, dxi) +
              g4(W(i, j - 2, k), W(i, j - 1, k), W(i, j, k), W(i, j + 1, k), W(i, j + 2, k), vc, dyi) +
              g4(W(i, j, k - 2), W(i, j, k - 1), W(i, j, k), W(i, j, k + 1), W(i, j, k + 2), wc, dzi));
  }
  // x-momentum viscous term
  {
    const double dudxp = (U(ip, j, k) - U(i, j, k)) * dxi, dudxm = (U(i, j, k) - U(im, j, k)) * dxi;
    const double dudyp = (U(i, jp, k) - U(i, j, k)) * dyi, dudym = (U(i, j, k) - U(i, jm, k)) * dyi;
    const double dudzp = (U(i, j, kp) - U(i, j, k)) * zci, dudzm = (U(i, j, k) - U(i, j, km)) * zcim;
    if constexpr (VAR == MOM_SP) {
      du = adv_u + (dxi * (dudxp - dudxm) + dyi * (dudyp - dudym) + zfi * (dudzp - dudzm)) * a.visc;
    } else {
      const double dvdxp = (V(ip, j, k) - V(i, j, k)) * dxi, dvdxm = (V(ip, jm, k) - V(i, jm, k)) * dxi;
      const double dwdxp = (W(ip, j, k) - W(i, j, k)) * dxi, dwdxm = (W(ip, j, km) - W(i, j, km)) * dxi;
      const double muxp = MU(ip, j, k), muxm = MU(i, j, k);
      const double muyp = 0.25 * (MU(i, j, k) + MU(i, jp, k) + MU(ip, jp, k) + MU(ip, j, k));
      const double muym = 0.25 * (MU(i, j, k) + MU(i, jm, k) + MU(ip, jm, k) + MU(ip, j, k));
      const double muzp = 0.25 * (MU(i, j, k) + MU(i, j, kp) + MU(ip, j, kp) + MU(ip, j, k));
      const double muzm = 0.25 * (MU(i, j, k) + MU(i, j, km) + MU(ip, j, km) + MU(ip, j, k));
      const double rhox = 0.5 * (RHO(ip, j, k) + RHO(i, j, k));
      du = adv_u + (dxi * ((dudxp + dudxp) * muxp - (dudxm + dudxm) * muxm) +
                    dyi * ((dudyp + dvdxp) * muyp - (dudym + dvdxm) * muym) +
                    zfi * ((dudzp + dwdxp) * muzp - (dudzm + dwdxm) * muzm)) / rhox;
    }
  }
  // y-momentum viscous term
  {
    const double dvdxp = (V(ip, j, k) - V(i, j, k)) * dxi, dvdxm = (V(i, j, k) - V(im, j, k)) * dxi;
    const double dvdyp = (V(i, jp, k) - V(i, j, k)) * dyi, dvdym = (V(i, j, k) - V(i, jm, k)) * dyi;
    const double dvdzp = (V(i, j, kp) - V(i, j, k)) * zci, dvdzm = (V(i, j, k) - V(i, j, km)) * zcim;
    if constexpr (VAR == MOM_SP) {
      dv = adv_v + (dxi * (dvdxp - dvdxm) + dyi * (dvdyp - dvdym) + zfi * (dvdzp - dvdzm)) * a.visc;
    } else {
      const double dudyp = (U(i, jp, k) - U(i, j, k)) * dyi, dudym = (U(im, jp, k) - U(im, j, k)) * dyi;
      const double dwdyp = (W(i, jp, k) - W(i, j, k)) * dyi, dwdym = (W(i, jp, km) - W(i, j, km)) * dyi;
      const double muxp = 0.25 * (MU(i, j, k) + MU(ip, j, k) + MU(ip, jp, k) + MU(i, jp, k));
      const double muxm = 0.25 * (MU(i, j, k) + MU(im, j, k) + MU(im, jp, k) + MU(i, jp, k));
      const double muyp = MU(i, jp, k), muym = MU(i, j, k);
      const double muzp = 0.25 * (MU(i, j, k) + MU(i, jp, k) + MU(i, jp, kp) + MU(i, j, kp));
      const double muzm = 0.25 * (MU(i, j, k) + MU(i, jp, k) + MU(i, jp, km) + MU(i, j, km));
      const double rhoy = 0.5 * (RHO(i, jp, k) + RHO(i, j, k));
      dv = adv_v + (dxi * ((dvdxp + dudyp) * muxp - (dvdxm + dudym) * muxm) +
                    dyi * ((dvdyp + dvdyp) * muyp - (dvdym + dvdym) * muym) +
                    zfi * ((dvdzp + dwdyp) * muzp - (dvdzm + dwdym) * muzm)) / rhoy;
    }
  }
  // z-momentum viscous term
  {
    const double dwdxp = (W(ip, j, k) - W(i, j, k)) * dxi, dwdxm = (W(i, j, k) - W(im, j, k)) * dxi;
    const double dwdyp = (W(i, jp, k) - W(i, j, k)) * dyi, dwdym = (W(i, j, k) - W(i, jm, k)) * dyi;
    const double dwdzp = (W(i, j, kp) - W(i, j, k)) * zfip, dwdzm = (W(i, j, k) - W(i, j, km)) * zfi;
    if constexpr (VAR == MOM_SP) {
      dw = adv_w + (dxi * (dwdxp - dwdxm) + dyi * (dwdyp - dwdym) + zci * (dwdzp - dwdzm)) * a.visc;
    } else {
      const double dudzp = (U(i, j, kp) - U(i, j, k)) * zci, dudzm = (U(im, j, kp) - U(im, j, k)) * zci;
      const double dvdzp = (V(i, j, kp) - V(i, j, k)) * zci, dvdzm = (V(i, jm, kp) - V(i, jm, k)) * zci;
      const double muxp = 0.25 * (MU(i, j, k) + MU(i, j, kp) + MU(ip, j, kp) + MU(ip, j, k));
      const double muxm = 0.25 * (MU(i, j, k) + MU(i, j, kp) + MU(im, j, kp) + MU(im, j, k));
      const double muyp = 0.25 * (MU(i, j, k) + MU(i, j, kp) + MU(i, jp, kp) + MU(i, jp, k));
      const double muym = 0.25 * (MU(i, j, k) + MU(i, j, kp) + MU(i, jm, kp) + MU(i, jm, k));
      const double muzp = MU(i, j, kp), muzm = MU(i, j, k);
      const double rhoz = 0.5 * (RHO(i, j, kp) + RHO(i, j, k));
      dw = adv_w + (dxi * ((dwdxp + dudzp) * muxp - (dwdxm + dudzm) * muxm) +
                    dyi * ((dwdyp + dvdzp) * muyp - (dwdym + dvdzm) * muym) +
                    zci * ((dwdzp + dwdzp) * muzp - (dwdzm + dwdzm) * muzm)) / rhoz;
    }
  }
#undef U
#undef V
#undef W
#undef MU
#undef RHO
}

// Right-hand sides and the new velocities (rk.f90:81-90) of every interior
// cell; x fastest across the threads of a warp (coalesced).
template <int VAR>
__global__ void __launch_bounds__(256) k_mom_rk(MomArgs a) {
  const long tot = (long)a.nx * a.ny * a.nz;
  const long UX = a.nx + 2 * a.h, UY = a.ny + 2 * a.h;
  for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < tot; c += (long)gridDim.x * blockDim.x) {
    const long row = c / a.nx, kk = row / a.ny;
    const int i = (int)(c - row * a.nx) + 1, j = (int)(row - kk * a.ny) + 1, k = (int)kk + 1;
    double du, dv, dw;
    mom_cell<VAR>(a, i, j, k, du, dv, dw);
    const long q = (long)(i - 1 + a.h) + UX * ((long)(j - 1 + a.h) + UY * (long)(k - 1 + a.h));
    a.un[c] = a.u[q] + a.f1 * du + a.f2 * a.du0[c];
    a.vn[c] = a.v[q] + a.f1 * dv + a.f2 * a.dv0[c];
    a.wn[c] = a.w[q] + a.f1 * dw + a.f2 * a.dw0[c];
    a.du0[c] = du;
    a.dv0[c] = dv;
    a.dw0[c] = dw;
  }
}

// The new velocities into the interior of u, v, w (the halo is left as it was).
__global__ void k_mom_store(int nx, int ny, int nz, int h, const double *un, const double *vn, const double *wn,
                            double *u, double *v, double *w) {
  const long tot = (long)nx * ny * nz;
  const long UX = nx + 2 * h, UY = ny + 2 * h;
  for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < tot; c += (long)gridDim.x * blockDim.x) {
    const long row = c / nx, k = row / ny;
    const long i = c - row * nx, j = row - k * ny;
    const long q = (i + h) + UX * ((j + h) + UY * (k + h));
    u[q] = un[c];
    v[q] = vn[c];
    w[q] = wn[c];
  }
}

// Device buffers of the predictor: three scratch fields and mirrors of host arrays.
struct Buf {
  void *p = nullptr;
  size_t bytes = 0;
  int ensure(size_t b) {
    if (b <= bytes) return 0;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    if (cudaMalloc(&p, b) != cudaSuccess) {
      cudaGetLastError();
      return mfail(FLUTAS_ENOMEM, "rk: cudaMalloc(%zu) failed", b);
    }
    bytes = b;
    return 0;
  }
};
std::mutex g_mom_mu;
Buf g_scratch;
std::vector<Buf> g_mirror(11);

// A device view of an array argument: used in place when it is device memory of
// this device (or managed), else copied to a mirror (and back after, if `out`).
struct Arg {
  double *d = nullptr;
  const void *host = nullptr;
  size_t bytes = 0;
  bool out = false;
};
int view(int slot, const void *user, size_t bytes, bool out, Arg *a) {
  if (!user) return mfail(FLUTAS_EINVAL, "rk: null array argument");
  cudaPointerAttributes at;
  const bool ok = cudaPointerGetAttributes(&at, user) == cudaSuccess;
  if (!ok) cudaGetLastError();
  int cur = 0;
  cudaGetDevice(&cur);
  const int kind = fg::classify_ptr(ok, ok ? (int)at.type : 0, ok ? at.device : -1, cur);
  if (kind == fg::PTR_OTHER_DEVICE) return mfail(FLUTAS_EINVAL, "rk: an array lives on another device");
  a->bytes = bytes;
  a->out = out;
  if (kind == fg::PTR_DEVICE) {
    a->d = (double *)user;
    return 0;
  }
  if (int rc = g_mirror[slot].ensure(bytes)) return rc;
  a->d = (double *)g_mirror[slot].p;
  a->host = user;
  MCK(cudaMemcpyAsync(a->d, user, bytes, cudaMemcpyHostToDevice, 0));
  return 0;
}

int run_rk(int variant, double f_t1, double f_t2, int nx, int ny, int nz, double dxi, double dyi, double dzi,
           int nh_d, int nh_u, const double *dzci, const double *dzfi, double *u, double *v, double *w,
           const double *mu, const double *rho, double visc, double *dudtrko, double *dvdtrko, double *dwdtrko) {
  if (nx < 1 || ny < 1 || nz < 1 || nh_d < 1 || nh_u < 1) return mfail(FLUTAS_EINVAL, "rk: bad sizes");
  const int need = variant == MOM_FLL ? 2 : 1;  // the flux-limiter stencil reaches two cells out
  if (nh_u < need || nh_d < 1)
    return mfail(FLUTAS_EINVAL, "rk: the '%s' scheme needs nh_u >= %d", variant == MOM_FLL ? "fll" : "cen", need);
  std::lock_guard<std::mutex> lk(g_mom_mu);
  const size_t N = (size_t)nx * ny * nz;
  const size_t ub = sizeof(double) * (size_t)(nx + 2 * nh_u) * (ny + 2 * nh_u) * (nz + 2 * nh_u);
  const size_t pb = sizeof(double) * (size_t)(nx + 2) * (ny + 2) * (nz + 2);
  const size_t zb = sizeof(double) * (size_t)(nz + 2 * nh_d);
  Arg A[11];
  int rc;
  if ((rc = view(0, u, ub, true, &A[0])) || (rc = view(1, v, ub, true, &A[1])) || (rc = view(2, w, ub, true, &A[2])) ||
      (rc = view(3, dudtrko, sizeof(double) * N, true, &A[3])) || (rc = view(4, dvdtrko, sizeof(double) * N, true, &A[4])) ||
      (rc = view(5, dwdtrko, sizeof(double) * N, true, &A[5])) || (rc = view(6, dzci, zb, false, &A[6])) ||
      (rc = view(7, dzfi, zb, false, &A[7])))
    return rc;
  if (variant != MOM_SP && ((rc = view(8, mu, pb, false, &A[8])) || (rc = view(9, rho, pb, false, &A[9]))))
    return rc;
  if ((rc = g_scratch.ensure(3 * sizeof(double) * N))) return rc;
  MomArgs a;
  a.nx = nx; a.ny = ny; a.nz = nz; a.h = nh_u;
  a.dxi = dxi; a.dyi = dyi; a.dzi = dzi;
  a.dzci = A[6].d + (nh_d - 1);
  a.dzfi = A[7].d + (nh_d - 1);
  a.u = A[0].d; a.v = A[1].d; a.w = A[2].d;
  a.mu = variant != MOM_SP ? A[8].d : nullptr;
  a.rho = variant != MOM_SP ? A[9].d : nullptr;
  a.visc = visc;
  a.f1 = f_t1; a.f2 = f_t2;
  a.un = (double *)g_scratch.p; a.vn = a.un + N; a.wn = a.vn + N;
  a.du0 = A[3].d; a.dv0 = A[4].d; a.dw0 = A[5].d;
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = (int)std::min<long>((long)((N + 255) / 256), (long)std::max(sms, 1) * 8);
  if (variant == MOM_CEN) k_mom_rk<MOM_CEN><<<grid, 256>>>(a);
  else if (variant == MOM_FLL) k_mom_rk<MOM_FLL><<<grid, 256>>>(a);
  else k_mom_rk<MOM_SP><<<grid, 256>>>(a);
  MCK(cudaGetLastError());
  k_mom_store<<<grid, 256>>>(nx, ny, nz, nh_u, a.un, a.vn, a.wn, A[0].d, A[1].d, A[2].d);
  MCK(cudaGetLastError());
  fg_note_launches(2);
  for (int t = 0; t < 6; t++)
    if (A[t].host) MCK(cudaMemcpyAsync((void *)A[t].host, A[t].d, A[t].bytes, cudaMemcpyDeviceToHost, 0));
  MCK(cudaStreamSynchronize(0));
  return FLUTAS_OK;
}

}  // namespace

extern "C" {

int flutas_gb300_rk(const char space_scheme_mom[3], double f_t1, double f_t2, int nx, int ny, int nz, double dxi,
                    double dyi, double dzi, int nh_d, int nh_u, const double *dzci, const double *dzfi, double *u,
                    double *v, double *w, const double *mu, const double *rho, double *dudtrko, double *dvdtrko,
                    double *dwdtrko) {
  // src/rk.f90:26-102 with the two-phase right-hand sides (_USE_VOF)
  if (!space_scheme_mom) return mfail(FLUTAS_EINVAL, "rk: null space_scheme_mom");
  int variant;
  if (!strncmp(space_scheme_mom, "cen", 3)) variant = MOM_CEN;
  else if (!strncmp(space_scheme_mom, "fll", 3)) variant = MOM_FLL;
  else return mfail(FLUTAS_EINVAL, "Invalid space discretization for momentum equation - check dns.in");
  return run_rk(variant, f_t1, f_t2, nx, ny, nz, dxi, dyi, dzi, nh_d, nh_u, dzci, dzfi, u, v, w, mu, rho, 0.0,
                dudtrko, dvdtrko, dwdtrko);
}

int flutas_gb300_rk_sp(double f_t1, double f_t2, int nx, int ny, int nz, double dxi, double dyi, double dzi,
                       int nh_d, int nh_u, const double *dzci, const double *dzfi, double visc_sp, double *u,
                       double *v, double *w, double *dudtrko, double *dvdtrko, double *dwdtrko) {
  // src/rk.f90:26-102 with momad_xyz_sp (the single-phase build): visc_sp = mu_sp/rho_sp
  return run_rk(MOM_SP, f_t1, f_t2, nx, ny, nz, dxi, dyi, dzi, nh_d, nh_u, dzci, dzfi, u, v, w, nullptr, nullptr,
                visc_sp, dudtrko, dvdtrko, dwdtrko);
}

int flutas_gb300_cmpt_time_factors(const char time_scheme[3], int restart, int istep, int irk_ss,
                                   const double rkcoeff[6], double dt, double dto, double *f_t1, double *f_t2,
                                   double *f_t12) {
  // src/rk.f90:104-135 (restart is accepted and unused, as in the reference)
  (void)restart;
  if (!time_scheme || !f_t1 || !f_t2 || !f_t12) return mfail(FLUTAS_EINVAL, "cmpt_time_factors: null argument");
  if (!strncmp(time_scheme, "ab2", 3)) {
    if (istep == 1) {  // first-order Euler in the first time step
      *f_t1 = 1.0 * dt;
      *f_t2 = 0.0 * dt;
    } else {
      *f_t1 = (1.0 + 0.5 * (dt / dto)) * dt;
      *f_t2 = (-0.5 * (dt / dto)) * dt;
    }
  } else if (!strncmp(time_scheme, "rk3", 3)) {
    if (!rkcoeff || irk_ss < 1 || irk_ss > 3) return mfail(FLUTAS_EINVAL, "cmpt_time_factors: bad rk3 substep");
    *f_t1 = rkcoeff[0 + 2 * (irk_ss - 1)] * dt;  // rkcoeff(1,irk_ss)
    *f_t2 = rkcoeff[1 + 2 * (irk_ss - 1)] * dt;  // rkcoeff(2,irk_ss)
  } else {
    return mfail(FLUTAS_EINVAL, "Invalid time discretization: only AB2 and RK3 available for now - check dns.in");
  }
  *f_t12 = *f_t1 + *f_t2;
  return FLUTAS_OK;
}

}  // extern "C"
