// grid.cu -- initgrid (src/initgrid.f90:17-97): the z grid of FluTAS, on the host.
//
// The apps compute dzc, dzf, zc, zf once at start-up and pass dzci = 1/dzc,
// dzfi = 1/dzf to initsolver, fillps and correc.  The grid itself is cheap
// host work; it is part of this library so an app (or a test) gets the exact
// spacings the solver's coefficients are built from.  Restated step by step:
// face coordinates from the clustering function, spacings, centres, then the
// mirrored extension into the halo.
#include "../../include/flutas_gb300.h"

#include <cmath>
#include <cstring>

void fg_set_error_text(const char *msg);  // flutas_gb300.cu

namespace {

// gridpoint_cluster_two_end (src/initgrid.f90:102-118)
double cluster_two_end(double alpha, double z0) {
  return alpha != 0.0 ? 0.5 * (1.0 + std::tanh((z0 - 0.5) * alpha) / std::tanh(alpha / 2.0)) : z0;
}
// gridpoint_cluster_one_end (src/initgrid.f90:120-135)
double cluster_one_end(double alpha, double z0) {
  return alpha != 0.0 ? 1.0 * (1.0 + std::tanh((z0 - 1.0) * alpha) / std::tanh(alpha / 1.0)) : z0;
}

}  // namespace

extern "C" int flutas_gb300_initgrid(const char inivel[3], int n, double gr, double lz, int nh_d, double *dzc,
                                     double *dzf, double *zc, double *zf) {
  if (!inivel || !dzc || !dzf || !zc || !zf || n < 1 || nh_d < 1 || nh_d > n) {
    fg_set_error_text("initgrid: null argument or bad n / nh_d");
    return FLUTAS_EINVAL;
  }
  // 'hcl' and 'hcp' cluster at the lower wall, every other initial condition at both (20-38)
  const bool one_end = !strncmp(inivel, "hcl", 3) || !strncmp(inivel, "hcp", 3);
  auto at = [&](double *x, int k) -> double & { return x[k - 1 + nh_d]; };  // x(1-nh_d:n+nh_d)
  for (int k = 1; k <= n; k++) {
    const double z0 = (k - 0.0) / (1.0 * n);
    at(zf, k) = (one_end ? cluster_one_end(gr, z0) : cluster_two_end(gr, z0)) * lz;
  }
  at(zf, 0) = 0.0;
  for (int k = 1; k <= n; k++) at(dzf, k) = at(zf, k) - at(zf, k - 1);
  at(dzf, 0) = at(dzf, 1);
  at(dzf, n + 1) = at(dzf, n);
  for (int k = 0; k <= n; k++) at(dzc, k) = 0.5 * (at(dzf, k) + at(dzf, k + 1));
  at(dzc, n + 1) = at(dzc, n);
  at(zc, 0) = -at(dzc, 0) / 2.0;
  at(zf, 0) = 0.0;
  for (int k = 1; k <= n + 1; k++) {
    at(zc, k) = at(zc, k - 1) + at(dzc, k - 1);
    at(zf, k) = at(zf, k - 1) + at(dzf, k);
  }
  for (int k = 1 - nh_d; k <= 0; k++) {
    at(dzf, k) = at(dzf, -k + 1);
    at(dzc, k) = at(dzc, -k);
  }
  for (int k = n + 1; k <= n + nh_d; k++) {
    at(dzf, k) = at(dzf, 2 * n - k - 1);
    at(dzc, k) = at(dzc, 2 * n - k);
  }
  for (int k = 0; k >= 1 - nh_d; k--) {
    at(zf, k) = at(zf, k + 1) - at(dzf, k);
    at(zc, k) = at(zf, k + 1) - at(dzc, k + 1);
  }
  for (int k = n + 1; k <= n + nh_d; k++) {
    at(zf, k) = at(zf, k - 1) + at(dzf, k);
    at(zc, k) = at(zf, k - 1) + at(dzc, k - 1);
  }
  return FLUTAS_OK;
}
