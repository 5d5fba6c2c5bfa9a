// io.cu -- restart-file I/O of the projection's fields (src/load.f90).
//
// The reference reads and writes each field as raw FP64 values of the global
// interior, x fastest, no header (load, src/load.f90:21-89), checks the file
// size against n(1)*n(2)*n(3)*8 bytes before reading, and keeps the time,
// time step and step number in a small text file (load_scalar, 91-128) or,
// in the CaNS layout, after four fields in one file (load_ns, 130-214).
// Here the fields move straight between the file and the interior of a halo
// array in host or device memory: device fields go through two pinned
// buffers of whole z-planes, one copy per plane (pitched rows into the halo
// layout), so reading a chunk from the file overlaps the copy of the last.
#include "../../include/flutas_gb300.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

void fg_set_error_text(const char *msg);  // flutas_gb300.cu

namespace {

int io_fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  fg_set_error_text(buf);
  return code;
}

bool on_device(const void *p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice;
}

struct Field {
  double *p;
  long n0, n1, n2;
  int nh;
  bool dev;
  long ldx() const { return n0 + 2 * nh; }
  long ldy() const { return n1 + 2 * nh; }
  // element (i,j,k) of the interior, 0-based
  double *at(long i, long j, long k) const { return p + (i + nh) + ldx() * ((j + nh) + ldy() * (k + nh)); }
};

// Pinned double buffer for device fields (plain memory for host fields).
struct Bounce {
  double *b[2] = {nullptr, nullptr};
  bool pinned = false;
  cudaEvent_t done[2] = {nullptr, nullptr};
  ~Bounce() {
    for (int i = 0; i < 2; i++) {
      if (done[i]) cudaEventDestroy(done[i]);
      if (b[i]) pinned ? (void)cudaFreeHost(b[i]) : free(b[i]);
    }
  }
  int alloc(size_t bytes, bool dev) {
    pinned = dev;
    for (int i = 0; i < 2; i++) {
      if (dev) {
        if (cudaMallocHost((void **)&b[i], bytes) != cudaSuccess || cudaEventCreate(&done[i]) != cudaSuccess) {
          cudaGetLastError();
          return io_fail(FLUTAS_ENOMEM, "load: pinned staging buffer of %zu bytes not available", bytes);
        }
      } else if (!(b[i] = (double *)malloc(bytes))) {
        return io_fail(FLUTAS_ENOMEM, "load: staging buffer of %zu bytes not available", bytes);
      }
    }
    return 0;
  }
};

// Planes [k0, k0+np) between a contiguous buffer (planes of n0*n1 values) and the field.
int planes_in(const Field &f, const double *buf, long k0, long np, cudaStream_t st) {
  const long row = f.n0, plane = f.n0 * f.n1;
  for (long k = 0; k < np; k++) {
    if (f.dev) {
      if (cudaMemcpy2DAsync(f.at(0, 0, k0 + k), sizeof(double) * f.ldx(), buf + k * plane, sizeof(double) * row,
                            sizeof(double) * row, f.n1, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return io_fail(FLUTAS_ECUDA, "load: copy to the device failed: %s", cudaGetErrorString(cudaGetLastError()));
    } else {
      for (long j = 0; j < f.n1; j++) memcpy(f.at(0, j, k0 + k), buf + k * plane + j * row, sizeof(double) * row);
    }
  }
  return 0;
}
int planes_out(const Field &f, double *buf, long k0, long np, cudaStream_t st) {
  const long row = f.n0, plane = f.n0 * f.n1;
  for (long k = 0; k < np; k++) {
    if (f.dev) {
      if (cudaMemcpy2DAsync(buf + k * plane, sizeof(double) * row, f.at(0, 0, k0 + k), sizeof(double) * f.ldx(),
                            sizeof(double) * row, f.n1, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return io_fail(FLUTAS_ECUDA, "load: copy from the device failed: %s",
                       cudaGetErrorString(cudaGetLastError()));
    } else {
      for (long j = 0; j < f.n1; j++) memcpy(buf + k * plane + j * row, f.at(0, j, k0 + k), sizeof(double) * row);
    }
  }
  return 0;
}

constexpr size_t CHUNK_BYTES = 64u << 20;

// Reads n0*n1*n2 values at the file's current position into the field.
int read_field(FILE *fp, const char *name, const Field &f) {
  const long plane = f.n0 * f.n1;
  if (!f.dev && f.nh == 0) {  // host interior: straight into place
    if (fread(f.p, sizeof(double), (size_t)(plane * f.n2), fp) != (size_t)(plane * f.n2))
      return io_fail(FLUTAS_EINVAL, "load: short read from %s", name);
    return 0;
  }
  const long per = std::max(1L, (long)(CHUNK_BYTES / (sizeof(double) * plane)));
  Bounce bb;
  if (int rc = bb.alloc(sizeof(double) * plane * std::min(per, f.n2), f.dev)) return rc;
  cudaStream_t st = 0;
  int c = 0;
  for (long k0 = 0; k0 < f.n2; k0 += per, c ^= 1) {
    const long np = std::min(per, f.n2 - k0);
    if (f.dev && cudaEventSynchronize(bb.done[c]) != cudaSuccess)  // the copy out of this buffer is finished
      return io_fail(FLUTAS_ECUDA, "load: %s", cudaGetErrorString(cudaGetLastError()));
    if (fread(bb.b[c], sizeof(double), (size_t)(np * plane), fp) != (size_t)(np * plane))
      return io_fail(FLUTAS_EINVAL, "load: short read from %s", name);
    if (int rc = planes_in(f, bb.b[c], k0, np, st)) return rc;
    if (f.dev && cudaEventRecord(bb.done[c], st) != cudaSuccess)
      return io_fail(FLUTAS_ECUDA, "load: %s", cudaGetErrorString(cudaGetLastError()));
  }
  if (f.dev && cudaStreamSynchronize(st) != cudaSuccess)
    return io_fail(FLUTAS_ECUDA, "load: %s", cudaGetErrorString(cudaGetLastError()));
  return 0;
}

int write_field(FILE *fp, const char *name, const Field &f) {
  const long plane = f.n0 * f.n1;
  if (!f.dev && f.nh == 0) {
    if (fwrite(f.p, sizeof(double), (size_t)(plane * f.n2), fp) != (size_t)(plane * f.n2))
      return io_fail(FLUTAS_EINVAL, "load: short write to %s", name);
    return 0;
  }
  const long per = std::max(1L, (long)(CHUNK_BYTES / (sizeof(double) * plane)));
  Bounce bb;
  if (int rc = bb.alloc(sizeof(double) * plane * std::min(per, f.n2), f.dev)) return rc;
  cudaStream_t st = 0;
  for (long k0 = 0; k0 < f.n2; k0 += per) {
    const long np = std::min(per, f.n2 - k0);
    if (int rc = planes_out(f, bb.b[0], k0, np, st)) return rc;
    if (f.dev && cudaStreamSynchronize(st) != cudaSuccess)
      return io_fail(FLUTAS_ECUDA, "load: %s", cudaGetErrorString(cudaGetLastError()));
    if (fwrite(bb.b[0], sizeof(double), (size_t)(np * plane), fp) != (size_t)(np * plane))
      return io_fail(FLUTAS_EINVAL, "load: short write to %s", name);
  }
  return 0;
}

int check_args(char io, const char *filename, const int n[3], int nh) {
  if (io != 'r' && io != 'w') return io_fail(FLUTAS_EINVAL, "load: io must be 'r' or 'w', got '%c'", io);
  if (!filename || !n) return io_fail(FLUTAS_EINVAL, "load: null argument");
  if (n[0] < 1 || n[1] < 1 || n[2] < 1 || nh < 0 || nh > 8) return io_fail(FLUTAS_EINVAL, "load: bad sizes");
  return 0;
}

// Opens `filename` for reading after the reference's checks: it must exist
// and hold exactly `good` bytes (src/load.f90:40-66).
int open_checked(const char *filename, long long good, FILE **out) {
  FILE *fp = fopen(filename, "rb");
  if (!fp) return io_fail(FLUTAS_EINVAL, "The restarting field %s does not exist", filename);
  fseek(fp, 0, SEEK_END);
  const long long size = ftell(fp);
  fseek(fp, 0, SEEK_SET);
  if (size != good) {
    fclose(fp);
    return io_fail(FLUTAS_EINVAL, "checkpoint file with incorrect size: file %s | expected size: %lld | actual size: %lld",
                   filename, good, size);
  }
  *out = fp;
  return 0;
}

// Fortran Ew.d edit descriptor (0.ddddE+ee form, right-justified in w).
std::string fortran_e(double x, int w, int d) {
  char tmp[64];
  snprintf(tmp, sizeof tmp, "%.*e", d - 1, std::fabs(x));  // d.ddd...e+XX
  std::string digits;
  const char *c = tmp;
  for (; *c && *c != 'e'; c++)
    if (*c != '.') digits += *c;
  int ex = atoi(c + 1);
  const bool zero = x == 0.0;
  if (!zero) ex += 1;  // 0.ddd form
  char exs[16];
  if (std::abs(ex) <= 99) snprintf(exs, sizeof exs, "E%c%02d", ex < 0 ? '-' : '+', std::abs(ex));
  else snprintf(exs, sizeof exs, "%c%03d", ex < 0 ? '-' : '+', std::abs(ex));
  std::string s = std::string(std::signbit(x) && !zero ? "-" : "") + "0." + digits + exs;
  if ((int)s.size() < w) s = std::string(w - s.size(), ' ') + s;
  return s;
}

}  // namespace

extern "C" {

int flutas_gb300_load(char io, const char *filename, const int n[3], int nh, double *fld) {
  if (int rc = check_args(io, filename, n, nh)) return rc;
  if (!fld) return io_fail(FLUTAS_EINVAL, "load: null field");
  Field f{fld, n[0], n[1], n[2], nh, on_device(fld)};
  const long long good = 8LL * n[0] * n[1] * n[2];
  if (io == 'r') {
    FILE *fp = nullptr;
    if (int rc = open_checked(filename, good, &fp)) return rc;
    const int rc = read_field(fp, filename, f);
    fclose(fp);
    return rc;
  }
  FILE *fp = fopen(filename, "wb");  // created or truncated, as MPI_FILE_SET_SIZE(0) does
  if (!fp) return io_fail(FLUTAS_EINVAL, "load: cannot create %s", filename);
  const int rc = write_field(fp, filename, f);
  if (fclose(fp) != 0 && rc == 0) return io_fail(FLUTAS_EINVAL, "load: cannot write %s", filename);
  return rc;
}

int flutas_gb300_load_scalar(char io, const char *filename, double *time, int *istep, double *dto) {
  if (io != 'r' && io != 'w') return io_fail(FLUTAS_EINVAL, "load_scalar: io must be 'r' or 'w'");
  if (!filename || !time || !istep || !dto) return io_fail(FLUTAS_EINVAL, "load_scalar: null argument");
  if (io == 'r') {
    FILE *fp = fopen(filename, "r");
    if (!fp) return io_fail(FLUTAS_EINVAL, "The restarting field %s does not exist", filename);
    char line[512] = {0};
    std::string all;
    while (fgets(line, sizeof line, fp)) all += line;
    fclose(fp);
    for (char &ch : all)  // list-directed input: D exponents and comma separators
      if (ch == 'D' || ch == 'd') ch = 'E';
      else if (ch == ',') ch = ' ';
    char *end = nullptr;
    const char *c = all.c_str();
    const double t = strtod(c, &end);
    if (end == c) return io_fail(FLUTAS_EINVAL, "load_scalar: no time in %s", filename);
    c = end;
    const double dt = strtod(c, &end);
    if (end == c) return io_fail(FLUTAS_EINVAL, "load_scalar: no dto in %s", filename);
    c = end;
    const long st = strtol(c, &end, 10);
    if (end == c) return io_fail(FLUTAS_EINVAL, "load_scalar: no istep in %s", filename);
    *time = t;
    *dto = dt;
    *istep = (int)st;
    return FLUTAS_OK;
  }
  FILE *fp = fopen(filename, "w");
  if (!fp) return io_fail(FLUTAS_EINVAL, "load_scalar: cannot create %s", filename);
  // write(88,'(2E15.7, 1I9.8)') time, dto, istep
  char num[32];
  snprintf(num, sizeof num, "%0*d", *istep < 0 ? 9 : 8, *istep);
  std::string s = fortran_e(*time, 15, 7) + fortran_e(*dto, 15, 7);
  std::string is = num;
  if ((int)is.size() < 9) is = std::string(9 - is.size(), ' ') + is;
  s += is + "\n";
  const bool ok = fputs(s.c_str(), fp) >= 0;
  if (fclose(fp) != 0 || !ok) return io_fail(FLUTAS_EINVAL, "load_scalar: cannot write %s", filename);
  return FLUTAS_OK;
}

int flutas_gb300_load_ns(char io, const char *filename, const int n[3], int nh, double *u, double *v, double *w,
                         double *p, double *time, double *istep) {
  if (int rc = check_args(io, filename, n, nh)) return rc;
  if (!u || !v || !w || !p || !time || !istep) return io_fail(FLUTAS_EINVAL, "load_ns: null argument");
  double *flds[4] = {u, v, w, p};
  const long long good = (4LL * n[0] * n[1] * n[2] + 2) * 8;
  if (io == 'r') {
    FILE *fp = nullptr;
    if (int rc = open_checked(filename, good, &fp)) return rc;
    int rc = 0;
    for (int i = 0; i < 4 && !rc; i++) rc = read_field(fp, filename, Field{flds[i], n[0], n[1], n[2], nh, on_device(flds[i])});
    double info[2];
    if (!rc && fread(info, sizeof(double), 2, fp) != 2) rc = io_fail(FLUTAS_EINVAL, "load_ns: short read from %s", filename);
    fclose(fp);
    if (rc) return rc;
    *time = info[0];
    *istep = info[1];
    return FLUTAS_OK;
  }
  FILE *fp = fopen(filename, "wb");
  if (!fp) return io_fail(FLUTAS_EINVAL, "load_ns: cannot create %s", filename);
  int rc = 0;
  for (int i = 0; i < 4 && !rc; i++) rc = write_field(fp, filename, Field{flds[i], n[0], n[1], n[2], nh, on_device(flds[i])});
  const double info[2] = {*time, *istep};
  if (!rc && fwrite(info, sizeof(double), 2, fp) != 2) rc = io_fail(FLUTAS_EINVAL, "load_ns: short write to %s", filename);
  if (fclose(fp) != 0 && !rc) rc = io_fail(FLUTAS_EINVAL, "load_ns: cannot write %s", filename);
  return rc;
}

}  // extern "C"
