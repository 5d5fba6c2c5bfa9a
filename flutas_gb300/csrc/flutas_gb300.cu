// flutas_gb300.cu -- host side of the C ABI (include/flutas_gb300.h).
//
// Owns the plan (the GPU counterpart of FluTAS's arrplan + the initsolver
// outputs), stages host-pointer arguments through device mirrors, and issues
// the sm_103a kernels of kernels.cuh.  Reference routines are cited at each
// entry point.
#include "../../include/flutas_gb300.h"
#include "axis_tables.cuh"
#include "kernels.cuh"
#include "fixed.h"
#include "ptrcheck.h"

#include <cuda_runtime.h>

#include <functional>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <map>
#include <mutex>
#include <sstream>
#include <tuple>
#include <type_traits>
#include <string>
#include <vector>

using namespace fg;

namespace {

thread_local std::string g_err;

int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

}  // namespace

// Sets the calling thread's error text (the server hands a worker's message to
// the thread that waits for the request).  Library-internal.
void fg_set_error_text(const char *msg) { g_err = msg ? msg : ""; }

namespace {

#define CK(call)                                                                                  \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess)                                                                        \
      return fail(FLUTAS_ECUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                  __LINE__);                                                                      \
  } while (0)

#define TRY(expr)             \
  do {                        \
    int rc_ = (expr);         \
    if (rc_ != 0) return rc_; \
  } while (0)

bool bc_ok(char c) { return c == 'P' || c == 'N' || c == 'D'; }

int pair_code(char b0, char b1) {
  if (b0 == 'P' && b1 == 'P') return BC_PP;
  if (b0 == 'N' && b1 == 'N') return BC_NN;
  if (b0 == 'D' && b1 == 'D') return BC_DD;
  if (b0 == 'N' && b1 == 'D') return BC_ND;
  if (b0 == 'D' && b1 == 'N') return BC_DN;
  return -1;
}

// ------------------------------------------------------------ device buffers
struct DBuf {
  void *p = nullptr;
  size_t bytes = 0;
  int ensure(size_t b) {
    if (b <= bytes) return 0;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, b);
    if (e != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      return fail(FLUTAS_ENOMEM, "cudaMalloc(%zu) failed: %s", b, cudaGetErrorString(e));
    }
    bytes = b;
    return 0;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <typename T> T *as() const { return (T *)p; }
};

int noalloc_prepare();  // set-up of flutas_gb300_chkdiv_noalloc on the current device

// Page-locked host memory (an asynchronous copy to it does not block the host).
bool is_pinned_host(const void *ptr) {
  if (!ptr) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

// Where an array argument lives (ptrcheck.h): host, device memory usable in
// place on the current device (or managed), or device memory of another GPU.
int ptr_kind(const void *ptr, int *ptr_dev = nullptr) {
  if (!ptr) return PTR_HOST;
  cudaPointerAttributes at;
  const bool ok = cudaPointerGetAttributes(&at, ptr) == cudaSuccess;
  if (!ok) cudaGetLastError();
  int cur = 0;
  if (cudaGetDevice(&cur) != cudaSuccess) cudaGetLastError();
  if (ptr_dev) *ptr_dev = ok ? at.device : -1;
  return classify_ptr(ok, ok ? (int)at.type : 0, ok ? at.device : -1, cur);
}

// Device memory (of any device): readable with cudaMemcpy.
bool is_device_ptr(const void *ptr) { return ptr_kind(ptr) != PTR_HOST; }

int reject_other_device(const char *who, const void *ptr) {
  int dev = -1, cur = -1;
  ptr_kind(ptr, &dev);
  cudaGetDevice(&cur);
  return fail(FLUTAS_EINVAL, "%s: an array lives on device %d, but the current device is %d", who, dev, cur);
}

// A field argument: device pointers are used in place, host pointers are
// copied to a mirror before the kernels and back after (if written).
struct Staged {
  double *d = nullptr;
  const void *host = nullptr;
  size_t bytes = 0;
  bool out = false;
};

struct Mirrors {
  std::vector<DBuf> bufs;
  int used = 0;
  void reset() { used = 0; }
  int get(size_t bytes, void **out) {
    if (used == (int)bufs.size()) bufs.emplace_back();
    TRY(bufs[used].ensure(bytes));
    *out = bufs[used].p;
    used++;
    return 0;
  }
  void release() {
    for (auto &b : bufs) b.release();
    bufs.clear();
    used = 0;
  }
};

int stage_in(Mirrors &m, const void *user, size_t bytes, bool in, bool out, cudaStream_t st, Staged *s,
             bool copy_now = true) {  // copy_now false: the caller copies a host array in itself
  s->host = nullptr;
  s->bytes = bytes;
  s->out = out;
  if (!user) return fail(FLUTAS_EINVAL, "null array argument");
  const int kind = ptr_kind(user);
  if (kind == PTR_OTHER_DEVICE) return reject_other_device("array argument", user);
  if (kind == PTR_DEVICE) {
    s->d = (double *)user;
    return 0;
  }
  void *d = nullptr;
  TRY(m.get(bytes, &d));
  s->d = (double *)d;
  s->host = user;
  if (in && copy_now) CK(cudaMemcpyAsync(d, user, bytes, cudaMemcpyHostToDevice, st));
  return 0;
}

int stage_out(const Staged &s, cudaStream_t st) {
  if (s.host && s.out) CK(cudaMemcpyAsync((void *)s.host, s.d, s.bytes, cudaMemcpyDeviceToHost, st));
  return 0;
}

int num_sms() {
  static std::atomic<int> cache{0};
  int sms = cache.load();
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
    cache.store(sms);
  }
  return sms;
}

int max_smem_optin() {
  static std::atomic<int> cache{0};
  int v = cache.load();
  if (!v) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cache.store(v);
  }
  return v;
}

// The dynamic shared-memory limit of a kernel belongs to the function and is
// shared by every host thread and plan: it is raised once per device, to the
// device maximum, under a lock.  (Setting it to each launch's own size raced:
// a thread launching a large plan could find the limit lowered by another.)
int allow_smem_fn(const void *kernel, bool nonportable_cluster) {
  static std::mutex mu;
  static std::map<std::pair<const void *, int>, bool> done;
  std::lock_guard<std::mutex> lk(mu);
  int dev = 0;
  CK(cudaGetDevice(&dev));
  const auto key = std::make_pair(kernel, dev);
  if (done.count(key)) return 0;
  cudaFuncAttributes fa;
  CK(cudaFuncGetAttributes(&fa, kernel));  // static shared memory counts against the same limit
  CK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          max_smem_optin() - (int)fa.sharedSizeBytes));
  if (nonportable_cluster) CK(cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  done[key] = true;
  return 0;
}
template <typename K> int allow_smem(K kernel, bool nonportable_cluster = false) {
  return allow_smem_fn((const void *)kernel, nonportable_cluster);
}

template <typename K> int grid_for(K kernel, int threads, size_t smem, long work_items) {
  TRY(allow_smem(kernel));
  int per_sm = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem));
  if (per_sm < 1) return fail(FLUTAS_EUNSUPPORTED, "kernel does not fit on an SM (smem %zu)", smem);
  long g = (long)per_sm * num_sms();
  if (work_items < g) g = work_items;
  if (g < 1) g = 1;
  return (int)g;
}

// ------------------------------------------------------------ axis tables
struct AxisTables {
  DBuf W, Q;
  AxisPlan ap{};
  bool ok = false;
};

template <typename T>
int build_axis(int n, int pair, AxisTables *t) {
  AxisPlan ap{};
  std::vector<C2<T>> W, Q;
  if (fill_axis_tables<T>(n, pair, &ap, W, Q) != 0) {
    if (pair > BC_DD && (n % 2))
      return fail(FLUTAS_EUNSUPPORTED, "ND/DN transforms need an even number of cells (n=%d)", n);
    return fail(FLUTAS_EUNSUPPORTED, "transform length %d has a prime factor above 13", n);
  }
  TRY(t->W.ensure(sizeof(C2<T>) * W.size()));
  TRY(t->Q.ensure(sizeof(C2<T>) * Q.size()));
  CK(cudaMemcpy(t->W.p, W.data(), sizeof(C2<T>) * W.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(t->Q.p, Q.data(), sizeof(C2<T>) * Q.size(), cudaMemcpyHostToDevice));
  ap.W = t->W.p;
  ap.Q = t->Q.p;
  t->ap = ap;
  t->ok = true;
  return 0;
}

// Device tables of an extended-FFT axis (FP64: the kinds it serves run on the
// FP64 path only).
struct ExtTables {
  DBuf W, Qa, Qb;
  ExtAxis ea{};
  void release() { W.release(); Qa.release(); Qb.release(); }
};

int build_ext(int n, int kf, int kb, ExtTables *t) {
  ExtAxis ea{};
  std::vector<C2<double>> W, Qa, Qb;
  if (fill_ext_tables<double>(n, kf, kb, &ea, W, Qa, Qb) != 0)
    return fail(FLUTAS_EUNSUPPORTED, "extended transform length %d (n=%d) has a prime factor above 13",
                ext_length(kf, n), n);
  TRY(t->W.ensure(sizeof(C2<double>) * W.size()));
  TRY(t->Qa.ensure(sizeof(C2<double>) * Qa.size()));
  TRY(t->Qb.ensure(sizeof(C2<double>) * Qb.size()));
  CK(cudaMemcpy(t->W.p, W.data(), sizeof(C2<double>) * W.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(t->Qa.p, Qa.data(), sizeof(C2<double>) * Qa.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(t->Qb.p, Qb.data(), sizeof(C2<double>) * Qb.size(), cudaMemcpyHostToDevice));
  ea.W = t->W.p;
  ea.Qa = t->Qa.p;
  ea.Qb = t->Qb.p;
  t->ea = ea;
  return 0;
}

// ------------------------------------------------------ launches + profiling
std::atomic<unsigned long long> g_launches{0};

}  // namespace

// Kernel launches made by the library's other translation units (momentum
// predictor, restart I/O) are counted here too.  Library-internal.
void fg_note_launches(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

namespace {

struct ProfRec {
  const char *name;
  cudaEvent_t a, b;
};
struct Profiler {
  std::mutex mu;
  bool on = false;
  std::vector<ProfRec> recs;
  std::vector<cudaEvent_t> pool;
  cudaEvent_t get() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
  }
} g_prof;

// Every kernel launch of the library goes through here: counts it and, when
// profiling is on, brackets it with CUDA events on its own stream.
template <typename F> int launch(const char *name, cudaStream_t st, F &&f) {
  cudaEvent_t a = nullptr, b = nullptr;
  const bool prof = g_prof.on;
  if (prof) {
    std::lock_guard<std::mutex> lk(g_prof.mu);
    a = g_prof.get();
    b = g_prof.get();
  }
  if (prof) cudaEventRecord(a, st);
  f();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(FLUTAS_ECUDA, "launch of %s failed: %s", name, cudaGetErrorString(e));
  if (prof) {
    cudaEventRecord(b, st);
    std::lock_guard<std::mutex> lk(g_prof.mu);
    g_prof.recs.push_back({name, a, b});
  }
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return 0;
}

}  // namespace

// ===========================================================================
// Plan
// ===========================================================================
struct flutas_plan {
  static constexpr unsigned MAGIC = 0xF1A7A5u;
  unsigned magic = MAGIC;
  int dev = 0;
  int n[3];
  char cbc[6];
  char c_or_f[3];
  double dli[3];
  double bc[6];
  int nh_d;
  double normfft;
  int nn;  // nz - q
  std::vector<double> lam_h, a_h, b_h, c_h, dzci_h, dzfi_h;
  const void *host_lam = nullptr, *host_a = nullptr, *host_b = nullptr, *host_c = nullptr;
  DBuf lam, a, b, c, dzci, dzfi, rhsb[3];
  DBuf a32, b32, c32;  // z coefficients rounded to FP32 (the mixed solve's arithmetic)
  DBuf zres;           // per-level coefficients of the FP64 residual (3 per level)
  DBuf czf;            // folded fillps factors dti*rho0*dzfi(k)
  DBuf czc;            // folded correc factors dt*dzci(k)/rho0
  DBuf zdf;            // per-level factors of the Dodd-Ferrante term
  AxisTables tx64, ty64, tx32, ty32;
  AxisTables txd, tyd;  // double-float tables of the FP64 solver's transforms (dd.cuh)
  DBuf S64, S32, fbuf, phi, phi2, nrm;
  bool face = false;      // a face-centred axis (c_or_f = 'f')
  bool ext[2] = {false, false};  // x / y transform through the extended FFT (fft_ext.cuh)
  bool fp64_only = false; // face-centred or extended kinds: the FP64 solver only
  ExtTables ex[2];
  DBuf nf_flag;         // set by the FP64 z kernel when a column's solution is not finite
  bool nf_armed = false;  // an FP64 solve since the flag was last read
  Mirrors mir;
  cudaStream_t stream = 0;
  cudaStream_t copy_stream = nullptr;  // device -> host copies that overlap the plan stream's kernels
  cudaEvent_t ev_ready = nullptr, ev_copied = nullptr;
  cudaEvent_t ev_u_ready = nullptr, ev_u_copied = nullptr;  // u's early copy to the host
  std::vector<cudaEvent_t> slab_ev;  // host-to-device copy of each z-slab done (copy stream)
  bool sync = true;
  int path64 = 0, path32 = 0;  // 0 separate passes, 1 fused plane kernel, 2 cluster plane kernel
  int clus32 = 0;              // cluster size of path 2 (FP32 transforms)
  bool pin_zero_mode = false;  // singular (lam == 0, z in N/N or P/P) column
  bool rhsb_zero = false;      // every boundary-RHS value is 0 (homogeneous BCs): updt_rhs_b adds nothing
  double last_relres = 0.0;    // relative residual / FP32 solves of the last mixed solve
  int last_iters = 0;
  double contraction = 1e-3;   // residual reduction of one FP32 solve, last measured (initial value:
                               // FLUTAS_GB300_CONTRACTION when set, for tests of the misprediction paths)
};

namespace {

int check_plan(void *p, flutas_plan **out) {
  flutas_plan *pl = (flutas_plan *)p;
  if (!pl || pl->magic != flutas_plan::MAGIC) return fail(FLUTAS_EINVAL, "invalid plan handle");
  *out = pl;
  return 0;
}

template <typename T> size_t plane_smem(int nx, int ny) {
  return align_up<T>(sizeof(T) * (size_t)ny * xpitch(nx)) + sizeof(T) * (size_t)nx * ny;
}

// Cluster plane kernels (FP32 transforms): smallest cluster (2..16 CTAs) whose
// per-CTA share of the plane fits two CTAs per SM (128 registers); 0 when the
// plane does not split evenly.
constexpr int CLUSTER_THREADS = 256;
template <typename T> int cluster_size_for(int nx, int ny, int smax) {
  for (int C = 2; C <= 16; C *= 2) {
    if (nx % C || ny % C || (nx / C) % 2 || (ny / C) % 2) continue;
    const size_t sm = cluster_plane_smem(nx, ny, C, sizeof(T));
    if (sm <= (!std::is_same<T, double>::value ? (size_t)smax / 2 - 1024 : (size_t)smax)) return C;
  }
  return 0;
}

template <typename K> int cluster_prepare(K kernel, size_t smem, int C) {
  (void)smem;
  (void)C;
  return allow_smem(kernel, true);
}

template <typename K, typename... Args>
cudaError_t cluster_launch(K kernel, int clusters, int C, size_t smem, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(clusters * C));
  cfg.blockDim = dim3(CLUSTER_THREADS);
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

// Co-resident clusters of a kernel (0 when a cluster of C cannot be placed).
template <typename K> int cluster_capacity(K kernel, size_t smem, int C) {
  if (cluster_prepare(kernel, smem, C)) return 0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)C);
  cfg.blockDim = dim3(CLUSTER_THREADS);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)C;
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

// Launch name "<base><f32|f64,tag>" per kernel, precision and functor.
enum KId { KID_XYFWD, KID_XFWD, KID_XYINV, KID_XINV, KID_XYFWD_CL, KID_XYINV_CL, KID_XYFWD_FIX, KID_XYINV_FIX };
template <int KID, typename T, typename F> const char *kname() {
  static const char *base[] = {"k_xyfwd_plane", "k_xfwd", "k_xyinv_plane", "k_xinv", "k_xyfwd_cluster",
                               "k_xyinv_cluster", "k_xyfwd_fix", "k_xyinv_fix"};
  const char *tn = std::is_same<T, dd>::value ? "<df64," : (sizeof(T) == 8 ? "<f64," : "<f32,");
  static const std::string s = std::string(base[KID]) + tn + F::tag + ">";
  return s.c_str();
}

// --------------------------------------------------------------------------
// forward (x,y) transform of one field into S, reading through functor In.
// --------------------------------------------------------------------------
template <typename T, typename In>
int fwd_xy(flutas_plan *pl, const In &in, T *S, const AxisTables &tx, const AxisTables &ty, int path,
           double *nrm = nullptr, int nz_planes = 0) {  // nz_planes: the first planes only (a z-slab)
  Geo g{pl->n[0], pl->n[1], nz_planes > 0 ? nz_planes : pl->n[2], 1};
  cudaStream_t st = pl->stream;
  if (path == 1) {
    const size_t sm = plane_smem<T>(g.nx, g.ny);
    int grid = grid_for(k_xyfwd_plane<T, In>, 512, sm, g.nz);
    if (grid < 0) return grid;
    TRY(launch(kname<KID_XYFWD, T, In>(), st, [&] { k_xyfwd_plane<T, In><<<grid, 512, sm, st>>>(tx.ap, ty.ap, in, S, g, nrm); }));
    return 0;
  }
  if constexpr (sizeof(T) == 4) if (path == 2) {  // cluster planes: FP32 only
    const int C = pl->clus32;
    if (fixed_supported(g.nx, g.ny, C, tx.ap.pair, ty.ap.pair)) {
      cudaError_t e = cudaSuccess;
      bool handled = false;
      TRY(launch(kname<KID_XYFWD_FIX, T, In>(), st,
                 [&] { e = xyfwd_fixed(tx.ap, ty.ap, in, S, g, nrm, C, st, &handled); }));
      if (e != cudaSuccess) return fail(FLUTAS_ECUDA, "fixed-size launch failed: %s", cudaGetErrorString(e));
      if (handled) return 0;
    }
    const size_t sm = cluster_plane_smem(g.nx, g.ny, C, sizeof(T));
    TRY(cluster_prepare(k_xyfwd_cluster<T, In>, sm, C));
    cudaError_t e = cudaSuccess;
    TRY(launch(kname<KID_XYFWD_CL, T, In>(), st,
               [&] { e = cluster_launch(k_xyfwd_cluster<T, In>, g.nz, C, sm, st, tx.ap, ty.ap, in, S, g, nrm); }));
    if (e != cudaSuccess) return fail(FLUTAS_ECUDA, "cluster launch failed: %s", cudaGetErrorString(e));
    return 0;
  }
  // x pass
  {
    const int P = xpitch(g.nx);
    int M = (int)((64 * 1024) / (sizeof(T) * (size_t)(P + g.nx)));
    M = (M / 2) * 2;
    if (M < 2) M = 2;
    const size_t sm = align_up<T>(sizeof(T) * (size_t)M * P) + sizeof(T) * (size_t)M * g.nx;
    const long rows = (long)g.ny * g.nz;
    int grid = grid_for(k_xfwd<T, In>, 256, sm, (rows + M - 1) / M);
    if (grid < 0) return grid;
    TRY(launch(kname<KID_XFWD, T, In>(), st, [&] { k_xfwd<T, In><<<grid, 256, sm, st>>>(tx.ap, in, S, g, M, nrm); }));
  }
  // y pass
  {
    int W = (int)((64 * 1024) / (2 * sizeof(T) * (size_t)g.ny));
    W = (W / 2) * 2;
    if (W > g.nx + (g.nx & 1)) W = g.nx + (g.nx & 1);
    if (W < 2) W = 2;
    const size_t sm = align_up<T>(sizeof(T) * (size_t)W * g.ny) + sizeof(T) * (size_t)W * g.ny;
    const long tiles = (long)((g.nx + W - 1) / W) * g.nz;
    int grid = grid_for(k_ypass<T, false>, 256, sm, tiles);
    if (grid < 0) return grid;
    TRY(launch(sizeof(T) == 8 ? "k_ypass_fwd<f64>" : "k_ypass_fwd<f32>", st, [&] { k_ypass<T, false><<<grid, 256, sm, st>>>(ty.ap, S, g, W); }));
  }
  return 0;
}

template <typename T, typename Out>
int inv_xy(flutas_plan *pl, const T *S, const Out &out, const AxisTables &tx, const AxisTables &ty, int path) {
  Geo g{pl->n[0], pl->n[1], pl->n[2], 1};
  cudaStream_t st = pl->stream;
  if (path == 1) {
    const size_t sm = plane_smem<T>(g.nx, g.ny);
    int grid = grid_for(k_xyinv_plane<T, Out>, 512, sm, g.nz);
    if (grid < 0) return grid;
    TRY(launch(kname<KID_XYINV, T, Out>(), st, [&] { k_xyinv_plane<T, Out><<<grid, 512, sm, st>>>(tx.ap, ty.ap, S, out, g); }));
    return 0;
  }
  if constexpr (sizeof(T) == 4) if (path == 2) {  // cluster planes: FP32 only
    const int C = pl->clus32;
    if (fixed_supported(g.nx, g.ny, C, tx.ap.pair, ty.ap.pair)) {
      cudaError_t e = cudaSuccess;
      bool handled = false;
      TRY(launch(kname<KID_XYINV_FIX, T, Out>(), st,
                 [&] { e = xyinv_fixed(tx.ap, ty.ap, S, out, g, C, st, &handled); }));
      if (e != cudaSuccess) return fail(FLUTAS_ECUDA, "fixed-size launch failed: %s", cudaGetErrorString(e));
      if (handled) return 0;
    }
    const size_t sm = cluster_plane_smem(g.nx, g.ny, C, sizeof(T));
    TRY(cluster_prepare(k_xyinv_cluster<T, Out>, sm, C));
    cudaError_t e = cudaSuccess;
    TRY(launch(kname<KID_XYINV_CL, T, Out>(), st,
               [&] { e = cluster_launch(k_xyinv_cluster<T, Out>, g.nz, C, sm, st, tx.ap, ty.ap, S, out, g); }));
    if (e != cudaSuccess) return fail(FLUTAS_ECUDA, "cluster launch failed: %s", cudaGetErrorString(e));
    return 0;
  }
  {
    int W = (int)((64 * 1024) / (2 * sizeof(T) * (size_t)g.ny));
    W = (W / 2) * 2;
    if (W > g.nx + (g.nx & 1)) W = g.nx + (g.nx & 1);
    if (W < 2) W = 2;
    const size_t sm = align_up<T>(sizeof(T) * (size_t)W * g.ny) + sizeof(T) * (size_t)W * g.ny;
    const long tiles = (long)((g.nx + W - 1) / W) * g.nz;
    int grid = grid_for(k_ypass<T, true>, 256, sm, tiles);
    if (grid < 0) return grid;
    TRY(launch(sizeof(T) == 8 ? "k_ypass_inv<f64>" : "k_ypass_inv<f32>", st, [&] { k_ypass<T, true><<<grid, 256, sm, st>>>(ty.ap, (T *)S, g, W); }));
  }
  {
    const int P = xpitch(g.nx);
    int M = (int)((64 * 1024) / (sizeof(T) * (size_t)(P + g.nx)));
    M = (M / 2) * 2;
    if (M < 2) M = 2;
    const size_t sm = align_up<T>(sizeof(T) * (size_t)M * P) + sizeof(T) * (size_t)M * g.nx;
    const long rows = (long)g.ny * g.nz;
    int grid = grid_for(k_xinv<T, Out>, 256, sm, (rows + M - 1) / M);
    if (grid < 0) return grid;
    TRY(launch(kname<KID_XINV, T, Out>(), st, [&] { k_xinv<T, Out><<<grid, 256, sm, st>>>(tx.ap, S, out, g, M); }));
  }
  return 0;
}

// T: the arithmetic of the sweeps; ST: the storage of the spectrum (T itself,
// or double-float pairs for the FP64 solver, swept in FP64).
template <typename T, typename ST = T>
int zsolve(flutas_plan *pl, ST *S, const double *lam, const double *a, const double *b, const double *c, bool pin) {
  ZArgs za;
  za.a = a; za.b = b; za.c = c; za.lam = lam;
  // the FP64 path has no residual norm: its z kernel flags a non-finite solution
  za.nonfinite = nullptr;
  if (sizeof(T) == 8) {
    TRY(pl->nf_flag.ensure(sizeof(int)));
    za.nonfinite = pl->nf_flag.as<int>();
    CK(cudaMemsetAsync(za.nonfinite, 0, sizeof(int), pl->stream));
    pl->nf_armed = true;
  }
  if (sizeof(T) == 8) { za.at = a; za.bt = b; za.ct = c; }
  else { za.at = pl->a32.p; za.bt = pl->b32.p; za.ct = pl->c32.p; }
  za.nq = pl->n[0] * pl->n[1];
  za.nz = pl->n[2];
  za.nn = pl->nn;
  za.periodic = (pl->cbc[4] == 'P' && pl->cbc[5] == 'P') ? 1 : 0;
  // only a singular z operator (N/N or P/P) has a null space to pin
  const bool zsing = (pl->cbc[4] == 'N' && pl->cbc[5] == 'N') || (pl->cbc[4] == 'P' && pl->cbc[5] == 'P');
  za.pin = (pin && zsing) ? 1 : 0;
  if (!za.periodic) {
    constexpr int CH = 16;
    const int nt = 128;
    const size_t sm = zstream_smem<T, CH>(za.nn, nt);
    if ((int)sm > max_smem_optin()) return fail(FLUTAS_EUNSUPPORTED, "nz=%d too large for the z kernel", za.nz);
    TRY(allow_smem(k_zstream<T, CH, ST>));
    // launch in column batches whose eliminated values (one column of T per
    // column) stay L2-resident between the two sweeps
    const long per_batch = std::max<long>(nt, (long)(80.0e6 / (sizeof(T) * (double)za.nn)) / nt * nt);
    for (long q0 = 0; q0 < za.nq; q0 += per_batch) {
      const long q1 = std::min<long>(za.nq, q0 + per_batch);
      const int grid = (int)((q1 - q0 + nt - 1) / nt);
      TRY(launch(sizeof(T) == 8 ? "k_zstream<f64>" : "k_zstream<f32>", pl->stream,
                 [&] { k_zstream<T, CH, ST><<<grid, nt, sm, pl->stream>>>(za, S, q0, q1); }));
    }
    return 0;
  }
  int TC = sizeof(T) == 8 ? 32 : 64;
  const size_t sm = sizeof(T) * (size_t)3 * za.nz * TC;
  if ((int)sm > max_smem_optin()) TC = 32;
  const size_t sm2 = sizeof(T) * (size_t)3 * za.nz * TC;
  if ((int)sm2 > max_smem_optin()) return fail(FLUTAS_EUNSUPPORTED, "nz=%d too large for the z kernel", za.nz);
  int grid = grid_for(k_zsolve<T, ST>, TC, sm2, ((long)za.nq + TC - 1) / TC);
  if (grid < 0) return grid;
  TRY(launch(sizeof(T) == 8 ? "k_zsolve<f64>" : "k_zsolve<f32>", pl->stream,
             [&] { k_zsolve<T, ST><<<grid, TC, sm2, pl->stream>>>(za, S); }));
  return 0;
}

// In-functors with side effects / norms for the mixed path ------------------
}  // namespace

namespace {

int stream_grid(long n, int threads = 256) {
  long g = (n + threads - 1) / threads;
  long cap = (long)num_sms() * 8;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

int scale_jobs(const ScaleJobs &j, cudaStream_t st) {
  if (j.count == 0) return 0;
  return launch("k_scale_vecs", st, [&] { k_scale_vecs<<<j.count, 256, 0, st>>>(j); });
}
int scale_vecs(const double *in, double s, double *out, int n, cudaStream_t st) {
  ScaleJobs j;
  j.add(in, s, out, n);
  return scale_jobs(j, st);
}

int finish(flutas_plan *pl) {
  if (pl->sync) CK(cudaStreamSynchronize(pl->stream));
  return 0;
}

// After a synchronised FP64 solve: FLUTAS_ENONFINITE when its solution holds a
// NaN or Inf (a non-finite right-hand side; the reference would carry it into
// the fields without a word).  In asynchronous mode nothing is read back.
int check_nonfinite(flutas_plan *pl, const char *who) {
  if (!pl->sync || !pl->nf_armed) return 0;
  pl->nf_armed = false;
  int h = 0;
  CK(cudaMemcpy(&h, pl->nf_flag.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (h) return fail(FLUTAS_ENONFINITE, "%s: the solution is not finite (NaN or Inf in the right-hand side)", who);
  return 0;
}

// x/y transforms of a plan with an extended-FFT axis, in place on the FP64
// spectral array S: per axis k_r2r_ext, or the paired/DCT-IV engine's separate
// pass (k_xfwd / k_ypass / k_xinv reading and writing S itself).
int ext_pass(flutas_plan *pl, double *S, int axis, bool backward) {
  const Geo g{pl->n[0], pl->n[1], pl->n[2], 1};
  cudaStream_t st = pl->stream;
  const ExtAxis &ea = pl->ex[axis].ea;
  const int kind = backward ? ea.kb : ea.kf;
  const size_t per_line = 2 * sizeof(C2<double>) * (size_t)ea.L + sizeof(double) * (size_t)ea.n;
  int B = (int)std::min<size_t>(16, (size_t)(144 * 1024) / per_line);
  if (B < 1) B = 1;
  const size_t sm = per_line * B;
  if ((int)sm > max_smem_optin()) return fail(FLUTAS_EUNSUPPORTED, "extended transform of n=%d too long", ea.n);
  TRY(allow_smem(k_r2r_ext<double>));
  const long lines = axis == 0 ? (long)g.ny * g.nz : (long)g.nx * g.nz;
  const int grid = grid_for(k_r2r_ext<double>, 256, sm, (lines + B - 1) / B);
  if (grid < 0) return grid;
  return launch(axis == 0 ? "k_r2r_ext<f64,x>" : "k_r2r_ext<f64,y>", st,
                [&] { k_r2r_ext<double><<<grid, 256, sm, st>>>(ea, kind, S, g, axis, B); });
}

int xy_ext(flutas_plan *pl, double *S, bool backward) {
  const Geo g{pl->n[0], pl->n[1], pl->n[2], 1};
  cudaStream_t st = pl->stream;
  const int P = xpitch(g.nx);
  int M = (int)((64 * 1024) / (sizeof(double) * (size_t)(P + g.nx)));
  M = std::max(2, (M / 2) * 2);
  const size_t smx = align_up<double>(sizeof(double) * (size_t)M * P) + sizeof(double) * (size_t)M * g.nx;
  const long rows = (long)g.ny * g.nz;
  int W = (int)((64 * 1024) / (2 * sizeof(double) * (size_t)g.ny));
  W = (W / 2) * 2;
  if (W > g.nx + (g.nx & 1)) W = g.nx + (g.nx & 1);
  if (W < 2) W = 2;
  const size_t smy = align_up<double>(sizeof(double) * (size_t)W * g.ny) + sizeof(double) * (size_t)W * g.ny;
  const long tiles = (long)((g.nx + W - 1) / W) * g.nz;
  auto xpass = [&]() -> int {
    if (pl->ext[0]) return ext_pass(pl, S, 0, backward);
    if (!backward) {
      const int grid = grid_for(k_xfwd<double, InPlain>, 256, smx, (rows + M - 1) / M);
      if (grid < 0) return grid;
      return launch("k_xfwd<f64,plain>", st,
                    [&] { k_xfwd<double, InPlain><<<grid, 256, smx, st>>>(pl->tx64.ap, InPlain{S, g}, S, g, M, nullptr); });
    }
    const int grid = grid_for(k_xinv<double, OutPlain>, 256, smx, (rows + M - 1) / M);
    if (grid < 0) return grid;
    return launch("k_xinv<f64,plain>", st,
                  [&] { k_xinv<double, OutPlain><<<grid, 256, smx, st>>>(pl->tx64.ap, S, OutPlain{S, g}, g, M); });
  };
  auto ypass = [&]() -> int {
    if (pl->ext[1]) return ext_pass(pl, S, 1, backward);
    if (!backward) {
      const int grid = grid_for(k_ypass<double, false>, 256, smy, tiles);
      if (grid < 0) return grid;
      return launch("k_ypass_fwd<f64>", st, [&] { k_ypass<double, false><<<grid, 256, smy, st>>>(pl->ty64.ap, S, g, W); });
    }
    const int grid = grid_for(k_ypass<double, true>, 256, smy, tiles);
    if (grid < 0) return grid;
    return launch("k_ypass_inv<f64>", st, [&] { k_ypass<double, true><<<grid, 256, smy, st>>>(pl->ty64.ap, S, g, W); });
  };
  if (!backward) {
    TRY(xpass());
    return ypass();
  }
  TRY(ypass());
  return xpass();
}

// The FP64 solve of a plan with an extended-FFT axis: p's interior into S,
// forward x and y in place, z, inverse y and x in place, S * normfft into p.
int solve_fp64_ext_spec(flutas_plan *pl, double *S, double *out_halo, const double *lam, const double *a,
                        const double *b, const double *c) {
  const Geo g{pl->n[0], pl->n[1], pl->n[2], 1};
  cudaStream_t st = pl->stream;
  TRY(xy_ext(pl, S, false));
  TRY(zsolve<double>(pl, S, lam, a, b, c, pl->pin_zero_mode));
  TRY(xy_ext(pl, S, true));
  const long cells = (long)g.nx * g.ny * g.nz;
  const int grid = (int)std::min<long>((cells + 255) / 256, (long)num_sms() * 8);
  return launch("k_spec_out", st, [&] { k_spec_out<double><<<grid, 256, 0, st>>>(S, OutHalo{out_halo, pl->normfft, g}, g); });
}

// FP64 solve on a device halo array (the plan's own stream).
int solve_fp64_dev(flutas_plan *pl, double *p, const double *lam, const double *a, const double *b, const double *c) {
  Geo g{pl->n[0], pl->n[1], pl->n[2], 1};
  if (pl->ext[0] || pl->ext[1]) {
    TRY(pl->S64.ensure(sizeof(double) * (size_t)g.nx * g.ny * g.nz));
    double *S = pl->S64.as<double>();
    const long cells = (long)g.nx * g.ny * g.nz;
    const int grid = grid_for(k_stencil_pass<InHalo, double>, 256, 0, (cells + 1023) / 1024);
    if (grid < 0) return grid;
    if (cells >= (1L << 31) - 4096)
      TRY(launch("k_stencil<f64,halo>", pl->stream, [&] {
        k_stencil_pass<InHalo, double, long long><<<grid, 256, 0, pl->stream>>>(InHalo{p, g}, g, nullptr, S, nullptr);
      }));
    else
      TRY(launch("k_stencil<f64,halo>", pl->stream, [&] {
        k_stencil_pass<InHalo, double><<<grid, 256, 0, pl->stream>>>(InHalo{p, g}, g, nullptr, S, nullptr);
      }));
    return solve_fp64_ext_spec(pl, S, p, lam, a, b, c);
  }
  TRY(pl->S64.ensure(sizeof(double) * (size_t)g.nx * g.ny * g.nz));
  // transforms in double-float (dd.cuh), z sweeps in FP64 on the same 8-byte spectrum
  dd *S = pl->S64.as<dd>();
  TRY(fwd_xy<dd>(pl, InHalo{p, g}, S, pl->txd, pl->tyd, pl->path64));
  TRY((zsolve<double, dd>(pl, S, lam, a, b, c, pl->pin_zero_mode)));
  TRY(inv_xy<dd>(pl, S, OutHalo{p, pl->normfft, g}, pl->txd, pl->tyd, pl->path64));
  return 0;
}

// Mixed solve.  The first pass evaluates the RHS through `first` (the halo
// array x itself, or fillps of u,v,w), keeps an FP64 copy of it in fbuf and
// accumulates ||f||^2; every later pass evaluates the FP64 residual
// r = f - A x, accumulates ||r||^2 and transforms it.  x (halo 1) receives
// the solution.  The norm of the residual decides on the host whether the
// FP32 correction of that pass is applied.  When the last measured reduction
// per FP32 solve predicts that a check will end the solve (or the iteration
// limit does), the check evaluates the residual norm alone (k_resnorm) and
// the transform of the residual is made only if the prediction was wrong.
// With the fixed-size cluster kernels, the FP64 RHS (fillps, residual) is
// evaluated by a stencil pass at full occupancy and the transform reads its
// FP32 values in place; the other paths evaluate it in the transform's loads.
// The correction a mixed projection applies after its solve (correc with
// phi = x, p = p + x), fused into the solve's last convergence check when the
// measured contraction predicts it (k_resnorm_correc).  If that check does not
// end the solve after all, the solve keeps a copy of the x it applied and the
// caller adds the correction of the difference (correc and the p update are
// linear in phi).
struct FinalCorrec {
  CorrecAddArgs ca;
  std::function<int()> boundp_phi;  // ghosts of phi, read by the correction
  // set: u's correction runs first (k_correc_u), then this (its ghost cells and
  // its copy to the host on the copy stream), then the check with the rest
  std::function<int()> u_first;
  // set: the ghost cells of the corrected fields, queued right behind the
  // fused check (before the host reads its norm); redone if the solve goes on
  std::function<int()> ghosts_after;
  double *snapshot = nullptr;       // x as applied, when the solve went on
  bool applied = false, continued = false, u_early = false, ghosts_queued = false;
};

template <typename First>
int solve_mixed_dev(flutas_plan *pl, const First &first, double *x, double tol, int max_iter, double *relres,
                    int *iters, FinalCorrec *fc = nullptr, bool first_done = false) {
  // first_done: the first pass (RHS kept in fbuf, FP32 RHS transformed in S32,
  // ||f||^2 in nrm[0], the other norms zeroed) was run by the caller (slab_first_pass)
  Geo g{pl->n[0], pl->n[1], pl->n[2], 1};
  const size_t halo_bytes = sizeof(double) * (size_t)(g.nx + 2) * (g.ny + 2) * (g.nz + 2);
  TRY(pl->S32.ensure(sizeof(float) * (size_t)g.nx * g.ny * g.nz));
  TRY(pl->fbuf.ensure(halo_bytes));
  if (max_iter < 1) max_iter = 1;
  TRY(pl->nrm.ensure(sizeof(double) * (max_iter + 2)));  // [0]: |f|^2, [it]: |r|^2 after solve it
  float *S = pl->S32.as<float>();
  double *f = pl->fbuf.as<double>();
  double *nrm = pl->nrm.as<double>();
  cudaStream_t st = pl->stream;
  const double *lam = pl->lam.as<double>(), *a = pl->a.as<double>(), *b = pl->b.as<double>(), *c = pl->c.as<double>();
  const bool split =
      pl->path32 == 2 && fixed_supported(g.nx, g.ny, pl->clus32, pl->tx32.ap.pair, pl->ty32.ap.pair);
  auto stencil = [&](const auto &in, double *keep, float *s32, double *acc) -> int {
    using In = std::decay_t<decltype(in)>;
    const long cells = (long)g.nx * g.ny * g.nz;
    const int grid = grid_for(k_stencil_pass<In, float>, 256, 0, (cells + 1023) / 1024);
    if (grid < 0) return grid;
    static const std::string name = std::string("k_stencil<") + In::tag + ">";
    const char *nm = (keep || s32) ? name.c_str() : "k_resnorm";
    if (cells >= (1L << 31) - 4096)  // the int variant also forms indices up to 3 blocks past the end
      return launch(nm, st, [&] { k_stencil_pass<In, float, long long><<<grid, 256, 0, st>>>(in, g, keep, s32, acc); });
    return launch(nm, st, [&] { k_stencil_pass<In, float><<<grid, 256, 0, st>>>(in, g, keep, s32, acc); });
  };
  auto transform = [&](const InResidual &R, double *acc) -> int {  // residual -> S
    if (!split) return fwd_xy<float>(pl, R, S, pl->tx32, pl->ty32, pl->path32, acc);
    TRY(stencil(R, nullptr, S, acc));
    return fwd_xy<float>(pl, InF32{S, g}, S, pl->tx32, pl->ty32, pl->path32);
  };
  if (first_done) {
    if (!split) return fail(FLUTAS_ECUDA, "internal: a slab first pass needs the split form");
  } else if (split) {
    CK(cudaMemsetAsync(nrm, 0, sizeof(double) * (max_iter + 2), st));
    TRY(stencil(first, f, S, nrm + 0));
    TRY(fwd_xy<float>(pl, InF32{S, g}, S, pl->tx32, pl->ty32, pl->path32));
  } else {
    CK(cudaMemsetAsync(nrm, 0, sizeof(double) * (max_iter + 2), st));
    TRY(fwd_xy<float>(pl, InKeep<First>{first, f, g}, S, pl->tx32, pl->ty32, pl->path32, nrm + 0));
  }
  TRY(zsolve<float>(pl, S, lam, a, b, c, true));
  TRY(inv_xy<float>(pl, S, OutHalo{x, pl->normfft, g}, pl->tx32, pl->ty32, pl->path32));
  InResidual R;
  R.f = f; R.x = x;
  R.zc = pl->zres.as<double>();
  R.dxi2 = pl->dli[0] * pl->dli[0];
  R.dyi2 = pl->dli[1] * pl->dli[1];
  memcpy(R.bc, pl->cbc, 6);
  R.g = g;
  int it = 1;
  double rel = 0.0, before = 1.0;  // relative residual before the latest FP32 solve
  bool measured = true;            // before was read back (not predicted)
  std::vector<double> h(max_iter + 2);
  for (;;) {
    const double predicted = before * pl->contraction;
    const bool norm_only = it >= max_iter || predicted <= 0.5 * tol;
    double *acc = nrm + it;
    if (norm_only && fc && !fc->applied) {
      TRY(fc->boundp_phi());
      const long cells = (long)g.nx * g.ny * g.nz;
      const int grid = grid_for(k_resnorm_correc<int>, 256, 0, (cells + 511) / 512);
      if (grid < 0) return grid;
      CorrecAddArgs ca = fc->ca;
      if (fc->u_first) {
        TRY(launch("k_correc_u", st, [&] { k_correc_u<<<grid_cells(ca.g), 256, 0, st>>>(ca); }));
        TRY(fc->u_first());
        fc->u_early = true;
        ca.u = nullptr;
      }
      if (cells >= (1L << 31) - 4096)
        TRY(launch("k_resnorm_correc", st, [&] { k_resnorm_correc<long long><<<grid, 256, 0, st>>>(R, ca, acc); }));
      else
        TRY(launch("k_resnorm_correc", st, [&] { k_resnorm_correc<int><<<grid, 256, 0, st>>>(R, ca, acc); }));
      fc->applied = true;
      if (fc->ghosts_after) {
        TRY(fc->ghosts_after());
        fc->ghosts_queued = true;
      }
    } else if (norm_only) {
      TRY(stencil(R, nullptr, nullptr, acc));
    } else {
      TRY(transform(R, acc));
    }
    if (!norm_only && measured && predicted > 1e3 * tol) {
      // the residual is predicted three orders of magnitude above tol: the next
      // solve is queued behind this check without a wait, and its norm is read
      // with the next check, which waits (were it converged after all, one more
      // solve changes nothing)
      before = predicted;
      measured = false;
    } else {
      CK(cudaMemcpyAsync(h.data(), nrm, sizeof(double) * (it + 1), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      for (int j = 0; j <= it; j++)
        if (!std::isfinite(h[j])) return fail(FLUTAS_ENONFINITE, "non-finite residual in mixed solve");
      auto relof = [&](int j) { return h[0] > 0 ? std::sqrt(h[j] / h[0]) : std::sqrt(h[j]); };
      rel = relof(it);
      const double prev = it > 1 ? relof(it - 1) : 1.0;
      if (prev > 0.0) pl->contraction = std::min(1.0, std::max(rel / prev, 1e-12));
      if (rel <= tol || it >= max_iter) break;
      before = rel;
      measured = true;
    }
    if (fc && fc->applied && !fc->continued) {  // the fused check did not end the solve: keep the applied x
      fc->continued = true;
      TRY(pl->phi2.ensure(halo_bytes));
      fc->snapshot = pl->phi2.as<double>();
      CK(cudaMemcpyAsync(fc->snapshot, x, halo_bytes, cudaMemcpyDeviceToDevice, st));
    }
    if (norm_only) TRY(transform(R, nullptr));  // prediction missed
    // correction of this pass: e = A^-1 r in FP32, x += e in FP64
    TRY(zsolve<float>(pl, S, lam, a, b, c, true));
    TRY(inv_xy<float>(pl, S, OutHaloAdd{x, pl->normfft, g}, pl->tx32, pl->ty32, pl->path32));
    it++;
  }
  if (relres) *relres = rel;
  if (iters) *iters = it;
  if (rel > tol) return fail(FLUTAS_EITER, "mixed solve reached %d solves at relative residual %.3e > %.3e", it, rel, tol);
  return 0;
}

}  // namespace

// FP32 plane transforms: the whole-plane form (one CTA, or a cluster) against
// separate x and y passes, the forward and inverse transforms of the grid's
// planes timed once per process and grid signature on scratch data (the faster wins; the
// plane forms lose on some sizes, e.g. 160^2 planes with radix-5 stages).  The choice is cached, so every plan
// of one signature in a process runs the same kernels.
std::mutex g_path_mu;
std::map<std::tuple<int, int, int, int, int, int>, int> g_path32;

int choose_path32(flutas_plan *pl) {
  const int nx = pl->n[0], ny = pl->n[1];
  const auto key = std::make_tuple(nx, ny, pl->n[2], pl->tx32.ap.pair, pl->ty32.ap.pair, pl->path32);
  {
    std::lock_guard<std::mutex> lk(g_path_mu);
    auto it = g_path32.find(key);
    if (it != g_path32.end()) {
      pl->path32 = it->second;
      return 0;
    }
  }
  const int planes = pl->n[2];  // every plane: the whole-plane forms run one CTA (or cluster) a plane
  DBuf scratch, xout;
  TRY(scratch.ensure(sizeof(float) * (size_t)nx * ny * planes));
  const size_t xbytes = sizeof(double) * (size_t)(nx + 2) * (ny + 2) * (planes + 2);
  TRY(xout.ensure(xbytes));
  float *S = scratch.as<float>();
  CK(cudaMemsetAsync(S, 0, sizeof(float) * (size_t)nx * ny * planes, pl->stream));
  CK(cudaMemsetAsync(xout.p, 0, xbytes, pl->stream));
  const Geo g{nx, ny, planes, 1};
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  float best[2] = {1e30f, 1e30f};
  const int cand[2] = {pl->path32, 0};
  int rc = 0;
  for (int rep = 0; rep < 4 && !rc; rep++)
    for (int c = 0; c < 2 && !rc; c++) {
      cudaEventRecord(a, pl->stream);
      rc = fwd_xy<float>(pl, InF32{S, g}, S, pl->tx32, pl->ty32, cand[c], nullptr, planes);
      if (!rc) rc = inv_xy<float>(pl, S, OutHalo{xout.as<double>(), 1.0, g}, pl->tx32, pl->ty32, cand[c]);
      cudaEventRecord(b, pl->stream);
      if (cudaEventSynchronize(b) != cudaSuccess) rc = fail(FLUTAS_ECUDA, "initsolver: transform timing failed");
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, a, b);
      if (rep > 0) best[c] = std::min(best[c], ms);  // the first round warms up
    }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  scratch.release();
  xout.release();
  if (rc) return rc;
  const int chosen = best[1] < best[0] ? 0 : cand[0];
  std::lock_guard<std::mutex> lk(g_path_mu);
  g_path32[key] = chosen;
  pl->path32 = chosen;
  return 0;
}

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int flutas_gb300_last_error(char *buf, int len) {
  if (!buf || len <= 0) return FLUTAS_EINVAL;
  snprintf(buf, (size_t)len, "%s", g_err.c_str());
  return FLUTAS_OK;
}

int flutas_gb300_initsolver(const int n[3], const double dli[3], int nh_d, const double *dzci,
                            const double *dzfi, const char cbc[6], const double bc[6],
                            const char c_or_f[3], double *lambdaxy, double *a, double *b, double *c,
                            void **arrplan, double *normfft, double *rhsbx, double *rhsby,
                            double *rhsbz) {
  // src/initsolver.f90:21-120
  if (!n || !dli || !dzci || !dzfi || !cbc || !bc || !c_or_f || !lambdaxy || !a || !b || !c || !arrplan ||
      !normfft || !rhsbx || !rhsby || !rhsbz)
    return fail(FLUTAS_EINVAL, "initsolver: null argument");
  const int nx = n[0], ny = n[1], nz = n[2];
  if (nx < 2 || ny < 2 || nz < 3 || nh_d < 1) return fail(FLUTAS_EINVAL, "initsolver: bad sizes n=(%d,%d,%d) nh_d=%d", nx, ny, nz, nh_d);
  for (int i = 0; i < 6; i++)
    if (!bc_ok(cbc[i])) return fail(FLUTAS_EINVAL, "initsolver: bad BC character '%c'", cbc[i]);
  for (int d = 0; d < 3; d++) {
    if ((cbc[2 * d] == 'P') != (cbc[2 * d + 1] == 'P'))
      return fail(FLUTAS_EINVAL, "initsolver: periodic BC must be set on both ends (axis %d)", d + 1);
  }
  for (int d = 0; d < 3; d++)
    if (c_or_f[d] != 'c' && c_or_f[d] != 'f')
      return fail(FLUTAS_EINVAL, "initsolver: c_or_f(%d) must be 'c' or 'f'", d + 1);
  const int bx = pair_code(cbc[0], cbc[1]), by = pair_code(cbc[2], cbc[3]);
  if (bx < 0 || by < 0 || pair_code(cbc[4], cbc[5]) < 0) return fail(FLUTAS_EINVAL, "initsolver: bad BC pair");
  // the transform of each x/y axis (find_fft, src/fft.f90:233-291): a kind of the paired /
  // DCT-IV engine (pair code), or an extended-FFT kind (fft_ext.cuh) for the face-centred
  // REDFT00, RODFT00, RODFT01/10 and the odd-length REDFT11 / RODFT11
  struct AxisKind {
    int pair, kf, kb;
  };
  auto axis_kind = [](int bcpair, char cf, int nn) -> AxisKind {
    if (cf == 'c') {
      if (bcpair == BC_ND && nn % 2) return {bcpair, EXT_DCT4, EXT_DCT4};
      if (bcpair == BC_DN && nn % 2) return {bcpair, EXT_DST4, EXT_DST4};
      return {bcpair, EXT_NONE, EXT_NONE};
    }
    switch (bcpair) {
      case BC_PP: return {BC_PP, EXT_NONE, EXT_NONE};           // R2HC / HC2R
      case BC_NN: return {BC_NN, EXT_DCT1, EXT_DCT1};           // REDFT00 / REDFT00
      case BC_DD: return {BC_DD, EXT_DST1, EXT_DST1};           // RODFT00 / RODFT00 on n-1 points
      case BC_ND: return {BC_NN, EXT_NONE, EXT_NONE};           // REDFT10 / REDFT01
      default: return {BC_DD, EXT_DST3, EXT_DST2};              // DN: RODFT01 / RODFT10
    }
  };
  const AxisKind kx = axis_kind(bx, c_or_f[0], nx), ky = axis_kind(by, c_or_f[1], ny);
  const int px = kx.pair, py = ky.pair;
  flutas_plan *pl = new flutas_plan();
  int rc = 0;
  auto bail = [&](int r) { pl->magic = 0; delete pl; return r; };
  cudaGetDevice(&pl->dev);
  memcpy(pl->n, n, sizeof(int) * 3);
  memcpy(pl->cbc, cbc, 6);
  memcpy(pl->c_or_f, c_or_f, 3);
  memcpy(pl->dli, dli, sizeof(double) * 3);
  memcpy(pl->bc, bc, sizeof(double) * 6);
  pl->nh_d = nh_d;
  pl->face = c_or_f[0] == 'f' || c_or_f[1] == 'f' || c_or_f[2] == 'f';
  pl->ext[0] = kx.kf != EXT_NONE;
  pl->ext[1] = ky.kf != EXT_NONE;
  pl->fp64_only = pl->face || pl->ext[0] || pl->ext[1];
  // eigenvalues (initsolver.f90:122-186), CPU natural order, times dli^2 (61-64).  The
  // face-centred NN pair keeps the cell-centred formula (the reference writes 2(n-1+1));
  // the face-centred DD pair transforms n-1 points and leaves lambda(n) unset (its point is
  // a boundary, not transformed): 0 here, as in the oracle.
  const double pi = 3.141592653589793238462643383279502884;
  auto eig = [&](int nn, int bcpair, char cf, double *lam) {
    for (int l = 1; l <= nn; l++) {
      double s;
      switch (bcpair) {
        case BC_PP: s = std::sin((1.0 * (l - 1)) * pi / (1.0 * nn)); break;
        case BC_NN: s = std::sin((1.0 * (l - 1)) * pi / (2.0 * nn)); break;
        case BC_DD: s = std::sin((1.0 * (l - 0)) * pi / (2.0 * nn)); break;
        default: s = std::sin((1.0 * (2 * l - 1)) * pi / (4.0 * nn)); break;
      }
      lam[l - 1] = (bcpair == BC_DD && cf == 'f' && l == nn) ? 0.0 : -4.0 * s * s;
    }
  };
  std::vector<double> lx(nx), ly(ny);
  eig(nx, bx, c_or_f[0], lx.data());
  eig(ny, by, c_or_f[1], ly.data());
  for (int i = 0; i < nx; i++) lx[i] = lx[i] * (dli[0] * dli[0]);
  for (int j = 0; j < ny; j++) ly[j] = ly[j] * (dli[1] * dli[1]);
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) lambdaxy[i + (long)nx * j] = lx[i] + ly[j];
  // tridmatrix (initsolver.f90:188-246), cell- or face-centred in z
  auto DZCI = [&](int k) { return dzci[k - 1 + nh_d]; };
  auto DZFI = [&](int k) { return dzfi[k - 1 + nh_d]; };
  const bool zface = c_or_f[2] == 'f';
  for (int k = 1; k <= nz; k++) {
    a[k - 1] = zface ? DZFI(k) * DZCI(k) : DZFI(k) * DZCI(k - 1);
    c[k - 1] = zface ? DZFI(k + 1) * DZCI(k) : DZFI(k) * DZCI(k);
  }
  for (int k = 0; k < nz; k++) b[k] = -(a[k] + c[k]);
  auto fac = [](char ch) { return ch == 'D' ? -1.0 : (ch == 'N' ? 1.0 : 0.0); };
  if (!zface) {
    b[0] = b[0] + fac(cbc[4]) * a[0];
    b[nz - 1] = b[nz - 1] + fac(cbc[5]) * c[nz - 1];
  } else {
    if (cbc[4] == 'N') b[0] = b[0] + fac(cbc[4]) * a[0];
    if (cbc[5] == 'N') b[nz - 1] = b[nz - 1] + fac(cbc[5]) * c[nz - 1];
  }
  // bc_rhs (initsolver.f90:248-298)
  auto bc_rhs = [&](const char *cb, int n1, int n2, const double *bv, const double dlc[2], const double dlf[2],
                    char cf, double *rhs) {
    double factor[2];
    for (int ib = 0; ib < 2; ib++) {
      double sgn = ib == 0 ? 1.0 : -1.0;
      if (cb[ib] == 'P') factor[ib] = 0.0;
      else if (cb[ib] == 'D') factor[ib] = cf == 'c' ? -2.0 * bv[ib] : -bv[ib];
      else factor[ib] = sgn * (cf == 'c' ? dlc[ib] : dlf[ib]) * bv[ib];
    }
    for (int ib = 0; ib < 2; ib++) {
      double v = factor[ib] / dlc[ib] / dlf[ib];
      for (long t = 0; t < (long)n1 * n2; t++) rhs[(long)ib * n1 * n2 + t] = v;
    }
  };
  {
    double dl0[2] = {1.0 / dli[0], 1.0 / dli[0]}, dl1[2] = {1.0 / dli[1], 1.0 / dli[1]};
    double dlc[2] = {1.0 / DZCI(zface ? 1 : 0), 1.0 / DZCI(zface ? nz - 1 : nz)};
    double dlf[2] = {1.0 / DZFI(1), 1.0 / DZFI(nz)};
    bc_rhs(cbc + 0, ny, nz, bc + 0, dl0, dl0, c_or_f[0], rhsbx);
    bc_rhs(cbc + 2, nx, nz, bc + 2, dl1, dl1, c_or_f[1], rhsby);
    bc_rhs(cbc + 4, nx, ny, bc + 4, dlc, dlf, c_or_f[2], rhsbz);
  }
  // fftini normalisation (fft.f90:71-150): norm(1)*(n + norm(2) - ix), the face-centred NN
  // pair 2(n-1), the face-centred DD pair 2(n+1-1)
  auto normf = [](int bcpair, char cf, int nn) {
    if (bcpair == BC_PP) return 1.0 * nn;
    if (cf == 'f' && bcpair == BC_NN) return 2.0 * (nn - 1);
    return 2.0 * nn;
  };
  pl->normfft = 1.0 / (normf(bx, c_or_f[0], nx) * normf(by, c_or_f[1], ny));
  *normfft = pl->normfft;
  pl->nn = nz - ((zface && cbc[5] == 'D') ? 1 : 0);  // solver_cpu.f90:71-72
  pl->pin_zero_mode = false;  // FP64 path follows dgtsv_homebrewed's z == 0 test
  // host copies + device copies
  pl->lam_h.assign(lambdaxy, lambdaxy + (long)nx * ny);
  pl->a_h.assign(a, a + nz);
  pl->b_h.assign(b, b + nz);
  pl->c_h.assign(c, c + nz);
  pl->dzci_h.assign(dzci, dzci + nz + 2 * nh_d);
  pl->dzfi_h.assign(dzfi, dzfi + nz + 2 * nh_d);
  pl->host_lam = lambdaxy; pl->host_a = a; pl->host_b = b; pl->host_c = c;
  auto up = [&](DBuf &d, const double *h, size_t cnt) -> int {
    TRY(d.ensure(sizeof(double) * cnt));
    CK(cudaMemcpy(d.p, h, sizeof(double) * cnt, cudaMemcpyHostToDevice));
    return 0;
  };
  if ((rc = up(pl->lam, lambdaxy, (size_t)nx * ny))) return bail(rc);
  if ((rc = up(pl->a, a, nz)) || (rc = up(pl->b, b, nz)) || (rc = up(pl->c, c, nz))) return bail(rc);
  {
    // the FP64 coefficients rounded once to FP32 for the bulk solve
    std::vector<float> f32(nz);
    DBuf *dst[3] = {&pl->a32, &pl->b32, &pl->c32};
    const double *src[3] = {a, b, c};
    for (int t = 0; t < 3; t++) {
      for (int k = 0; k < nz; k++) f32[k] = (float)src[t][k];
      if ((rc = dst[t]->ensure(sizeof(float) * nz))) return bail(rc);
      if (cudaMemcpy(dst[t]->p, f32.data(), sizeof(float) * nz, cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(fail(FLUTAS_ECUDA, "initsolver: upload of FP32 coefficients failed"));
    }
  }
  if ((rc = up(pl->dzci, dzci, nz + 2 * nh_d)) || (rc = up(pl->dzfi, dzfi, nz + 2 * nh_d))) return bail(rc);
  {
    // residual coefficients of level k (1-based): czm = dzfi(k)dzci(k-1),
    // czp = dzfi(k)dzci(k), cc = -2 dxi^2 - 2 dyi^2 - czm - czp
    std::vector<double> zr(3 * (size_t)nz);
    const double dxi2 = dli[0] * dli[0], dyi2 = dli[1] * dli[1];
    for (int k = 1; k <= nz; k++) {
      const double czm = DZFI(k) * DZCI(k - 1), czp = DZFI(k) * DZCI(k);
      zr[3 * (k - 1)] = czm;
      zr[3 * (k - 1) + 1] = czp;
      zr[3 * (k - 1) + 2] = -2.0 * dxi2 - 2.0 * dyi2 - czm - czp;
    }
    if ((rc = up(pl->zres, zr.data(), zr.size()))) return bail(rc);
  }
  {
    auto zero = [](const double *v, size_t n) { return std::all_of(v, v + n, [](double x) { return x == 0.0; }); };
    pl->rhsb_zero = zero(rhsbx, 2 * (size_t)ny * nz) && zero(rhsby, 2 * (size_t)nx * nz) &&
                    zero(rhsbz, 2 * (size_t)nx * ny);
  }
  if ((rc = up(pl->rhsb[0], rhsbx, 2 * (size_t)ny * nz)) || (rc = up(pl->rhsb[1], rhsby, 2 * (size_t)nx * nz)) ||
      (rc = up(pl->rhsb[2], rhsbz, 2 * (size_t)nx * ny)))
    return bail(rc);
  if ((rc = pl->ext[0] ? build_ext(nx, kx.kf, kx.kb, &pl->ex[0]) : build_axis<double>(nx, px, &pl->tx64)) ||
      (rc = pl->ext[1] ? build_ext(ny, ky.kf, ky.kb, &pl->ex[1]) : build_axis<double>(ny, py, &pl->ty64)))
    return bail(rc);
  if (!pl->ext[0] && !pl->ext[1] &&
      ((rc = build_axis<dd>(nx, px, &pl->txd)) || (rc = build_axis<dd>(ny, py, &pl->tyd))))
    return bail(rc);
  if (!pl->fp64_only &&
      ((rc = build_axis<float>(nx, px, &pl->tx32)) || (rc = build_axis<float>(ny, py, &pl->ty32))))
    return bail(rc);
  const int smax = max_smem_optin();
  pl->path64 = (nx % 2 == 0 && ny % 2 == 0 && (int)plane_smem<dd>(nx, ny) <= smax) ? 1 : 0;
  pl->path32 = (nx % 2 == 0 && ny % 2 == 0 && (int)plane_smem<float>(nx, ny) <= smax) ? 1 : 0;
  // The FP64 solver's double-float transforms take no cluster path: its separate x and y
  // passes measured faster than the cluster plane kernels at 192^2 to 256^2 planes (2.39
  // against 2.56 ms a 256^3 solve) and even at 128^2.
  if (!pl->path32 && (pl->clus32 = cluster_size_for<float>(nx, ny, smax)) &&
      cluster_capacity(k_xyinv_cluster<float, OutHalo>, cluster_plane_smem(nx, ny, pl->clus32, 4), pl->clus32) > 0)
    pl->path32 = 2;
  if (!pl->path32) {  // planes whose only cluster split is a compile-time-sized variant (512^2: 16 CTAs)
    const int cf = fixed_cluster_size(nx, ny, px, py);
    if (cf) {
      pl->path32 = 2;
      pl->clus32 = cf;
    }
  }
  if (pl->path32 && !getenv("FLUTAS_GB300_XY_PATH") && (rc = choose_path32(pl))) return bail(rc);
  // FLUTAS_GB300_XY_PATH: unset, the FP32 form is timed (choose_path32); 0 forces separate
  // passes; any other value keeps the whole-plane form where one exists (A/B timing, tests)
  if (const char *e = getenv("FLUTAS_GB300_XY_PATH")) {
    if (atoi(e) == 0) pl->path64 = pl->path32 = 0;
  }
  if (const char *e = getenv("FLUTAS_GB300_XY_PATH64")) {  // the FP64 solver's transforms alone (A/B timing)
    if (atoi(e) == 0) pl->path64 = 0;
  }
  if (pl->ext[0] || pl->ext[1]) pl->path64 = pl->path32 = 0;  // one pass per axis (k_r2r_ext or k_xfwd/k_ypass)
  if (const char *e = getenv("FLUTAS_GB300_CONTRACTION")) {  // initial predicted contraction (tests)
    const double c = atof(e);
    if (c > 0.0 && c <= 1.0) pl->contraction = c;
  }
  if ((rc = noalloc_prepare())) return bail(rc);  // the allocation-free check is ready on this device
  arrplan[0] = pl;
  arrplan[1] = arrplan[2] = arrplan[3] = nullptr;
  return FLUTAS_OK;
}

int flutas_gb300_fftend(void **arrplan) {
  if (!arrplan) return fail(FLUTAS_EINVAL, "fftend: null arrplan");
  flutas_plan *pl;
  TRY(check_plan(arrplan[0], &pl));
  cudaStreamSynchronize(pl->stream);
  if (pl->copy_stream) {
    cudaStreamSynchronize(pl->copy_stream);
    cudaStreamDestroy(pl->copy_stream);
    cudaEventDestroy(pl->ev_ready);
    cudaEventDestroy(pl->ev_copied);
    cudaEventDestroy(pl->ev_u_ready);
    cudaEventDestroy(pl->ev_u_copied);
  }
  for (cudaEvent_t e : pl->slab_ev) cudaEventDestroy(e);
  DBuf *bufs[] = {&pl->zdf, &pl->zres, &pl->czf, &pl->czc, &pl->a32, &pl->b32, &pl->c32, &pl->lam, &pl->a, &pl->b, &pl->c, &pl->dzci, &pl->dzfi, &pl->rhsb[0], &pl->rhsb[1], &pl->rhsb[2],
                  &pl->tx64.W, &pl->tx64.Q, &pl->ty64.W, &pl->ty64.Q, &pl->tx32.W, &pl->tx32.Q, &pl->ty32.W,
                  &pl->ty32.Q, &pl->S64, &pl->S32, &pl->fbuf, &pl->phi, &pl->phi2, &pl->nrm, &pl->nf_flag,
                  &pl->txd.W, &pl->txd.Q, &pl->tyd.W, &pl->tyd.Q};
  for (DBuf *d : bufs) d->release();
  pl->ex[0].release();
  pl->ex[1].release();
  pl->mir.release();
  pl->magic = 0;
  delete pl;
  arrplan[0] = nullptr;
  return FLUTAS_OK;
}

int flutas_gb300_plan_set_stream(void *plan, void *stream, int synchronous) {
  flutas_plan *pl;
  TRY(check_plan(plan, &pl));
  pl->stream = (cudaStream_t)stream;
  pl->sync = synchronous != 0;
  return FLUTAS_OK;
}

int flutas_gb300_plan_info(void *plan, size_t *device_bytes, int *xy_path_fp64, int *xy_path_fp32) {
  flutas_plan *pl;
  TRY(check_plan(plan, &pl));
  if (device_bytes) {
    size_t s = 0;
    const DBuf *bufs[] = {&pl->zdf, &pl->zres, &pl->czf, &pl->czc, &pl->a32, &pl->b32, &pl->c32, &pl->lam, &pl->a, &pl->b, &pl->c, &pl->dzci, &pl->dzfi, &pl->rhsb[0], &pl->rhsb[1],
                          &pl->rhsb[2], &pl->tx64.W, &pl->tx64.Q, &pl->ty64.W, &pl->ty64.Q, &pl->tx32.W,
                          &pl->tx32.Q, &pl->ty32.W, &pl->ty32.Q, &pl->S64, &pl->S32, &pl->fbuf, &pl->phi, &pl->phi2, &pl->nrm, &pl->nf_flag,
                          &pl->txd.W, &pl->txd.Q, &pl->tyd.W, &pl->tyd.Q};
    for (const DBuf *d : bufs) s += d->bytes;
    for (const DBuf &d : pl->mir.bufs) s += d.bytes;
    *device_bytes = s;
  }
  if (xy_path_fp64) *xy_path_fp64 = pl->path64;
  if (xy_path_fp32) *xy_path_fp32 = pl->path32;
  return FLUTAS_OK;
}

// src/solver_cpu.f90:20-115 (behaviour), src/solver_gpu.f90:31 (GPU form)
int flutas_gb300_solver(const int n[3], void *const *arrplan, double normfft, const double *lambdaxy,
                        const double *a, const double *b, const double *c, const char bcz[2],
                        const char c_or_f[3], double *p) {
  if (!n || !arrplan || !bcz || !c_or_f || !p) return fail(FLUTAS_EINVAL, "solver: null argument");
  flutas_plan *pl;
  TRY(check_plan(arrplan[0], &pl));
  if (n[0] != pl->n[0] || n[1] != pl->n[1] || n[2] != pl->n[2])
    return fail(FLUTAS_EINVAL, "solver: n=(%d,%d,%d) differs from the plan's (%d,%d,%d)", n[0], n[1], n[2], pl->n[0], pl->n[1], pl->n[2]);
  if (bcz[0] != pl->cbc[4] || bcz[1] != pl->cbc[5])
    return fail(FLUTAS_EINVAL, "solver: bcz differs from the plan's z BCs");
  if (c_or_f[0] != pl->c_or_f[0] || c_or_f[1] != pl->c_or_f[1] || c_or_f[2] != pl->c_or_f[2])
    return fail(FLUTAS_EINVAL, "solver: c_or_f differs from the plan's");
  (void)normfft;  // the plan's normfft (identical to initsolver's output) is used
  // coefficient arrays: device pointers are used as given; host arrays must be
  // the ones initsolver filled (their device copies live in the plan)
  auto pick = [&](const double *user, const void *hostinit, const DBuf &dev, size_t cnt, const double **out) -> int {
    if (!user || user == hostinit) { *out = dev.as<double>(); return 0; }
    const int kind = ptr_kind(user);
    if (kind == PTR_OTHER_DEVICE) return reject_other_device("solver", user);
    if (kind == PTR_DEVICE) { *out = user; return 0; }
    // a different host array: refresh the plan's device copy
    CK(cudaMemcpyAsync(dev.p, user, sizeof(double) * cnt, cudaMemcpyHostToDevice, pl->stream));
    *out = dev.as<double>();
    return 0;
  };
  const double *dl, *da, *db, *dc;
  TRY(pick(lambdaxy, pl->host_lam, pl->lam, (size_t)pl->n[0] * pl->n[1], &dl));
  TRY(pick(a, pl->host_a, pl->a, pl->n[2], &da));
  TRY(pick(b, pl->host_b, pl->b, pl->n[2], &db));
  TRY(pick(c, pl->host_c, pl->c, pl->n[2], &dc));
  pl->mir.reset();
  Staged sp;
  const size_t pbytes = sizeof(double) * (size_t)(pl->n[0] + 2) * (pl->n[1] + 2) * (pl->n[2] + 2);
  TRY(stage_in(pl->mir, p, pbytes, true, true, pl->stream, &sp));
  TRY(solve_fp64_dev(pl, sp.d, dl, da, db, dc));
  TRY(stage_out(sp, pl->stream));
  if (sp.host) CK(cudaStreamSynchronize(pl->stream));
  TRY(finish(pl));
  return check_nonfinite(pl, "solver");
}

int flutas_gb300_solve_mixed(void *plan, double *p, double tol, int max_iter, double *relres, int *iters) {
  flutas_plan *pl;
  TRY(check_plan(plan, &pl));
  if (!p) return fail(FLUTAS_EINVAL, "solve_mixed: null p");
  if (!(tol > 0.0) || max_iter < 1) return fail(FLUTAS_EINVAL, "solve_mixed: need tol > 0 and max_iter >= 1");
  if (pl->fp64_only)
    return fail(FLUTAS_EUNSUPPORTED, "solve_mixed: face-centred and odd-length ND/DN plans have the FP64 solver only");
  pl->mir.reset();
  Staged sp;
  const size_t pbytes = sizeof(double) * (size_t)(pl->n[0] + 2) * (pl->n[1] + 2) * (pl->n[2] + 2);
  TRY(stage_in(pl->mir, p, pbytes, true, true, pl->stream, &sp));
  const Geo gh{pl->n[0], pl->n[1], pl->n[2], 1};
  int rc = solve_mixed_dev(pl, InHalo{sp.d, gh}, sp.d, tol, max_iter, &pl->last_relres, &pl->last_iters);
  if (relres) *relres = pl->last_relres;
  if (iters) *iters = pl->last_iters;
  if (rc != 0 && rc != FLUTAS_EITER) return rc;
  TRY(stage_out(sp, pl->stream));
  CK(cudaStreamSynchronize(pl->stream));
  return rc;
}

}  // extern "C"

// ===========================================================================
// Plan-less stencil entry points: a process-wide context (mirrors + stream 0)
// ===========================================================================
namespace {
std::mutex g_ctx_mu;
Mirrors g_ctx_mir;
DBuf g_ctx_small[4];
int boundp_dev(double *p, const int n[3], const char cbc[6], const double bc[6], const double dl[3], double dzc0,
               double dzcn, cudaStream_t st, double *p2 = nullptr);
}  // namespace

extern "C" {

int flutas_gb300_fillps(int nx, int ny, int nz, int nh_d, int nh_u, double dxi, double dyi, double dzi,
                        const double *dzfi, double dti, double rho0, const double *u, const double *v,
                        const double *w, double *p) {
  // src/fillps.f90:16-69
  (void)dzi;
  if (nx < 1 || ny < 1 || nz < 1 || nh_u < 1 || nh_d < 1) return fail(FLUTAS_EINVAL, "fillps: bad sizes");
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  g_ctx_mir.reset();
  cudaStream_t st = 0;
  const size_t ub = sizeof(double) * (size_t)(nx + 2 * nh_u) * (ny + 2 * nh_u) * (nz + 2 * nh_u);
  const size_t pb = sizeof(double) * (size_t)(nx + 2) * (ny + 2) * (nz + 2);
  Staged su, sv, sw, sp, sz;
  TRY(stage_in(g_ctx_mir, u, ub, true, false, st, &su));
  TRY(stage_in(g_ctx_mir, v, ub, true, false, st, &sv));
  TRY(stage_in(g_ctx_mir, w, ub, true, false, st, &sw));
  TRY(stage_in(g_ctx_mir, dzfi, sizeof(double) * (nz + 2 * nh_d), true, false, st, &sz));
  TRY(stage_in(g_ctx_mir, p, pb, true, true, st, &sp));
  TRY(g_ctx_small[1].ensure(sizeof(double) * (nz + 2 * nh_d)));
  double *cz = g_ctx_small[1].as<double>();
  TRY(scale_vecs(sz.d, dti * rho0, cz, nz + 2 * nh_d, st));
  InFillps in;
  in.u = su.d; in.v = sv.d; in.w = sw.d;
  in.cz = cz + (nh_d - 1);
  in.cx = dti * dxi * rho0; in.cy = dti * dyi * rho0;
  in.rhsbx = in.rhsby = in.rhsbz = nullptr;
  in.q1 = in.q2 = in.q3 = 0;
  in.g = Geo{nx, ny, nz, nh_u};
  TRY(launch("k_fillps", st, [&] { k_fillps<<<grid_cells(in.g), 256, 0, st>>>(in, sp.d); }));
  TRY(stage_out(sp, st));
  CK(cudaStreamSynchronize(st));
  return FLUTAS_OK;
}

int flutas_gb300_update_property(const int n[3], const double prop12[2], const double *vof, double *prop) {
  // src/vof.f90:240-271
  if (!n || !prop12 || !vof || !prop) return fail(FLUTAS_EINVAL, "update_property: null argument");
  if (n[0] < 1 || n[1] < 1 || n[2] < 1) return fail(FLUTAS_EINVAL, "update_property: bad sizes");
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  g_ctx_mir.reset();
  cudaStream_t st = 0;
  const size_t pb = sizeof(double) * (size_t)(n[0] + 2) * (n[1] + 2) * (n[2] + 2);
  Staged sv, sp;
  TRY(stage_in(g_ctx_mir, vof, pb, true, false, st, &sv));
  TRY(stage_in(g_ctx_mir, prop, pb, true, true, st, &sp));  // the halo comes back as it went in
  const Geo g{n[0], n[1], n[2], 1};
  TRY(launch("k_update_property", st,
             [&] { k_update_property<<<grid_cells(g), 256, 0, st>>>(sv.d, sp.d, prop12[0], prop12[1], g); }));
  TRY(stage_out(sp, st));
  CK(cudaStreamSynchronize(st));
  return FLUTAS_OK;
}

int flutas_gb300_correc(int nx, int ny, int nz, int nh_d, int nh_u, double dxi, double dyi, double dzi,
                        const double *dzci, double dt, double rho0, const double *p, double *u, double *v,
                        double *w, const double *rho) {
  // src/correc.f90:16-81 (constant-coefficient branch 57-60)
  (void)dzi;
  (void)rho;
  if (nx < 1 || ny < 1 || nz < 1 || nh_u < 1 || nh_d < 1) return fail(FLUTAS_EINVAL, "correc: bad sizes");
  if (rho0 == 0.0) return fail(FLUTAS_EINVAL, "correc: rho0 == 0");
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  g_ctx_mir.reset();
  cudaStream_t st = 0;
  const size_t ub = sizeof(double) * (size_t)(nx + 2 * nh_u) * (ny + 2 * nh_u) * (nz + 2 * nh_u);
  const size_t pb = sizeof(double) * (size_t)(nx + 2) * (ny + 2) * (nz + 2);
  Staged su, sv, sw, sp, sz;
  TRY(stage_in(g_ctx_mir, u, ub, true, true, st, &su));
  TRY(stage_in(g_ctx_mir, v, ub, true, true, st, &sv));
  TRY(stage_in(g_ctx_mir, w, ub, true, true, st, &sw));
  TRY(stage_in(g_ctx_mir, dzci, sizeof(double) * (nz + 2 * nh_d), true, false, st, &sz));
  TRY(stage_in(g_ctx_mir, p, pb, true, false, st, &sp));
  CorrecArgs ca;
  ca.p = sp.d; ca.dzci = sz.d + (nh_d - 1);
  ca.u = su.d; ca.v = sv.d; ca.w = sw.d;
  ca.factori = dt * dxi; ca.factorj = dt * dyi; ca.dt = dt; ca.rho0i = 1.0 / rho0;
  ca.g = Geo{nx, ny, nz, nh_u};
  TRY(launch("k_correc", st, [&] { k_correc<<<grid_cells(ca.g), 256, 0, st>>>(ca); }));
  TRY(stage_out(su, st));
  TRY(stage_out(sv, st));
  TRY(stage_out(sw, st));
  CK(cudaStreamSynchronize(st));
  return FLUTAS_OK;
}

int flutas_gb300_boundp(const char cbc[6], const int n[3], const double bc[6], int nh_d, int nh_p,
                        const int halo[3], const double dl[3], const double *dzc, const double *dzf, double *p) {
  // src/bound.f90:146-225 boundp, set_bc 227-646 (centred, nh_p = 1)
  (void)halo;
  (void)dzf;
  if (!cbc || !n || !bc || !dl || !dzc || !p) return fail(FLUTAS_EINVAL, "boundp: null argument");
  if (nh_p != 1) return fail(FLUTAS_EUNSUPPORTED, "boundp: nh_p must be 1");
  for (int i = 0; i < 6; i++)
    if (!bc_ok(cbc[i])) return fail(FLUTAS_EINVAL, "boundp: bad BC character");
  const int nx = n[0], ny = n[1], nz = n[2];
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  g_ctx_mir.reset();
  cudaStream_t st = 0;
  const size_t pb = sizeof(double) * (size_t)(nx + 2) * (ny + 2) * (nz + 2);
  Staged sp;
  TRY(stage_in(g_ctx_mir, p, pb, true, true, st, &sp));
  // dzc may live on the device: read the two spacings we need
  double dzc0, dzcn;
  if (is_device_ptr(dzc)) {
    CK(cudaMemcpy(&dzc0, dzc + (0 - 1 + nh_d), sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&dzcn, dzc + (nz - 1 + nh_d), sizeof(double), cudaMemcpyDeviceToHost));
  } else {
    dzc0 = dzc[0 - 1 + nh_d];
    dzcn = dzc[nz - 1 + nh_d];
  }
  TRY(boundp_dev(sp.d, n, cbc, bc, dl, dzc0, dzcn, st));
  TRY(stage_out(sp, st));
  CK(cudaStreamSynchronize(st));
  return FLUTAS_OK;
}

int flutas_gb300_chkdiv(int nx, int ny, int nz, double dxi, double dyi, double dzi, int nh_d, int nh_u,
                        const double *dzfi, const double *u, const double *v, const double *w, double *divtot,
                        double *divmax) {
  // src/chkdiv.f90:18-69
  (void)dzi;
  if (!divtot || !divmax) return fail(FLUTAS_EINVAL, "chkdiv: null output");
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  g_ctx_mir.reset();
  cudaStream_t st = 0;
  const size_t ub = sizeof(double) * (size_t)(nx + 2 * nh_u) * (ny + 2 * nh_u) * (nz + 2 * nh_u);
  Staged su, sv, sw, sz;
  TRY(stage_in(g_ctx_mir, u, ub, true, false, st, &su));
  TRY(stage_in(g_ctx_mir, v, ub, true, false, st, &sv));
  TRY(stage_in(g_ctx_mir, w, ub, true, false, st, &sw));
  TRY(stage_in(g_ctx_mir, dzfi, sizeof(double) * (nz + 2 * nh_d), true, false, st, &sz));
  const Geo gd{nx, ny, nz, nh_u};
  dim3 grid3 = grid_cells(gd);
  grid3.y = std::min<unsigned>(grid3.y, 64u);
  grid3.z = std::min<unsigned>(grid3.z, 64u);
  const int grid = (int)(grid3.x * grid3.y * grid3.z);
  TRY(g_ctx_small[0].ensure(sizeof(double) * 2 * grid));
  DivArgs da;
  da.u = su.d; da.v = sv.d; da.w = sw.d; da.dzfi = sz.d + (nh_d - 1);
  da.dxi = dxi; da.dyi = dyi;
  da.g = Geo{nx, ny, nz, nh_u};
  TRY(launch("k_chkdiv", st, [&] { k_chkdiv<<<grid3, 256, 0, st>>>(da, g_ctx_small[0].as<double>()); }));
  std::vector<double> part(2 * grid);
  CK(cudaMemcpyAsync(part.data(), g_ctx_small[0].p, sizeof(double) * 2 * grid, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  double tot = 0.0, mx = 0.0;
  for (int i = 0; i < grid; i++) {
    tot += part[2 * i];
    mx = std::fmax(mx, part[2 * i + 1]);
  }
  *divtot = tot;
  *divmax = mx;
  return FLUTAS_OK;
}

}  // extern "C"

namespace {

// ---- ghost cells in one launch (k_ghosts; maps and their composition: ghosts.cuh).
// Completes a, checks that the maps compose and launches k_ghosts; *done =
// false (nothing launched) when they do not compose.
template <int NC> int ghosts_launch(GhostArgs<NC> &a, cudaStream_t st, bool *done) {
  long tot = 0;
  *done = ghosts_ready(a, &tot);
  if (!*done) return 0;
  static const char *const names[] = {"", "k_ghosts<1>", "k_ghosts<2>", "k_ghosts<3>"};
  TRY(launch(names[NC], st, [&] { k_ghosts<NC><<<stream_grid(tot), 256, 0, st>>>(a, tot); }));
  return 0;
}
// boundp on a device halo array with the plan-less BoundArgs kernel
int boundp_dev(double *p, const int n[3], const char cbc[6], const double bc[6], const double dl[3], double dzc0,
               double dzcn, cudaStream_t st, double *p2) {
  const int nx = n[0], ny = n[1], nz = n[2];
  const double dr[3][2] = {{dl[0], dl[0]}, {dl[1], dl[1]}, {dzc0, dzcn}};
  bool done;
  if (p2) {  // two fields of the same BCs in one launch
    GhostArgs<2> ga;
    ga.f[0] = p;
    ga.f[1] = p2;
    boundp_maps(ga, n, cbc, bc, dr);
    TRY(ghosts_launch(ga, st, &done));
    if (done) return 0;
    TRY(boundp_dev(p2, n, cbc, bc, dl, dzc0, dzcn, st, nullptr));
  } else {
    GhostArgs<1> ga;
    ga.f[0] = p;
    boundp_maps(ga, n, cbc, bc, dr);
    TRY(ghosts_launch(ga, st, &done));
    if (done) return 0;
  }
  for (int d = 0; d < 3; d++) {
    BoundArgs ba;
    ba.p = p;
    ba.g = Geo{nx, ny, nz, 1};
    ba.idir = d + 1;
    ba.ctype0 = cbc[2 * d];
    ba.ctype1 = cbc[2 * d + 1];
    auto fs = [&](char ct, int ib, double rv, double drv, double *f, double *s) {
      if (ct == 'D') { *f = 2.0 * rv; *s = -1.0; }
      else if (ct == 'N') { *f = ib == 0 ? -drv * rv : drv * rv; *s = 1.0; }
      else { *f = 0.0; *s = 0.0; }
    };
    fs(ba.ctype0, 0, bc[2 * d], dr[d][0], &ba.f0, &ba.s0);
    fs(ba.ctype1, 1, bc[2 * d + 1], dr[d][1], &ba.f1, &ba.s1);
    long cnt = d == 0 ? (long)(ny + 2) * (nz + 2) : (d == 1 ? (long)(nx + 2) * (nz + 2) : (long)(nx + 2) * (ny + 2));
    TRY(launch("k_boundp_dir", st, [&] { k_boundp_dir<<<stream_grid(cnt), 256, 0, st>>>(ba); }));
  }
  return 0;
}

// Constants of the Dodd-Ferrante increment (see PresTwArgs): x/y scalars and
// the per-level z factors zA = f_t12*f2/rho0*dzci(k), zB = 2*f_t12*dzci(k)
// computed on the device into zab (2*(nz+2nh_d) doubles); dzci_d is (1-nh_d:).
int presw_consts(PresTwArgs *a, const double *dzci_d, int nh_d, int nz, double dxi, double dyi, double rho0i,
                 double f_t12, double f2, double *zab, ScaleJobs &jobs) {
  const int len = nz + 2 * nh_d;
  a->f2 = f2;
  a->xA = f_t12 * dxi * f2 * rho0i;
  a->xB = 2.0 * f_t12 * dxi;
  a->yA = f_t12 * dyi * f2 * rho0i;
  a->yB = 2.0 * f_t12 * dyi;
  a->xA32 = (float)a->xA; a->xB32 = (float)a->xB; a->yA32 = (float)a->yA; a->yB32 = (float)a->yB;
  a->f2_32 = (float)f2;
  jobs.add(dzci_d, f_t12 * f2 * rho0i, zab, len);
  jobs.add(dzci_d, 2.0 * f_t12, zab + len, len);
  a->zA = zab + (nh_d - 1);
  a->zB = zab + len + (nh_d - 1);
  return 0;
}

int updt_rhs_b_dev(double *p, Geo g, const double *rx, const double *ry, const double *rz, int q1, int q2, int q3,
                   cudaStream_t st) {
  const double *r[3] = {rx, ry, rz};
  const int q[3] = {q1, q2, q3};
  const long cnt[3] = {(long)g.ny * g.nz, (long)g.nx * g.nz, (long)g.nx * g.ny};
  for (int d = 0; d < 3; d++) {
    RhsbArgs ra{p, r[d], g, d + 1, q[d]};
    TRY(launch("k_updt_rhs_b_dir", st, [&] { k_updt_rhs_b_dir<<<stream_grid(cnt[d]), 256, 0, st>>>(ra); }));
  }
  return 0;
}

}  // namespace

extern "C" {

int flutas_gb300_updt_rhs_b(int nx, int ny, int nz, const char c_or_f[3], const char cbc[6], int nh_p,
                            const double *rhsbx, const double *rhsby, const double *rhsbz, double *p) {
  // src/bound.f90:829-944 (single domain: every face is a physical boundary)
  if (!c_or_f || !cbc) return fail(FLUTAS_EINVAL, "updt_rhs_b: null argument");
  if (nh_p != 1) return fail(FLUTAS_EUNSUPPORTED, "updt_rhs_b: nh_p must be 1");
  const int q1 = (c_or_f[0] == 'f' && cbc[1] == 'D'), q2 = (c_or_f[1] == 'f' && cbc[3] == 'D'),
            q3 = (c_or_f[2] == 'f' && cbc[5] == 'D');
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  g_ctx_mir.reset();
  cudaStream_t st = 0;
  const size_t pb = sizeof(double) * (size_t)(nx + 2) * (ny + 2) * (nz + 2);
  Staged sp, sx, sy, sz;
  TRY(stage_in(g_ctx_mir, p, pb, true, true, st, &sp));
  TRY(stage_in(g_ctx_mir, rhsbx, sizeof(double) * 2 * (size_t)ny * nz, true, false, st, &sx));
  TRY(stage_in(g_ctx_mir, rhsby, sizeof(double) * 2 * (size_t)nx * nz, true, false, st, &sy));
  TRY(stage_in(g_ctx_mir, rhsbz, sizeof(double) * 2 * (size_t)nx * ny, true, false, st, &sz));
  TRY(updt_rhs_b_dev(sp.d, Geo{nx, ny, nz, 1}, sx.d, sy.d, sz.d, q1, q2, q3, st));
  TRY(stage_out(sp, st));
  CK(cudaStreamSynchronize(st));
  return FLUTAS_OK;
}

int flutas_gb300_pres_tw_src(int nx, int ny, int nz, double dxi, double dyi, double dzi, int nh_d, int nh_u,
                             const double *dzci, double rho0i, double f_t12, double f_t12_o, const double *p,
                             const double *pold, const double *rho, double *u, double *v, double *w) {
  // src/source.f90:247-309, constant-coefficient branch (289-295)
  (void)dzi;
  if (f_t12_o == 0.0) return fail(FLUTAS_EINVAL, "pres_tw_src: f_t12_o == 0");
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  g_ctx_mir.reset();
  cudaStream_t st = 0;
  const size_t ub = sizeof(double) * (size_t)(nx + 2 * nh_u) * (ny + 2 * nh_u) * (nz + 2 * nh_u);
  const size_t pb = sizeof(double) * (size_t)(nx + 2) * (ny + 2) * (nz + 2);
  Staged su, sv, sw, sp, so, sr, sz;
  TRY(stage_in(g_ctx_mir, u, ub, true, true, st, &su));
  TRY(stage_in(g_ctx_mir, v, ub, true, true, st, &sv));
  TRY(stage_in(g_ctx_mir, w, ub, true, true, st, &sw));
  TRY(stage_in(g_ctx_mir, p, pb, true, false, st, &sp));
  TRY(stage_in(g_ctx_mir, pold, pb, true, false, st, &so));
  TRY(stage_in(g_ctx_mir, rho, pb, true, false, st, &sr));
  TRY(stage_in(g_ctx_mir, dzci, sizeof(double) * (nz + 2 * nh_d), true, false, st, &sz));
  const double f2 = (f_t12 / f_t12_o);
  TRY(g_ctx_small[2].ensure(sizeof(double) * 2 * (nz + 2 * nh_d)));
  double *zab = g_ctx_small[2].as<double>();
  PresTwArgs a;
  a.p = sp.d; a.pold = so.d; a.rho = sr.d;
  a.u = su.d; a.v = sv.d; a.w = sw.d;
  ScaleJobs jobs;
  TRY(presw_consts(&a, sz.d, nh_d, nz, dxi, dyi, rho0i, f_t12, f2, zab, jobs));
  TRY(scale_jobs(jobs, st));
  a.fp32 = 0;
  a.g = Geo{nx, ny, nz, nh_u};
  TRY(launch("k_pres_tw_src", st, [&] { k_pres_tw_src<<<presw_grid(a.g), PRESTW_NT, 0, st>>>(a); }));
  TRY(stage_out(su, st));
  TRY(stage_out(sv, st));
  TRY(stage_out(sw, st));
  CK(cudaStreamSynchronize(st));
  return FLUTAS_OK;
}

}  // extern "C"

namespace {

// bounduvw (src/bound.f90:17-144), single domain, with the outflow faces of
// src/bound.f90:649-773 when isoutflow is given.  dzc/dzf host
// values.  One k_ghosts launch for the three set_bc passes (the pass-by-pass
// kernel, x then y then z as the reference, where the maps do not compose).
// bounduvw's ghost maps (one launch of k_ghosts for the three passes).
void bounduvw_maps(const char *cbc, const double *bc, int nx, int ny, int nz, int nh_d, int h, const double dl[3],
                   const double *dzc_h, const double *dzf_h, double *u, double *v, double *w, GhostArgs<3> *ga,
                   BcSide sides[3][3][2]) {
  setbc_sides(cbc, bc, nz, nh_d, h, dl, dzc_h, dzf_h, sides);
  ga->f[0] = u; ga->f[1] = v; ga->f[2] = w;
  ga->n[0] = nx; ga->n[1] = ny; ga->n[2] = nz; ga->h = h;
  for (int d = 0; d < 3; d++)
    for (int c = 0; c < 3; c++) setbc_maps(ga->m[c][d], sides[d][c], ga->n[d], h);
}

int bounduvw_dev(const char *cbc, const double *bc, int nx, int ny, int nz, int nh_d, int h, const double dl[3],
                 const double *dzc_h, const double *dzf_h, double *u, double *v, double *w, cudaStream_t st,
                 const int *isoutflow = nullptr, const double *dzf_d = nullptr) {
  if (h < 1 || h > 4) return fail(FLUTAS_EUNSUPPORTED, "bounduvw: halo %d not in 1..4", h);
  BcSide sides[3][3][2];
  GhostArgs<3> ga;
  bounduvw_maps(cbc, bc, nx, ny, nz, nh_d, h, dl, dzc_h, dzf_h, u, v, w, &ga, sides);
  SetBc3Args passes[3];
  for (int d = 0; d < 3; d++) {
    SetBc3Args &a = passes[d];
    a.f[0] = u; a.f[1] = v; a.f[2] = w;
    a.nx = nx; a.ny = ny; a.nz = nz; a.h = h; a.idir = d + 1;
    for (int c = 0; c < 3; c++)
      for (int ib = 0; ib < 2; ib++) a.side[c][ib] = sides[d][c][ib];
  }
  bool done;
  TRY(ghosts_launch(ga, st, &done));
  for (int d = 0; d < 3 && !done; d++) {  // grids too small for the maps to compose: pass by pass
    const SetBc3Args &a = passes[d];
    const int na = d == 0 ? ny : nx, nb = d == 2 ? ny : nz;
    const long cnt = (long)(na + 2 * h) * (nb + 2 * h);
    TRY(launch("k_set_bc3", st, [&] { k_set_bc3<<<stream_grid(cnt), 256, 0, st>>>(a); }));
  }
  if (isoutflow)  // src/bound.f90:130-141: directions in order, low side first
    for (int q = 1; q <= 3; q++)
      for (int id = 0; id <= 1; id++) {
        if (!isoutflow[id + 2 * (q - 1)]) continue;
        OutflowArgs o;
        o.u = u; o.v = v; o.w = w;
        o.dzf = dzf_d;
        o.dx = dl[0]; o.dy = dl[1]; o.dxi = 1.0 / dl[0]; o.dyi = 1.0 / dl[1];
        o.nx = nx; o.ny = ny; o.nz = nz; o.h = h; o.idir = id == 0 ? -q : q;
        const long pts = (long)(q == 1 ? ny : nx) * (q == 3 ? ny : nz) * (h + 1);
        TRY(launch("k_outflow", st, [&] { k_outflow<<<stream_grid(pts), 256, 0, st>>>(o); }));
      }
  return 0;
}

int check_cbcvel(const char *cbcvel) {
  for (int i = 0; i < 18; i++)
    if (!bc_ok(cbcvel[i])) return fail(FLUTAS_EINVAL, "bad velocity BC character '%c'", cbcvel[i]);
  return 0;
}

}  // namespace

extern "C" {

int flutas_gb300_bounduvw(const char cbcvel[18], const int n[3], const double bcvel[18], int nh_d, int nh_u,
                          const int halo[3], const int isoutflow[6], const double dl[3], const double *dzc,
                          const double *dzf, double *u, double *v, double *w) {
  // src/bound.f90:17-144
  (void)halo;
  if (!cbcvel || !n || !bcvel || !dl || !dzc || !dzf) return fail(FLUTAS_EINVAL, "bounduvw: null argument");
  TRY(check_cbcvel(cbcvel));
  if (nh_u < 1 || nh_u > 4 || nh_d < nh_u) return fail(FLUTAS_EINVAL, "bounduvw: bad halo sizes");
  bool any_outflow = false;
  if (isoutflow)
    for (int i = 0; i < 6; i++) any_outflow |= isoutflow[i] != 0;
  const int nx = n[0], ny = n[1], nz = n[2];
  std::vector<double> dzc_h(nz + 2 * nh_d), dzf_h(nz + 2 * nh_d);
  const size_t zb = sizeof(double) * (nz + 2 * nh_d);
  if (is_device_ptr(dzc)) {
    CK(cudaMemcpy(dzc_h.data(), dzc, zb, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(dzf_h.data(), dzf, zb, cudaMemcpyDeviceToHost));
  } else {
    memcpy(dzc_h.data(), dzc, zb);
    memcpy(dzf_h.data(), dzf, zb);
  }
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  g_ctx_mir.reset();
  cudaStream_t st = 0;
  const size_t ub = sizeof(double) * (size_t)(nx + 2 * nh_u) * (ny + 2 * nh_u) * (nz + 2 * nh_u);
  Staged su, sv, sw;
  TRY(stage_in(g_ctx_mir, u, ub, true, true, st, &su));
  TRY(stage_in(g_ctx_mir, v, ub, true, true, st, &sv));
  TRY(stage_in(g_ctx_mir, w, ub, true, true, st, &sw));
  double *dzf_d = nullptr;
  if (any_outflow) {  // the outflow faces need dzf on the device
    TRY(g_ctx_small[2].ensure(zb));
    dzf_d = g_ctx_small[2].as<double>();
    CK(cudaMemcpyAsync(dzf_d, dzf_h.data(), zb, cudaMemcpyHostToDevice, st));
  }
  TRY(bounduvw_dev(cbcvel, bcvel, nx, ny, nz, nh_d, nh_u, dl, dzc_h.data(), dzf_h.data(), su.d, sv.d, sw.d, st,
                   any_outflow ? isoutflow : nullptr, dzf_d ? dzf_d + (nh_d - 1) : nullptr));
  TRY(stage_out(su, st));
  TRY(stage_out(sv, st));
  TRY(stage_out(sw, st));
  CK(cudaStreamSynchronize(st));
  return FLUTAS_OK;
}

}  // extern "C"

namespace {

int ensure_copy_stream(flutas_plan *pl) {
  if (pl->copy_stream) return 0;
  CK(cudaStreamCreateWithFlags(&pl->copy_stream, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&pl->ev_ready, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&pl->ev_copied, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&pl->ev_u_ready, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&pl->ev_u_copied, cudaEventDisableTiming));
  return 0;
}

// The mixed solve's first pass runs as a stencil pass plus the compile-time
// plane kernels (solve_mixed_dev's split form).
bool mixed_split(const flutas_plan *pl) {
  return pl->path32 == 2 && fixed_supported(pl->n[0], pl->n[1], pl->clus32, pl->tx32.ap.pair, pl->ty32.ap.pair);
}

// Host fields of the fused mixed projection copied in on the plan's copy
// stream, the last one (w) in z-slabs, with the step's first pass
// (Dodd-Ferrante terms, ghost cells of u*, v*, w*, fillps into the FP64 RHS
// and the FP32 spectrum, the forward plane transforms) running slab by slab
// behind the copies on the plan stream.  None of them reads w above the planes
// it writes, so slab s runs once w's slab s is in; the other fields arrive
// whole, first (one copy each: the link loses ~5 us a copy, and while kernels
// run beside it the copies also slow down, so only the last field is cut).
// Fields: halo h, device mirror, host array (page-locked), cut in slabs or not.
struct SlabIn {
  int nslab = 0, K = 0;  // slabs of K interior planes (the last one may be shorter)
  struct Field {
    const void *host;
    double *dev;
    int h;
    bool sliced;
  } f[6];
  int nf = 0;
  GhostArgs<3> ga;  // bounduvw's maps (cbcvel given)
  bool ghosts = false;
};

// Slab s's extended planes [e0, e1) of a field with halo h: its interior
// planes, and the ghost planes below the first slab / above the last one.
void slab_planes(int s, int nslab, int K, int nz, int h, int *e0, int *e1) {
  const int ka = 1 + s * K, kb = std::min(nz, ka + K - 1);
  *e0 = s == 0 ? 0 : ka + h - 1;
  *e1 = s == nslab - 1 ? nz + 2 * h : kb + h;
}

// The slab form of the fused mixed projection, when it applies: every field
// a page-locked host array, the split first pass, no boundary RHS (fillps adds
// no plane-dependent terms), and bounduvw's z ghost cells below the first slab
// computed from planes of the first slab (not z-periodic velocities).
bool slab_plan(flutas_plan *pl, int nh_u, double dxi, double dyi, const char *cbcvel, const double *bcvel,
               const void *const hosts[6], SlabIn *sl) {
  const char *e = getenv("FLUTAS_GB300_SLABS");
  if (e && atoi(e) == 0) return false;
  if (!mixed_split(pl) || !pl->rhsb_zero) return false;
  for (int q = 0; q < 6; q++)
    if (hosts[q] && (ptr_kind(hosts[q]) != PTR_HOST || !is_pinned_host(hosts[q]))) return false;
  const int nx = pl->n[0], ny = pl->n[1], nz = pl->n[2], nh_d = pl->nh_d;
  sl->K = std::max(16, ((nz + 7) / 8 + 15) / 16 * 16);  // about eight slabs of a multiple of 16 planes
  sl->nslab = (nz + sl->K - 1) / sl->K;
  if (sl->nslab < 2 || sl->K < nh_u + 2) return false;
  if (cbcvel) {
    std::vector<double> dzc_h(nz + 2 * nh_d), dzf_h(nz + 2 * nh_d);
    for (int k = 0; k < nz + 2 * nh_d; k++) {
      dzc_h[k] = 1.0 / pl->dzci_h[k];
      dzf_h[k] = 1.0 / pl->dzfi_h[k];
    }
    const double dl[3] = {1.0 / dxi, 1.0 / dyi, 0.0};
    BcSide sides[3][3][2];
    bounduvw_maps(cbcvel, bcvel, nx, ny, nz, nh_d, nh_u, dl, dzc_h.data(), dzf_h.data(), nullptr, nullptr,
                  nullptr, &sl->ga, sides);
    long tot = 0;
    if (!ghosts_ready(sl->ga, &tot)) return false;
    for (int c = 0; c < 3; c++)
      for (int t = 1 - nh_u; t <= 0; t++) {
        const GMap &m = sl->ga.m[c][2][-t];
        if ((m.kind == GM_COPY || m.kind == GM_AFF) && m.src > sl->K) return false;
      }
    sl->ghosts = true;
  }
  return true;
}

// The copies in on the copy stream (the sliced field slab by slab, after the
// whole ones), and the first pass of the step behind them on the plan stream
// (slab s once the sliced field's slab s is in):
// pres_tw_src (a non-null), bounduvw's ghost cells of the slab's planes,
// fillps into the FP64 RHS (fbuf) and the FP32 spectrum with ||f||^2, and the
// forward plane transforms.  The kernels take the slab as a grid of nzs
// planes whose arrays start ka - 1 planes in (every access is relative to the
// cell); the results equal one pass over the grid bit for bit.
int slab_first_pass(flutas_plan *pl, SlabIn &sl, const PresTwArgs *a, const InFillps &in, int max_iter,
                    cudaStream_t st) {
  const int nx = pl->n[0], ny = pl->n[1], nz = pl->n[2];
  TRY(ensure_copy_stream(pl));
  while ((int)pl->slab_ev.size() < sl.nslab) {
    cudaEvent_t e;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    pl->slab_ev.push_back(e);
  }
  cudaStream_t cs = pl->copy_stream;
  CK(cudaEventRecord(pl->ev_ready, st));  // the mirrors are free once the plan stream's earlier work is done
  CK(cudaStreamWaitEvent(cs, pl->ev_ready, 0));
  for (int q = 0; q < sl.nf; q++) {
    const SlabIn::Field &F = sl.f[q];
    if (!F.sliced)
      CK(cudaMemcpyAsync(F.dev, F.host, sizeof(double) * (size_t)(nx + 2 * F.h) * (ny + 2 * F.h) * (nz + 2 * F.h),
                         cudaMemcpyHostToDevice, cs));
  }
  for (int s = 0; s < sl.nslab; s++) {
    for (int q = 0; q < sl.nf; q++) {
      const SlabIn::Field &F = sl.f[q];
      if (!F.sliced) continue;
      const size_t plane = sizeof(double) * (size_t)(nx + 2 * F.h) * (ny + 2 * F.h);
      int e0, e1;
      slab_planes(s, sl.nslab, sl.K, nz, F.h, &e0, &e1);
      CK(cudaMemcpyAsync((char *)F.dev + plane * e0, (const char *)F.host + plane * e0, plane * (e1 - e0),
                         cudaMemcpyHostToDevice, cs));
    }
    CK(cudaEventRecord(pl->slab_ev[s], cs));
  }
  const int nrm_len = std::max(max_iter, 1) + 2;
  TRY(pl->S32.ensure(sizeof(float) * (size_t)nx * ny * nz));
  TRY(pl->fbuf.ensure(sizeof(double) * (size_t)(nx + 2) * (ny + 2) * (nz + 2)));
  TRY(pl->nrm.ensure(sizeof(double) * nrm_len));
  float *S = pl->S32.as<float>();
  double *f = pl->fbuf.as<double>(), *nrm = pl->nrm.as<double>();
  CK(cudaMemsetAsync(nrm, 0, sizeof(double) * nrm_len, st));
  const long psz = (long)(nx + 2) * (ny + 2), usz = (long)(nx + 2 * in.g.h) * (ny + 2 * in.g.h);
  const long ssz = (long)nx * ny;
  for (int s = 0; s < sl.nslab; s++) {
    const int ka = 1 + s * sl.K, kb = std::min(nz, ka + sl.K - 1), nzs = kb - ka + 1;
    const long sh = ka - 1;
    CK(cudaStreamWaitEvent(st, pl->slab_ev[s], 0));
    if (a) {
      PresTwArgs as = *a;
      as.p += sh * psz; as.pold += sh * psz; as.rho += sh * psz;
      as.u += sh * usz; as.v += sh * usz; as.w += sh * usz;
      as.zA += sh; as.zB += sh;
      as.g.nz = nzs;
      TRY(launch("k_pres_tw_src", st, [&] { k_pres_tw_src<<<presw_grid(as.g), PRESTW_NT, 0, st>>>(as); }));
    }
    if (sl.ghosts) {
      int e0, e1;
      slab_planes(s, sl.nslab, sl.K, nz, sl.ga.h, &e0, &e1);
      const GhostSegs gs = ghost_segs_of_planes(sl.ga, e0, e1);
      if (gs.total > 0)
        TRY(launch("k_ghosts<3>", st, [&] { k_ghosts_seg<3><<<stream_grid(gs.total), 256, 0, st>>>(sl.ga, gs); }));
    }
    InFillps is = in;
    is.u += sh * usz; is.v += sh * usz; is.w += sh * usz;
    is.cz += sh;
    is.g.nz = nzs;
    const Geo gs{nx, ny, nzs, 1};
    const long cells = (long)nx * ny * nzs;
    const int grid = grid_for(k_stencil_pass<InFillps, float>, 256, 0, (cells + 1023) / 1024);
    if (grid < 0) return grid;
    if (cells >= (1L << 31) - 4096)
      TRY(launch("k_stencil<fillps>", st, [&] {
        k_stencil_pass<InFillps, float, long long><<<grid, 256, 0, st>>>(is, gs, f + sh * psz, S + sh * ssz, nrm);
      }));
    else
      TRY(launch("k_stencil<fillps>", st, [&] {
        k_stencil_pass<InFillps, float><<<grid, 256, 0, st>>>(is, gs, f + sh * psz, S + sh * ssz, nrm);
      }));
    TRY(fwd_xy<float>(pl, InF32{S + sh * ssz, gs}, S + sh * ssz, pl->tx32, pl->ty32, pl->path32, nullptr, nzs));
  }
  return 0;
}

// Body of the fused projection on staged device pointers (plan stream).
// rho/pold non-null: the Dodd-Ferrante explicit terms of pres_tw_src
// (src/source.f90:247-309) are added to u*,v*,w* first.
int projection_dev(flutas_plan *pl, int nh_u, double dxi, double dyi, const double *dzci_d, const double *dzfi_d,
                   double dt, double rho0, double *u, double *v, double *w, double *p, int precision, double tol,
                   int max_iter, const double *rho, double *pold, double f_t12_o, const char *cbcvel,
                   const double *bcvel, Staged *pold_host = nullptr, SlabIn *slabs = nullptr,
                   Staged *u_host = nullptr) {
  const int nx = pl->n[0], ny = pl->n[1], nz = pl->n[2], nh_d = pl->nh_d;
  Geo g{nx, ny, nz, nh_u};
  std::vector<double> dzc_h(nz + 2 * nh_d), dzf_h(nz + 2 * nh_d);
  for (int k = 0; k < nz + 2 * nh_d; k++) {
    dzc_h[k] = 1.0 / pl->dzci_h[k];
    dzf_h[k] = 1.0 / pl->dzfi_h[k];
  }
  const double dlv[3] = {1.0 / dxi, 1.0 / dyi, 0.0};
  cudaStream_t st = pl->stream;
  const size_t pb = sizeof(double) * (size_t)(nx + 2) * (ny + 2) * (nz + 2);
  const double dl[3] = {1.0 / dxi, 1.0 / dyi, 0.0};
  const double dzc0 = 1.0 / pl->dzci_h[0 - 1 + nh_d], dzcn = 1.0 / pl->dzci_h[nz - 1 + nh_d];
  bool pold_early = false;  // pold = p done right after pres_tw_src, its host copy overlapping the solve
  // every folded z factor of the step in one launch: Dodd-Ferrante, fillps, correc
  const double dti = 1.0 / dt, rho0i = 1.0 / rho0;
  ScaleJobs jobs;
  PresTwArgs a;
  if (rho) {
    TRY(pl->zdf.ensure(sizeof(double) * 2 * (nz + 2 * nh_d)));
    TRY(presw_consts(&a, dzci_d, nh_d, nz, dxi, dyi, rho0i, dt, dt / f_t12_o, pl->zdf.as<double>(), jobs));
  }
  TRY(pl->czf.ensure(sizeof(double) * (nz + 2 * nh_d)));
  TRY(pl->czc.ensure(sizeof(double) * (nz + 2 * nh_d)));
  jobs.add(dzfi_d, dti * rho0, pl->czf.as<double>(), nz + 2 * nh_d);
  jobs.add(dzci_d, dt * rho0i, pl->czc.as<double>(), nz + 2 * nh_d);
  TRY(scale_jobs(jobs, st));
  InFillps in;
  in.u = u; in.v = v; in.w = w;
  in.cz = pl->czf.as<double>() + (nh_d - 1);
  in.cx = dti * dxi * rho0; in.cy = dti * dyi * rho0;
  in.rhsbx = pl->rhsb[0].as<double>(); in.rhsby = pl->rhsb[1].as<double>(); in.rhsbz = pl->rhsb[2].as<double>();
  if (pl->rhsb_zero) in.rhsbx = in.rhsby = in.rhsbz = nullptr;  // adding zeros changes nothing
  in.q1 = in.q2 = in.q3 = 0;
  in.g = g;
  if (rho) {
    a.p = p; a.pold = pold; a.rho = rho;
    a.u = u; a.v = v; a.w = w;
    a.fp32 = precision == 1 ? 1 : 0;  // FP32 increment in the mixed path, FP64 in the FP64 path
    a.g = g;
  }
  if (slabs) TRY(slab_first_pass(pl, *slabs, rho ? &a : nullptr, in, max_iter, st));
  if (rho) {
    if (!slabs)
      TRY(launch("k_pres_tw_src", st, [&] { k_pres_tw_src<<<presw_grid(a.g), PRESTW_NT, 0, st>>>(a); }));
    if (pold_host && pold_host->host && pold_host->out && is_pinned_host(pold_host->host)) {
      // pres_tw_src has read pold: pold = p now (whole array, then boundp: the same values as the
      // correction pass would write), and its copy to the page-locked host array runs on the
      // plan's copy stream while the solve runs on this one
      CK(cudaMemcpyAsync(pold, p, pb, cudaMemcpyDeviceToDevice, st));
      TRY(boundp_dev(pold, pl->n, pl->cbc, pl->bc, dl, dzc0, dzcn, st));
      TRY(ensure_copy_stream(pl));
      CK(cudaEventRecord(pl->ev_ready, st));
      CK(cudaStreamWaitEvent(pl->copy_stream, pl->ev_ready, 0));
      CK(cudaMemcpyAsync((void *)pold_host->host, pold, pb, cudaMemcpyDeviceToHost, pl->copy_stream));
      CK(cudaEventRecord(pl->ev_copied, pl->copy_stream));
      pold_host->out = false;  // copied: the caller's stage_out skips it
      pold_early = true;
    }
  }
  // ghosts of u*,v*,w* as the app leaves them before fillps (bounduvw)
  if (cbcvel && !slabs)
    TRY(bounduvw_dev(cbcvel, bcvel, nx, ny, nz, nh_d, nh_u, dlv, dzc_h.data(), dzf_h.data(), u, v, w, st));
  TRY(pl->phi.ensure(pb));
  double *phi = pl->phi.as<double>();
  const Geo gp{nx, ny, nz, 1};
  int rc = 0;
  if (precision == 0) {
    TRY(pl->S64.ensure(sizeof(double) * (size_t)nx * ny * nz));
    // fillps at full occupancy (the FP64 pipe bounds it) into the spectrum array, then the
    // transforms in place: double-float (dd.cuh) for the paired / DCT-IV kinds, FP64 for
    // the extended-FFT kinds
    const Geo gs{nx, ny, nz, 1};
    const long cells = (long)nx * ny * nz;
    auto fill = [&](auto *S) -> int {
      using TO = std::remove_pointer_t<decltype(S)>;
      const int grid = grid_for(k_stencil_pass<InFillps, TO>, 256, 0, (cells + 1023) / 1024);
      if (grid < 0) return grid;
      const char *nm = std::is_same<TO, dd>::value ? "k_stencil<df64,fillps>" : "k_stencil<f64,fillps>";
      if (cells >= (1L << 31) - 4096)  // the int variant also forms indices up to 3 blocks past the end
        return launch(nm, st, [&] {
          k_stencil_pass<InFillps, TO, long long><<<grid, 256, 0, st>>>(in, gs, nullptr, S, nullptr);
        });
      return launch(nm, st, [&] { k_stencil_pass<InFillps, TO><<<grid, 256, 0, st>>>(in, gs, nullptr, S, nullptr); });
    };
    if (pl->ext[0] || pl->ext[1]) {  // odd-length ND/DN: extended-FFT passes
      double *S = pl->S64.as<double>();
      TRY(fill(S));
      TRY(solve_fp64_ext_spec(pl, S, phi, pl->lam.as<double>(), pl->a.as<double>(), pl->b.as<double>(),
                              pl->c.as<double>()));
    } else {
      dd *S = pl->S64.as<dd>();
      TRY(fill(S));
      TRY(fwd_xy<dd>(pl, InPlainDD{S, gs}, S, pl->txd, pl->tyd, pl->path64));
      TRY((zsolve<double, dd>(pl, S, pl->lam.as<double>(), pl->a.as<double>(), pl->b.as<double>(),
                              pl->c.as<double>(), pl->pin_zero_mode)));
      TRY(inv_xy<dd>(pl, S, OutHalo{phi, pl->normfft, gp}, pl->txd, pl->tyd, pl->path64));
    }
  }
  CorrecAddArgs ca;
  ca.phi = phi; ca.cz = pl->czc.as<double>() + (nh_d - 1);
  ca.u = u; ca.v = v; ca.w = w; ca.p = p;
  ca.pold = pold_early ? nullptr : pold;  // two-phase step: pold = p^n (main__two_phase_inc_isot.f90:655-674)
  ca.cx = (dt * dxi) * rho0i; ca.cy = (dt * dyi) * rho0i;
  ca.g = g;
  FinalCorrec fc;
  // u's copy to a page-locked host array starts while v, w and p are corrected:
  // its ghost cells (bounduvw's maps of u alone; v's and w's after the solve)
  GhostArgs<1> gu;
  GhostArgs<2> gvw;
  bool u_split = false;
  if (precision != 0 && u_host && u_host->host && u_host->out && is_pinned_host(u_host->host)) {
    u_split = true;
    if (cbcvel) {
      GhostArgs<3> g3;
      BcSide sides[3][3][2];
      bounduvw_maps(cbcvel, bcvel, nx, ny, nz, nh_d, nh_u, dlv, dzc_h.data(), dzf_h.data(), u, v, w, &g3, sides);
      gu.f[0] = u;
      gvw.f[0] = v; gvw.f[1] = w;
      for (int d = 0; d < 3; d++) {
        gu.n[d] = gvw.n[d] = g3.n[d];
        for (int sl = 0; sl < GM_SLOTS; sl++) {
          gu.m[0][d][sl] = g3.m[0][d][sl];
          gvw.m[0][d][sl] = g3.m[1][d][sl];
          gvw.m[1][d][sl] = g3.m[2][d][sl];
        }
      }
      gu.h = gvw.h = g3.h;
      long t1 = 0, t2 = 0;
      u_split = ghosts_ready(gu, &t1) && ghosts_ready(gvw, &t2);
    }
  }
  // ghost cells of the corrected u, v, w (bounduvw; v and w only when u went back early
  // with its own) and of p and pold (boundp)
  auto final_ghosts = [&](bool skip_u) -> int {
    if (cbcvel) {
      if (skip_u) {
        bool done = false;
        TRY(ghosts_launch(gvw, st, &done));
      } else {
        TRY(bounduvw_dev(cbcvel, bcvel, nx, ny, nz, nh_d, nh_u, dlv, dzc_h.data(), dzf_h.data(), u, v, w, st));
      }
    }
    return boundp_dev(p, pl->n, pl->cbc, pl->bc, dl, dzc0, dzcn, st, pold_early ? nullptr : pold);  // and pold
  };
  if (precision != 0) {
    fc.ca = ca;
    fc.boundp_phi = [&] { return boundp_dev(phi, pl->n, pl->cbc, pl->bc, dl, dzc0, dzcn, st); };
    fc.ghosts_after = [&] { return final_ghosts(u_split); };
    if (u_split)
      fc.u_first = [&]() -> int {
        if (cbcvel) {
          bool done = false;
          TRY(ghosts_launch(gu, st, &done));
        }
        TRY(ensure_copy_stream(pl));
        CK(cudaEventRecord(pl->ev_u_ready, st));
        CK(cudaStreamWaitEvent(pl->copy_stream, pl->ev_u_ready, 0));
        CK(cudaMemcpyAsync((void *)u_host->host, u, u_host->bytes, cudaMemcpyDeviceToHost, pl->copy_stream));
        CK(cudaEventRecord(pl->ev_u_copied, pl->copy_stream));
        return 0;
      };
    rc = solve_mixed_dev(pl, in, phi, tol, max_iter, &pl->last_relres, &pl->last_iters, &fc, slabs != nullptr);
    if (rc != 0 && rc != FLUTAS_EITER) return rc;
  }
  // u changes again below (the solve went on after its fused check): after its early copy
  if (fc.u_early && fc.continued) CK(cudaStreamWaitEvent(st, pl->ev_u_copied, 0));
  if (!fc.applied) {
    TRY(boundp_dev(phi, pl->n, pl->cbc, pl->bc, dl, dzc0, dzcn, st));
    TRY(launch("k_correc_padd", st, [&] { k_correc_padd<<<grid_cells(ca.g), 256, 0, st>>>(ca); }));
  } else if (fc.continued) {  // the correction of x - (x as applied)
    double *d = fc.snapshot;
    const long n = (long)(nx + 2) * (ny + 2) * (nz + 2);
    TRY(launch("k_sub", st, [&] { k_sub<<<stream_grid(n), 256, 0, st>>>(phi, d, d, n); }));
    TRY(boundp_dev(d, pl->n, pl->cbc, pl->bc, dl, dzc0, dzcn, st));
    CorrecAddArgs cd = ca;
    cd.phi = d;
    cd.pold = nullptr;  // written by the first application
    TRY(launch("k_correc_padd", st, [&] { k_correc_padd<<<grid_cells(cd.g), 256, 0, st>>>(cd); }));
  }
  const bool u_final = fc.u_early && !fc.continued;  // u's early copy holds its final values
  if (!fc.ghosts_queued || fc.continued) TRY(final_ghosts(u_final));
  if (pold_early) CK(cudaStreamWaitEvent(st, pl->ev_copied, 0));  // the stream's end covers the copy
  if (fc.u_early) {
    if (u_final) u_host->out = false;  // copied; the caller's stage_out skips it
    CK(cudaStreamWaitEvent(st, pl->ev_u_copied, 0));
  }
  return rc;
}

int projection_entry(void *plan, int nh_u, double dxi, double dyi, const double *dzci, const double *dzfi,
                     const double bcpre[6], double dt, double rho0, double *u, double *v, double *w, double *p,
                     int precision, double tol, int max_iter, const double *rho, double *pold,
                     double f_t12_o, const char *cbcvel, const double *bcvel) {
  flutas_plan *pl;
  TRY(check_plan(plan, &pl));
  if (!dzci || !dzfi || !bcpre || !u || !v || !w || !p) return fail(FLUTAS_EINVAL, "projection: null argument");
  if (nh_u < 1 || dt == 0.0 || rho0 == 0.0) return fail(FLUTAS_EINVAL, "projection: bad nh_u/dt/rho0");
  if (precision == 1 && (!(tol > 0.0) || max_iter < 1)) return fail(FLUTAS_EINVAL, "projection: need tol > 0, max_iter >= 1");
  if (pl->face) return fail(FLUTAS_EUNSUPPORTED, "projection: the fused projection is cell-centred (c_or_f = 'ccc')");
  if (precision == 1 && pl->fp64_only)
    return fail(FLUTAS_EUNSUPPORTED, "projection: odd-length ND/DN plans project in FP64 only (precision 0)");
  for (int i = 0; i < 6; i++)
    if (bcpre[i] != pl->bc[i]) return fail(FLUTAS_EINVAL, "projection: bcpre differs from initsolver's bc");
  if (cbcvel) {
    TRY(check_cbcvel(cbcvel));
    if (!bcvel) return fail(FLUTAS_EINVAL, "projection: cbcvel given without bcvel");
    if (nh_u > 4 || pl->nh_d < nh_u) return fail(FLUTAS_EINVAL, "projection: bad nh_u for bounduvw");
  }
  const int nx = pl->n[0], ny = pl->n[1], nz = pl->n[2], nh_d = pl->nh_d;
  cudaStream_t st = pl->stream;
  pl->mir.reset();
  const size_t ub = sizeof(double) * (size_t)(nx + 2 * nh_u) * (ny + 2 * nh_u) * (nz + 2 * nh_u);
  const size_t pb = sizeof(double) * (size_t)(nx + 2) * (ny + 2) * (nz + 2);
  Staged su, sv, sw, sp, sci, sfi, sr, so;
  // host arrays: copied in z-slabs behind which the first pass runs, when the form allows it
  SlabIn sl;
  const void *hosts[6] = {u, v, w, p, rho, pold};
  const bool slab = precision == 1 && slab_plan(pl, nh_u, dxi, dyi, cbcvel, bcvel, hosts, &sl);
  TRY(stage_in(pl->mir, u, ub, true, true, st, &su, !slab));
  TRY(stage_in(pl->mir, v, ub, true, true, st, &sv, !slab));
  TRY(stage_in(pl->mir, w, ub, true, true, st, &sw, !slab));
  TRY(stage_in(pl->mir, p, pb, true, true, st, &sp, !slab));
  TRY(stage_in(pl->mir, dzci, sizeof(double) * (nz + 2 * nh_d), true, false, st, &sci));
  TRY(stage_in(pl->mir, dzfi, sizeof(double) * (nz + 2 * nh_d), true, false, st, &sfi));
  if (rho) {
    TRY(stage_in(pl->mir, rho, pb, true, false, st, &sr, !slab));
    TRY(stage_in(pl->mir, pold, pb, true, true, st, &so, !slab));  // in: p^(n-1); out: p^n
  }
  if (slab) {
    const Staged *fs[6] = {&su, &sv, &sw, &sp, &sr, &so};
    const int order[6] = {3, 4, 5, 0, 1, 2};  // p, rho, pold, u, v whole; w last, in slabs
    for (int i = 0; i < 6; i++) {
      const int q = order[i];
      if (q >= 4 && !rho) continue;
      sl.f[sl.nf++] = SlabIn::Field{fs[q]->host, fs[q]->d, q < 3 ? nh_u : 1, q == 2};
    }
    sl.ga.f[0] = su.d; sl.ga.f[1] = sv.d; sl.ga.f[2] = sw.d;
  }
  int rc = projection_dev(pl, nh_u, dxi, dyi, sci.d, sfi.d, dt, rho0, su.d, sv.d, sw.d, sp.d, precision, tol,
                          max_iter, rho ? sr.d : nullptr, rho ? so.d : nullptr, f_t12_o, cbcvel, bcvel,
                          rho ? &so : nullptr, slab ? &sl : nullptr, &su);
  if (rc != 0 && rc != FLUTAS_EITER) {
    if (pl->copy_stream) cudaStreamSynchronize(pl->copy_stream);  // no copy into the caller's array after return
    return rc;
  }
  TRY(stage_out(su, st));
  TRY(stage_out(sv, st));
  TRY(stage_out(sw, st));
  TRY(stage_out(sp, st));
  if (rho) TRY(stage_out(so, st));
  if (su.host || sp.host || (rho && so.host)) CK(cudaStreamSynchronize(st));
  TRY(finish(pl));
  if (precision == 0) TRY(check_nonfinite(pl, "projection"));
  return rc;
}

}  // namespace

extern "C" {

int flutas_gb300_projection(void *plan, int nh_u, double dxi, double dyi, const double *dzci, const double *dzfi,
                            const double bcpre[6], const char *cbcvel, const double *bcvel, double dt, double rho0,
                            double *u, double *v, double *w, double *p, int precision, double tol, int max_iter) {
  // fillps -> updt_rhs_b -> solver -> boundp -> correc -> p = pold + p -> boundp
  // (src/apps/single_phase/main__single_phase.f90:705-747)
  return projection_entry(plan, nh_u, dxi, dyi, dzci, dzfi, bcpre, dt, rho0, u, v, w, p, precision, tol, max_iter,
                          nullptr, nullptr, 0.0, cbcvel, bcvel);
}

int flutas_gb300_projection_df(void *plan, int nh_u, double dxi, double dyi, const double *dzci,
                               const double *dzfi, const double bcpre[6], const char *cbcvel,
                               const double *bcvel, double f_t12, double f_t12_o,
                               double rho0, const double *rho, double *pold, double *u, double *v,
                               double *w, double *p, int precision, double tol, int max_iter) {
  // pres_tw_src (src/source.f90:247-309) then the projection of
  // src/apps/two_phase_inc_isot/main__two_phase_inc_isot.f90:624,655-716
  if (!rho || !pold) return fail(FLUTAS_EINVAL, "projection_df: null rho/pold");
  if (f_t12_o == 0.0) return fail(FLUTAS_EINVAL, "projection_df: f_t12_o == 0");
  return projection_entry(plan, nh_u, dxi, dyi, dzci, dzfi, bcpre, f_t12, rho0, u, v, w, p, precision, tol,
                          max_iter, rho, pold, f_t12_o, cbcvel, bcvel);
}

int flutas_gb300_last_solve(void *plan, double *relres, int *iters) {
  flutas_plan *pl;
  TRY(check_plan(plan, &pl));
  if (relres) *relres = pl->last_relres;
  if (iters) *iters = pl->last_iters;
  return FLUTAS_OK;
}

}  // extern "C"


extern "C" {

int flutas_gb300_launch_count(unsigned long long *count) {
  if (!count) return fail(FLUTAS_EINVAL, "launch_count: null");
  *count = g_launches.load();
  return FLUTAS_OK;
}

int flutas_gb300_profile(int enable) {
  std::lock_guard<std::mutex> lk(g_prof.mu);
  g_prof.on = enable != 0;
  return FLUTAS_OK;
}

int flutas_gb300_profile_report(char *buf, int len, int reset) {
  if (!buf || len <= 0) return fail(FLUTAS_EINVAL, "profile_report: bad buffer");
  std::lock_guard<std::mutex> lk(g_prof.mu);
  std::map<std::string, std::pair<long, double>> agg;
  for (auto &r : g_prof.recs) {
    float ms = 0.f;
    CK(cudaEventSynchronize(r.b));
    CK(cudaEventElapsedTime(&ms, r.a, r.b));
    auto &e = agg[r.name];
    e.first += 1;
    e.second += ms;
  }
  std::string out;
  char line[256];
  for (auto &kv : agg) {
    snprintf(line, sizeof line, "%s %ld %.6f\n", kv.first.c_str(), kv.second.first, kv.second.second);
    out += line;
  }
  snprintf(buf, (size_t)len, "%s", out.c_str());
  if (reset) {
    for (auto &r : g_prof.recs) {
      g_prof.pool.push_back(r.a);
      g_prof.pool.push_back(r.b);
    }
    g_prof.recs.clear();
  }
  return (int)out.size() < len ? FLUTAS_OK : FLUTAS_EINVAL;
}

}  // extern "C"

// ===========================================================================
// Divergence check that allocates nothing.
//
// Scratch: one (sum, max) pair per (j,k) row of cells, kept in a file-scope
// device array of FLUTAS_NOALLOC_MAX_ROWS rows (1 MiB), which every GPU that
// loads this library holds until the process exits.  Host code must not pass
// the array's name to a kernel (on the host it is only a stand-in); the
// device address is looked up once per device with cudaGetSymbolAddress.
// ===========================================================================
#define FLUTAS_NOALLOC_MAX_ROWS 65536
static __device__ __align__(256) double g_noalloc_rows[2 * FLUTAS_NOALLOC_MAX_ROWS];

namespace {

// One block per (j,k) row (grid-stride): the row's divergence sum and max |div|
// go to rows[2r], rows[2r+1].  Every row is written, so nothing needs clearing.
__global__ void k_chkdiv_rows(DivArgs a, double *rows) {
  const Geo &g = a.g;
  const long nrow = (long)g.ny * g.nz;
  __shared__ double s_tot[32], s_mx[32];
  for (long r = blockIdx.x; r < nrow; r += gridDim.x) {
    const int j = (int)(r % g.ny) + 1, k = (int)(r / g.ny) + 1;
    double tot = 0.0, mx = 0.0;
    for (int i = threadIdx.x + 1; i <= g.nx; i += blockDim.x) {
      const double div = (a.w[g.uidx(i, j, k)] - a.w[g.uidx(i, j, k - 1)]) * a.dzfi[k] +
                         (a.v[g.uidx(i, j, k)] - a.v[g.uidx(i, j - 1, k)]) * a.dyi +
                         (a.u[g.uidx(i, j, k)] - a.u[g.uidx(i - 1, j, k)]) * a.dxi;
      tot += div;
      mx = fmax(mx, fabs(div));
    }
    for (int o = 16; o > 0; o >>= 1) {
      tot += __shfl_down_sync(0xffffffffu, tot, o);
      mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) { s_tot[wid] = tot; s_mx[wid] = mx; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0, m = 0.0;
      for (int q = 0; q < nw; q++) { t += s_tot[q]; m = fmax(m, s_mx[q]); }
      rows[2 * r] = t;
      rows[2 * r + 1] = m;
    }
    __syncthreads();
  }
}

// One block: fixed-order reduction of the row pairs into rows[0], rows[1].
__global__ void k_chkdiv_rows_reduce(double *rows, long nrow) {
  __shared__ double s_tot[1024], s_mx[1024];
  double t = 0.0, m = 0.0;
  for (long r = threadIdx.x; r < nrow; r += blockDim.x) {
    t += rows[2 * r];
    m = fmax(m, rows[2 * r + 1]);
  }
  s_tot[threadIdx.x] = t;
  s_mx[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      s_tot[threadIdx.x] += s_tot[threadIdx.x + s];
      s_mx[threadIdx.x] = fmax(s_mx[threadIdx.x], s_mx[threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    rows[0] = s_tot[0];
    rows[1] = s_mx[0];
  }
}

std::mutex g_noalloc_mu;
bool g_noalloc_ready[64] = {};

// Set-up of the allocation-free check on the current device, once per device:
// loads both kernels (under CUDA's lazy module loading a kernel is otherwise
// loaded, and its code and the module's device arrays allocated, at its first
// launch) and checks that the scratch array's address resolves.  initsolver
// runs it too, so an application that created a plan has it done already.
int noalloc_prepare() {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(FLUTAS_EUNSUPPORTED, "chkdiv_noalloc: device index %d above 63", dev);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (g_noalloc_ready[dev]) return 0;
  cudaFuncAttributes fa;
  CK(cudaFuncGetAttributes(&fa, k_chkdiv_rows));
  CK(cudaFuncGetAttributes(&fa, k_chkdiv_rows_reduce));
  void *p = nullptr;
  CK(cudaGetSymbolAddress(&p, g_noalloc_rows));
  g_noalloc_ready[dev] = true;
  return 0;
}

// Device address of g_noalloc_rows in the current context.  Looked up on
// every call (a table lookup once the module is loaded), so a context that
// was torn down and re-created (cudaDeviceReset) never leaves a stale address.
int noalloc_rows(double **out) {
  TRY(noalloc_prepare());
  void *p = nullptr;
  CK(cudaGetSymbolAddress(&p, g_noalloc_rows));
  *out = (double *)p;
  return 0;
}

}  // namespace

extern "C" {

int flutas_gb300_chkdiv_noalloc(int nx, int ny, int nz, double dxi, double dyi, double dzi, int nh_d, int nh_u,
                                const double *dzfi, const double *u, const double *v, const double *w,
                                double *divtot, double *divmax) {
  (void)dzi;
  if (!divtot || !divmax || !dzfi || !u || !v || !w) return fail(FLUTAS_EINVAL, "chkdiv_noalloc: null argument");
  if (nx < 1 || ny < 1 || nz < 1 || nh_u < 1 || nh_d < 1) return fail(FLUTAS_EINVAL, "chkdiv_noalloc: bad sizes");
  if ((long)ny * nz > FLUTAS_NOALLOC_MAX_ROWS)
    return fail(FLUTAS_EINVAL, "chkdiv_noalloc: ny*nz = %ld exceeds the %d rows of its fixed scratch",
                (long)ny * nz, FLUTAS_NOALLOC_MAX_ROWS);
  for (const void *q : {(const void *)u, (const void *)v, (const void *)w, (const void *)dzfi}) {
    const int kind = ptr_kind(q);
    if (kind == PTR_OTHER_DEVICE) return reject_other_device("chkdiv_noalloc", q);
    if (kind != PTR_DEVICE)
      return fail(FLUTAS_EINVAL, "chkdiv_noalloc: u, v, w and dzfi must be device (or managed) memory");
  }
  double *rows = nullptr;
  TRY(noalloc_rows(&rows));
  DivArgs da;
  da.u = u; da.v = v; da.w = w; da.dzfi = dzfi + (nh_d - 1);
  da.dxi = dxi; da.dyi = dyi;
  da.g = Geo{nx, ny, nz, nh_u};
  const long nrow = (long)ny * nz;
  const int grid = (int)std::min<long>(nrow, (long)num_sms() * 16);
  k_chkdiv_rows<<<grid, 128, 0, 0>>>(da, rows);
  CK(cudaGetLastError());
  k_chkdiv_rows_reduce<<<1, 1024, 0, 0>>>(rows, nrow);
  CK(cudaGetLastError());
  g_launches.fetch_add(2, std::memory_order_relaxed);
  double res[2];
  CK(cudaMemcpy(res, rows, sizeof res, cudaMemcpyDeviceToHost));
  *divtot = res[0];
  *divmax = res[1];
  return FLUTAS_OK;
}

}  // extern "C"

// ===========================================================================
// Batched solves (many independent grids of uneven sizes and BCs)
// ===========================================================================
struct flutas_batch {
  static constexpr unsigned MAGIC = 0xBA7C4u;
  unsigned magic = MAGIC;
  int ng = 0;
  std::vector<void *> plans;  // one plan per grid (tables, coefficients)
  DBuf arena;                 // x, f (FP64 halo), S, S2 (FP32) of every grid
  std::vector<double *> x;    // device halo arrays handed to the caller
  DBuf d_grids, d_prefix, d_counters, d_nrm, d_active, d_relres, d_iters;
  DBuf d_act, d_ids, d_nslots;  // compacted work lists of the grids still refining
  // the persistent kernel's queue: tile totals (z tiles of 256 columns), passes, counts, norms, error flags
  DBuf p_prefix, p_type, p_iter, p_off, p_start, p_done, p_pdone, p_nrm, p_err;
  std::vector<BatchGrid> grids;
  size_t smem_x = 0, smem_y = 0, smem_z = 0, smem_p = 0, smem_pl0 = 0, smem_pl1 = 0, smem_xr = 0, smem_yr = 0;
  int grid_x = 0, grid_y = 0, grid_z = 0, grid_p = 0, grid_pl0 = 0, grid_pl1 = 0;
  bool planes0 = false, planes1 = false;  // some grids take the whole-plane kernels (small / large planes)
  bool per_pass = true;   // false (FLUTAS_GB300_BATCH_PERSISTENT=1): the whole refinement in one persistent kernel
  int chunk = 4;          // FLUTAS_GB300_BATCH_CHUNK: items a block takes from the queue at once
  bool stats = false;     // FLUTAS_GB300_BATCH_STATS=1: queue statistics and per-pass-type timers
  cudaStream_t stream = nullptr;
  cudaGraphExec_t exec = nullptr;
  double g_tol = -1.0;
  int g_maxit = -1;
  int nodes = 0;
  std::string report;
};

namespace {

// ------------------------------------------------------------- autotuner
// Picks, per (axis length, BC pair, other-axis length), the radix cap of the
// FP32 transform plan and the tile shape of its pass (rows per x tile, columns
// per y tile) by timing the candidates on scratch data with CUDA events.
struct TuneKey {
  int pass, n, pair, other;
  bool operator<(const TuneKey &o) const {
    return std::tie(pass, n, pair, other) < std::tie(o.pass, o.n, o.pair, o.other);
  }
};
struct TuneVal {
  int maxe, tile;
  float ms;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneVal> g_tune;

size_t smem_xpass(int nx, int M) { return align_up<float>(sizeof(float) * (size_t)M * xpitch(nx)) + sizeof(float) * (size_t)M * nx; }
size_t smem_ypass(int ny, int W) { return align_up<float>(sizeof(float) * (size_t)W * ny) + sizeof(float) * (size_t)W * ny; }

int build_axis32(int n, int pair, int maxe, AxisTables *t) {
  AxisPlan ap{};
  std::vector<C2<float>> W, Q;
  if (fill_axis_tables<float>(n, pair, &ap, W, Q) != 0) return fail(FLUTAS_EUNSUPPORTED, "axis of length %d not supported", n);
  if (ap.N > 1) {
    const int ns = make_radix_plan(ap.N, ap.radix, maxe);
    if (ns < 0) return fail(FLUTAS_EUNSUPPORTED, "axis of length %d not supported", n);
    ap.nst = ns;
  }
  TRY(t->W.ensure(sizeof(C2<float>) * W.size()));
  TRY(t->Q.ensure(sizeof(C2<float>) * Q.size()));
  CK(cudaMemcpy(t->W.p, W.data(), sizeof(C2<float>) * W.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(t->Q.p, Q.data(), sizeof(C2<float>) * Q.size(), cudaMemcpyHostToDevice));
  ap.W = t->W.p;
  ap.Q = t->Q.p;
  t->ap = ap;
  t->ok = true;
  return 0;
}

// pass 0: x pass over (n = nx, other = ny*nz rows); pass 1: y pass (n = ny, other = nx*nz)
int autotune(int pass, int n, int pair, int other, size_t smem_budget, TuneVal *out, bool enabled) {
  TuneKey key{pass, n, pair, enabled ? other : -1};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) { *out = it->second; return 0; }
  }
  std::vector<int> tiles;
  for (int t : {4, 8, 16, 32, 64}) {
    const size_t sm = pass == 0 ? smem_xpass(n, t) : smem_ypass(n, t);
    if (sm <= smem_budget) tiles.push_back(t);
  }
  if (tiles.empty()) return fail(FLUTAS_EUNSUPPORTED, "axis of length %d does not fit the tile budget", n);
  TuneVal best{4, tiles.size() > 2 ? tiles[2] : tiles.back(), 0.f};
  if (enabled) {
    // scratch problem: `other` lines of length n (capped): FP64 input, FP32 output
    const long lines = std::max<long>(2, std::min<long>(other, 1L << 15));
    DBuf buf, in64;
    TRY(buf.ensure(sizeof(float) * (size_t)n * lines + 256));
    TRY(in64.ensure(sizeof(double) * (size_t)n * lines + 256));
    CK(cudaMemset(buf.p, 0, sizeof(float) * (size_t)n * lines));
    CK(cudaMemset(in64.p, 0, sizeof(double) * (size_t)n * lines));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float best_ms = 1e30f;
    for (int maxe : {4, 3}) {
      AxisTables t;
      if (build_axis32(n, pair, maxe, &t) != 0) continue;
      for (int tile : tiles) {
        float ms = 0.f;
        for (int rep = 0; rep < 3; rep++) {
          if (pass == 0) {
            const Geo g{n, (int)lines, 1, 1};
            const size_t sm = smem_xpass(n, tile);
            int grid = grid_for(k_xfwd<float, InPlain>, 256, sm, (lines + tile - 1) / tile);
            if (grid < 0) break;
            const InPlain in{(const double *)in64.p, g};
            CK(cudaEventRecord(e0));
            k_xfwd<float, InPlain><<<grid, 256, sm>>>(t.ap, in, (float *)buf.p, g, tile, nullptr);
            CK(cudaEventRecord(e1));
          } else {
            Geo g{(int)std::min<long>(lines, 4096), n, 1, 1};
            const size_t sm = smem_ypass(n, tile);
            int grid = grid_for(k_ypass<float, false>, 256, sm, (g.nx + tile - 1) / tile);
            if (grid < 0) break;
            CK(cudaEventRecord(e0));
            k_ypass<float, false><<<grid, 256, sm>>>(t.ap, (float *)buf.p, g, tile);
            CK(cudaEventRecord(e1));
          }
          CK(cudaEventSynchronize(e1));
          float m = 0.f;
          CK(cudaEventElapsedTime(&m, e0, e1));
          if (rep > 0) ms += m;
        }
        if (ms > 0.f && ms < best_ms) {
          best_ms = ms;
          best = TuneVal{maxe, tile, ms};
        }
      }
      t.W.release();
      t.Q.release();
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    buf.release();
    in64.release();
  }
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = best;
  *out = best;
  return 0;
}

int check_batch(void *b, flutas_batch **out) {
  flutas_batch *bt = (flutas_batch *)b;
  if (!bt || bt->magic != flutas_batch::MAGIC) return fail(FLUTAS_EINVAL, "invalid batch handle");
  *out = bt;
  return 0;
}

void batch_free(flutas_batch *bt) {
  if (bt->exec) cudaGraphExecDestroy(bt->exec);
  for (void *p : bt->plans) {
    void *arr[4] = {p, nullptr, nullptr, nullptr};
    if (p) flutas_gb300_fftend(arr);
  }
  DBuf *bufs[] = {&bt->arena, &bt->d_grids, &bt->d_prefix, &bt->d_counters, &bt->d_nrm, &bt->d_active,
                  &bt->d_relres, &bt->d_iters, &bt->d_act, &bt->d_ids, &bt->d_nslots, &bt->p_prefix,
                  &bt->p_type, &bt->p_iter, &bt->p_off, &bt->p_start, &bt->p_done, &bt->p_pdone, &bt->p_nrm,
                  &bt->p_err};
  for (DBuf *d : bufs) d->release();
  if (bt->stream) cudaStreamDestroy(bt->stream);
  bt->magic = 0;
  delete bt;
}

// The whole refinement as one persistent kernel (kb_persist) and the read-out
// of the per-grid residuals (kb_finalize), after the resets of the queue.
int batch_capture_persistent(flutas_batch *bt, double tol, int max_iter) {
  const int ng = bt->ng;
  std::vector<int> ptype, piter;
  auto add = [&](int t, int it) { ptype.push_back(t); piter.push_back(it); };
  add(PB_XF0, 0); add(PB_Y, 0); add(PB_Z, 0); add(PB_YI, 0); add(PB_XI0, 0);
  for (int it = 1; it <= max_iter; it++) {
    add(PB_XR, it);
    if (it < max_iter) { add(PB_Y, it); add(PB_Z, it); add(PB_YI, it); add(PB_XI1, it); }
  }
  const int npass = (int)ptype.size();
  std::vector<long> pre(3 * (size_t)(ng + 1));
  CK(cudaMemcpy(pre.data(), bt->p_prefix.p, sizeof(long) * pre.size(), cudaMemcpyDeviceToHost));
  std::vector<long> poff(npass + 1, 0);
  for (int p = 0; p < npass; p++) poff[p + 1] = poff[p] + pre[(size_t)pass_kind(ptype[p]) * (ng + 1) + ng];
  if (poff[npass] >= (1L << 31) - 1) return fail(FLUTAS_EUNSUPPORTED, "batch: too many work items");
  std::vector<int> pstart((size_t)npass * ng + 1);
  for (int p = 0; p < npass; p++)
    for (int g = 0; g < ng; g++) pstart[(size_t)p * ng + g] = (int)(poff[p] + pre[(size_t)pass_kind(ptype[p]) * (ng + 1) + g]);
  pstart[(size_t)npass * ng] = (int)poff[npass];
  TRY(bt->p_start.ensure(sizeof(int) * pstart.size()));
  TRY(bt->p_pdone.ensure(sizeof(int) * npass));
  CK(cudaMemcpy(bt->p_start.p, pstart.data(), sizeof(int) * pstart.size(), cudaMemcpyHostToDevice));
  TRY(bt->p_type.ensure(sizeof(int) * npass));
  TRY(bt->p_iter.ensure(sizeof(int) * npass));
  TRY(bt->p_off.ensure(sizeof(long) * (npass + 1)));
  TRY(bt->p_done.ensure(sizeof(int) * (size_t)npass * ng));
  TRY(bt->p_nrm.ensure(sizeof(double) * (size_t)ng * (max_iter + 1)));
  TRY(bt->p_err.ensure(sizeof(int) * 4 + sizeof(unsigned long long) * 12));  // flags, counter; queue statistics
  CK(cudaMemcpy(bt->p_type.p, ptype.data(), sizeof(int) * npass, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(bt->p_iter.p, piter.data(), sizeof(int) * npass, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(bt->p_off.p, poff.data(), sizeof(long) * (npass + 1), cudaMemcpyHostToDevice));
  PersistArgs a;
  a.grids = bt->d_grids.as<BatchGrid>();
  a.ng = ng;
  a.prefix = bt->p_prefix.as<long>();
  a.ptype = bt->p_type.as<int>();
  a.piter = bt->p_iter.as<int>();
  a.poff = bt->p_off.as<long>();
  a.npass = npass;
  a.chunk = bt->chunk;
  a.pstart = bt->p_start.as<int>();
  a.pass_done = bt->p_pdone.as<int>();
  a.err = bt->p_err.as<int>();
  a.counter = a.err + 2;
  a.done = bt->p_done.as<int>();
  a.nrm = bt->p_nrm.as<double>();
  a.stride = max_iter + 1;
  a.tol = tol;
  a.max_iter = max_iter;
  a.spin_limit = 1L << 25;  // polls of about 100 ns: a few seconds
  a.stats = bt->stats ? (unsigned long long *)(a.err + 4) : nullptr;
  auto kern = kb_persist;
  int per_sm = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, bt->smem_p));
  if (per_sm < 1) return fail(FLUTAS_EUNSUPPORTED, "batch: the persistent kernel does not fit an SM");
  bt->grid_p = (int)std::min<long>(poff[npass], (long)per_sm * num_sms());
  cudaStream_t st = bt->stream;
  cudaGraph_t graph = nullptr;
  CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  cudaMemsetAsync(a.err, 0, sizeof(int) * 4 + sizeof(unsigned long long) * 12, st);  // flags, counter, statistics
  cudaMemsetAsync(a.done, 0, sizeof(int) * (size_t)npass * ng, st);
  cudaMemsetAsync(a.pass_done, 0, sizeof(int) * npass, st);
  cudaMemsetAsync(a.nrm, 0, sizeof(double) * (size_t)ng * (max_iter + 1), st);
  kern<<<bt->grid_p, 256, bt->smem_p, st>>>(a);
  kb_finalize<<<(ng + 255) / 256, 256, 0, st>>>(a, bt->d_relres.as<double>(), bt->d_iters.as<int>());
  cudaError_t e = cudaStreamEndCapture(st, &graph);
  if (e != cudaSuccess) return fail(FLUTAS_ECUDA, "batch graph capture failed: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(&bt->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return fail(FLUTAS_ECUDA, "batch graph instantiation failed: %s", cudaGetErrorString(e));
  bt->g_tol = tol;
  bt->g_maxit = max_iter;
  bt->nodes = 2;
  return 0;
}

int batch_capture(flutas_batch *bt, double tol, int max_iter) {
  if (bt->exec) {
    cudaGraphExecDestroy(bt->exec);
    bt->exec = nullptr;
  }
  if (!bt->per_pass) return batch_capture_persistent(bt, tol, max_iter);
  const int ng = bt->ng;
  const int npass = 9 + 9 * max_iter;  // queue counters: up to 9 work-queue launches per iteration
  TRY(bt->d_counters.ensure(sizeof(int) * npass));
  BatchGrid *dg = bt->d_grids.as<BatchGrid>();
  const long *full = bt->d_prefix.as<long>();
  long *act = bt->d_act.as<long>();
  const long *px = act, *py = px + (ng + 1), *pz = py + (ng + 1), *pq0 = pz + (ng + 1), *pq1 = pq0 + (ng + 1);
  int *ids = bt->d_ids.as<int>(), *nslots = bt->d_nslots.as<int>();
  int *cnt = bt->d_counters.as<int>();
  double *relres = bt->d_relres.as<double>();
  int *iters = bt->d_iters.as<int>();
  cudaStream_t st = bt->stream;
  cudaGraph_t graph = nullptr;
  int nodes = 0, c = 0;
  CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  auto Q = [&](const long *pre) { return BatchQueue{dg, pre, ids, nslots, cnt + (c++)}; };
  auto compact = [&] {
    kb_compact<<<1, 1024, 0, st>>>(dg, ng, full, act, ids, nslots);
    nodes++;
  };
  auto fwd_chain = [&](int xmode, int outmode) {
    kb_xfwd<<<bt->grid_x, 256, bt->smem_x, st>>>(Q(px), xmode);
    nodes++;
    if (bt->planes0) {  // both transforms of the planes that fit one CTA
      kb_xyfwd_plane<256><<<bt->grid_pl0, 256, bt->smem_pl0, st>>>(Q(pq0), xmode);
      nodes++;
    }
    if (bt->planes1) {
      kb_xyfwd_plane<512><<<bt->grid_pl1, 512, bt->smem_pl1, st>>>(Q(pq1), xmode);
      nodes++;
    }
    (void)outmode;
  };
  auto rest_chain = [&](int outmode) {
    kb_ypass<false><<<bt->grid_y, 256, bt->smem_y, st>>>(Q(py));
    kb_z<<<bt->grid_z, 128, bt->smem_z, st>>>(Q(pz));
    kb_ypass<true><<<bt->grid_y, 256, bt->smem_y, st>>>(Q(py));
    kb_xinv<<<bt->grid_x, 256, bt->smem_x, st>>>(Q(px), outmode);
    nodes += 4;
    if (bt->planes0) {
      kb_xyinv_plane<256><<<bt->grid_pl0, 256, bt->smem_pl0, st>>>(Q(pq0), outmode);
      nodes++;
    }
    if (bt->planes1) {
      kb_xyinv_plane<512><<<bt->grid_pl1, 512, bt->smem_pl1, st>>>(Q(pq1), outmode);
      nodes++;
    }
  };
  cudaMemsetAsync(cnt, 0, sizeof(int) * npass, st);
  kb_reset<<<(ng + 255) / 256, 256, 0, st>>>(dg, ng);
  nodes += 1;
  compact();
  fwd_chain(0, 0);
  rest_chain(0);
  for (int it = 1; it <= max_iter; it++) {
    fwd_chain(1, 1);
    kb_update<<<(ng + 255) / 256, 256, 0, st>>>(dg, ng, tol, it, max_iter, relres, iters);
    nodes++;
    if (it < max_iter) compact();
    if (it < max_iter) rest_chain(1);
  }
  cudaError_t e = cudaStreamEndCapture(st, &graph);
  if (e != cudaSuccess) return fail(FLUTAS_ECUDA, "batch graph capture failed: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(&bt->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return fail(FLUTAS_ECUDA, "batch graph instantiation failed: %s", cudaGetErrorString(e));
  bt->g_tol = tol;
  bt->g_maxit = max_iter;
  bt->nodes = nodes;
  return 0;
}

}  // namespace

extern "C" {

int flutas_gb300_batch_create(int ngrids, const int *n, const double *dli, int nh_d, const double *const *dzci,
                              const double *const *dzfi, const char *cbc, int autotune_tiles, void **batch) {
  if (ngrids < 1 || !n || !dli || !dzci || !dzfi || !cbc || !batch) return fail(FLUTAS_EINVAL, "batch_create: bad arguments");
  flutas_batch *bt = new flutas_batch();
  bt->ng = ngrids;
  auto bail = [&](int rc) { batch_free(bt); return rc; };
  int rc = 0;
  if (cudaStreamCreateWithFlags(&bt->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(FLUTAS_ECUDA, "batch_create: stream creation failed"));
  bt->plans.assign(ngrids, nullptr);
  bt->grids.resize(ngrids);
  if (const char *e = getenv("FLUTAS_GB300_BATCH_PERSISTENT")) bt->per_pass = atoi(e) == 0;
  // pass-kernel form: grids whose planes fit one CTA transform a whole plane per item
  // (FLUTAS_GB300_BATCH_PLANES=0: row and column tiles for every grid)
  bool use_planes = true;
  if (const char *e = getenv("FLUTAS_GB300_BATCH_PLANES")) use_planes = atoi(e) != 0;
  // largest plane (nx*ny) taken whole: every plane that fits one CTA's shared memory (512 grids
  // of 32..192: 65.2 ms a batch against 66.8 ms with 144^2 as the limit and 85.5 ms without)
  long plane_max = 1L << 30;
  size_t small_plane = 60 * 1024;  // planes up to this shared memory: 256 threads, two CTAs a SM
  if (const char *e = getenv("FLUTAS_GB300_BATCH_SMALL_PLANE")) small_plane = (size_t)atol(e);
  if (const char *e = getenv("FLUTAS_GB300_BATCH_PLANE_MAX")) plane_max = atol(e);
  const size_t budget = 96 * 1024;
  // plans and tile choices
  std::vector<size_t> sx(ngrids), sf(ngrids), sS(ngrids), sS2(ngrids);
  size_t total = 0;
  auto take = [&](size_t bytes) { size_t o = total; total += (bytes + 255) & ~(size_t)255; return o; };
  std::vector<long> tx(ngrids), ty(ngrids), tz(ngrids), tp0(ngrids), tp1(ngrids), txr(ngrids), tyr(ngrids);
  std::ostringstream rep;
  for (int g = 0; g < ngrids; g++) {
    const int *ng3 = n + 3 * g;
    const int nx = ng3[0], ny = ng3[1], nz = ng3[2];
    std::vector<double> lam((size_t)nx * ny), a(nz), b(nz), c(nz), rx(2 * (size_t)ny * nz), ry(2 * (size_t)nx * nz),
        rz(2 * (size_t)nx * ny);
    void *arr[4] = {};
    double nf = 0.0, bc6[6] = {0, 0, 0, 0, 0, 0};
    if ((rc = flutas_gb300_initsolver(ng3, dli + 3 * g, nh_d, dzci[g], dzfi[g], cbc + 6 * g, bc6, "ccc", lam.data(),
                                      a.data(), b.data(), c.data(), arr, &nf, rx.data(), ry.data(), rz.data())))
      return bail(rc);
    bt->plans[g] = arr[0];
    flutas_plan *pl = (flutas_plan *)arr[0];
    if (pl->fp64_only) return bail(fail(FLUTAS_EUNSUPPORTED, "batch_create: grid %d has an odd-length ND/DN axis "
                                                             "(the batched solve is mixed precision)", g));
    BatchGrid &G = bt->grids[g];
    G.g = Geo{nx, ny, nz, 1};
    // tuned transform plans and tiles
    TuneVal vx, vy;
    if ((rc = autotune(0, nx, pair_code(pl->cbc[0], pl->cbc[1]), ny * nz, budget, &vx, autotune_tiles != 0)) ||
        (rc = autotune(1, ny, pair_code(pl->cbc[2], pl->cbc[3]), nx * nz, budget, &vy, autotune_tiles != 0)))
      return bail(rc);
    if ((rc = build_axis32(nx, pair_code(pl->cbc[0], pl->cbc[1]), vx.maxe, &pl->tx32)) ||
        (rc = build_axis32(ny, pair_code(pl->cbc[2], pl->cbc[3]), vy.maxe, &pl->ty32)))
      return bail(rc);
    G.ax = pl->tx32.ap;
    G.ay = pl->ty32.ap;
    G.M = vx.tile;
    G.W = vy.tile;
    rep << "grid " << g << " n=" << nx << "x" << ny << "x" << nz << " cbc=" << std::string(pl->cbc, 6) << " x:maxe=" << vx.maxe
        << ",M=" << vx.tile << " y:maxe=" << vy.maxe << ",W=" << vy.tile << "\n";
    ZArgs za;
    za.nonfinite = nullptr;  // the per-grid residual norms flag non-finite values
    za.a = pl->a.as<double>(); za.b = pl->b.as<double>(); za.c = pl->c.as<double>();
    za.at = pl->a32.p; za.bt = pl->b32.p; za.ct = pl->c32.p;
    za.lam = pl->lam.as<double>();
    za.nq = nx * ny;
    za.nz = nz;
    za.nn = nz;
    za.periodic = (pl->cbc[4] == 'P' && pl->cbc[5] == 'P') ? 1 : 0;
    const bool zsing = (pl->cbc[4] == 'N' && pl->cbc[5] == 'N') || za.periodic;
    za.pin = zsing ? 1 : 0;
    G.za = za;
    G.zres = pl->zres.as<double>();
    G.dxi2 = pl->dli[0] * pl->dli[0];
    G.dyi2 = pl->dli[1] * pl->dli[1];
    G.normfft = pl->normfft;
    memcpy(G.bc, pl->cbc, 6);
    const size_t halo = sizeof(double) * (size_t)(nx + 2) * (ny + 2) * (nz + 2);
    sx[g] = take(halo);
    sf[g] = take(halo);
    sS[g] = take(sizeof(float) * (size_t)nx * ny * nz);
    sS2[g] = za.periodic ? take(sizeof(float) * (size_t)nx * ny * nz) : (size_t)-1;
    txr[g] = ((long)ny * nz + G.M - 1) / G.M;  // row tiles (the persistent form: every grid)
    tyr[g] = (long)((nx + G.W - 1) / G.W) * nz;
    // whole planes where one fits a CTA
    const size_t psm = plane_smem<float>(nx, ny);
    G.plane = (use_planes && bt->per_pass && nx % 2 == 0 && ny % 2 == 0 && (long)nx * ny <= plane_max &&
               (int)psm <= max_smem_optin()) ? 1 : 0;
    // two classes of planes, each launched with its own shared memory: the small ones run
    // several CTAs a SM, the large ones one
    const bool small = psm <= small_plane;
    tx[g] = G.plane ? 0 : txr[g];
    ty[g] = G.plane ? 0 : tyr[g];
    tp0[g] = G.plane && small ? nz : 0;
    tp1[g] = G.plane && !small ? nz : 0;
    tz[g] = ((long)nx * ny + 127) / 128;
    if (G.plane) {
      size_t &sm = small ? bt->smem_pl0 : bt->smem_pl1;
      sm = std::max(sm, psm);
    } else {
      bt->smem_x = std::max(bt->smem_x, smem_xpass(nx, G.M));
      bt->smem_y = std::max(bt->smem_y, smem_ypass(ny, G.W));
    }
    bt->smem_xr = std::max(bt->smem_xr, smem_xpass(nx, G.M));
    bt->smem_yr = std::max(bt->smem_yr, smem_ypass(ny, G.W));
    bt->smem_z = std::max(bt->smem_z, sizeof(float) * (size_t)((nz + 15) / 16) * 128);
    if (G.plane) rep << "grid " << g << ": whole planes\n";
  }
  bt->report = rep.str();
  if ((rc = bt->arena.ensure(total))) return bail(rc);
  if (cudaMemset(bt->arena.p, 0, total) != cudaSuccess) return bail(fail(FLUTAS_ECUDA, "batch_create: memset failed"));
  if ((rc = bt->d_nrm.ensure(sizeof(double) * 2 * ngrids)) || (rc = bt->d_active.ensure(sizeof(int) * ngrids)) ||
      (rc = bt->d_relres.ensure(sizeof(double) * ngrids)) || (rc = bt->d_iters.ensure(sizeof(int) * ngrids)))
    return bail(rc);
  unsigned char *base = (unsigned char *)bt->arena.p;
  bt->x.resize(ngrids);
  for (int g = 0; g < ngrids; g++) {
    BatchGrid &G = bt->grids[g];
    G.x = (double *)(base + sx[g]);
    G.f = (double *)(base + sf[g]);
    G.S = (float *)(base + sS[g]);
    G.S2 = sS2[g] == (size_t)-1 ? nullptr : (float *)(base + sS2[g]);
    G.nrm = bt->d_nrm.as<double>() + 2 * g;
    G.active = bt->d_active.as<int>() + g;
    bt->x[g] = G.x;
  }
  std::vector<long> pre(BATCH_KINDS * (size_t)(ngrids + 1), 0);
  for (int g = 0; g < ngrids; g++) {
    const long *t[BATCH_KINDS] = {tx.data(), ty.data(), tz.data(), tp0.data(), tp1.data()};
    for (int k = 0; k < BATCH_KINDS; k++)
      pre[k * (size_t)(ngrids + 1) + g + 1] = pre[k * (size_t)(ngrids + 1) + g] + t[k][g];
  }
  if ((rc = bt->d_prefix.ensure(sizeof(long) * pre.size())) || (rc = bt->d_grids.ensure(sizeof(BatchGrid) * ngrids)) ||
      (rc = bt->d_act.ensure(sizeof(long) * pre.size())) || (rc = bt->d_ids.ensure(sizeof(int) * ngrids)) ||
      (rc = bt->d_nslots.ensure(sizeof(int))))
    return bail(rc);
  if (cudaMemcpy(bt->d_prefix.p, pre.data(), sizeof(long) * pre.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(bt->d_grids.p, bt->grids.data(), sizeof(BatchGrid) * ngrids, cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(fail(FLUTAS_ECUDA, "batch_create: upload failed"));
  if ((int)std::max({bt->smem_x, bt->smem_y, bt->smem_z, bt->smem_pl0, bt->smem_pl1}) > max_smem_optin())
    return bail(fail(FLUTAS_EUNSUPPORTED, "batch_create: tiles exceed shared memory"));
  {
    // the persistent kernel's tiles: row and column tiles for every grid, z in blocks of 256 columns
    std::vector<long> pp(3 * (size_t)(ngrids + 1), 0);
    size_t smz = 0;
    for (int g = 0; g < ngrids; g++) {
      const Geo &G = bt->grids[g].g;
      pp[g + 1] = pp[g] + txr[g];
      pp[(ngrids + 1) + g + 1] = pp[(ngrids + 1) + g] + tyr[g];
      pp[2 * (ngrids + 1) + g + 1] = pp[2 * (ngrids + 1) + g] + ((long)G.nx * G.ny + 255) / 256;
      smz = std::max(smz, sizeof(float) * (size_t)((G.nz + 15) / 16) * 256);
    }
    bt->smem_p = std::max({bt->smem_xr, bt->smem_yr, smz});
    if ((rc = bt->p_prefix.ensure(sizeof(long) * pp.size()))) return bail(rc);
    if (cudaMemcpy(bt->p_prefix.p, pp.data(), sizeof(long) * pp.size(), cudaMemcpyHostToDevice) != cudaSuccess)
      return bail(fail(FLUTAS_ECUDA, "batch_create: upload failed"));
    if ((rc = allow_smem(kb_persist))) return bail(rc);
    // the persistent kernel's own tables take about 2 KB of static shared memory besides the tiles
    // (tiles too large for it: the pass kernels run the batch, with the row and column tiles
    // chosen for the persistent form)
    if (!bt->per_pass && (int)bt->smem_p + 2048 > max_smem_optin()) bt->per_pass = true;
    if (const char *e = getenv("FLUTAS_GB300_BATCH_CHUNK")) bt->chunk = std::max(1, std::min(64, atoi(e)));
    if (const char *e = getenv("FLUTAS_GB300_BATCH_STATS")) bt->stats = atoi(e) != 0;
  }
  auto total_of = [&](int k) { return std::max<long>(1, pre[k * (size_t)(ngrids + 1) + ngrids]); };
  int g1, g2, g3, g4 = 0, g5 = 0;
  if ((g1 = grid_for(kb_xfwd, 256, bt->smem_x, total_of(0))) < 0) return bail(g1);
  if ((g2 = grid_for(kb_ypass<false>, 256, bt->smem_y, total_of(1))) < 0) return bail(g2);
  if ((g3 = grid_for(kb_z, 128, bt->smem_z, total_of(2))) < 0) return bail(g3);
  if ((rc = allow_smem(kb_xinv)) || (rc = allow_smem(kb_ypass<true>))) return bail(rc);
  bt->planes0 = pre[3 * (size_t)(ngrids + 1) + ngrids] > 0;
  bt->planes1 = pre[4 * (size_t)(ngrids + 1) + ngrids] > 0;
  if (bt->planes0 && (g4 = grid_for(kb_xyfwd_plane<256>, 256, bt->smem_pl0, total_of(3))) < 0) return bail(g4);
  if (bt->planes1 && (g5 = grid_for(kb_xyfwd_plane<512>, 512, bt->smem_pl1, total_of(4))) < 0) return bail(g5);
  if ((rc = allow_smem(kb_xyinv_plane<256>)) || (rc = allow_smem(kb_xyinv_plane<512>))) return bail(rc);
  bt->grid_x = g1;
  bt->grid_y = g2;
  bt->grid_z = g3;
  bt->grid_pl0 = g4;
  bt->grid_pl1 = g5;
  *batch = bt;
  return FLUTAS_OK;
}

int flutas_gb300_batch_field(void *batch, int g, double **p) {
  flutas_batch *bt;
  TRY(check_batch(batch, &bt));
  if (g < 0 || g >= bt->ng || !p) return fail(FLUTAS_EINVAL, "batch_field: bad grid index");
  *p = bt->x[g];
  return FLUTAS_OK;
}

int flutas_gb300_batch_solve(void *batch, double tol, int max_iter, double *relres, int *iters) {
  flutas_batch *bt;
  TRY(check_batch(batch, &bt));
  if (!(tol > 0.0) || max_iter < 1 || max_iter > 32) return fail(FLUTAS_EINVAL, "batch_solve: need tol > 0 and 1 <= max_iter <= 32");
  if (!bt->exec || bt->g_tol != tol || bt->g_maxit != max_iter) TRY(batch_capture(bt, tol, max_iter));
  CK(cudaGraphLaunch(bt->exec, bt->stream));
  g_launches.fetch_add((unsigned long long)bt->nodes, std::memory_order_relaxed);
  std::vector<double> rr(bt->ng);
  std::vector<int> it(bt->ng);
  CK(cudaMemcpyAsync(rr.data(), bt->d_relres.p, sizeof(double) * bt->ng, cudaMemcpyDeviceToHost, bt->stream));
  CK(cudaMemcpyAsync(it.data(), bt->d_iters.p, sizeof(int) * bt->ng, cudaMemcpyDeviceToHost, bt->stream));
  int perr = 0;
  if (!bt->per_pass) CK(cudaMemcpyAsync(&perr, bt->p_err.p, sizeof(int), cudaMemcpyDeviceToHost, bt->stream));
  CK(cudaStreamSynchronize(bt->stream));
  if (perr) return fail(FLUTAS_ECUDA, "batch_solve: a work item's wait for its grid's previous pass gave up");
  int rc = FLUTAS_OK;
  for (int g = 0; g < bt->ng; g++) {
    if (relres) relres[g] = rr[g];
    if (iters) iters[g] = it[g];
    if (!std::isfinite(rr[g])) rc = FLUTAS_ENONFINITE;
    else if (!(rr[g] <= tol) && rc == FLUTAS_OK) rc = FLUTAS_EITER;
  }
  if (rc == FLUTAS_ENONFINITE) fail(rc, "batch_solve: non-finite residual (NaN or Inf in a right-hand side)");
  else if (rc) fail(rc, "batch_solve: some grids did not reach tol in %d solves", max_iter);
  return rc;
}

int flutas_gb300_batch_set(void *batch, int g, const double *src) {
  flutas_batch *bt;
  TRY(check_batch(batch, &bt));
  if (g < 0 || g >= bt->ng || !src) return fail(FLUTAS_EINVAL, "batch_set: bad arguments");
  const Geo &G = bt->grids[g].g;
  const size_t bytes = sizeof(double) * (size_t)(G.nx + 2) * (G.ny + 2) * (G.nz + 2);
  CK(cudaMemcpyAsync(bt->x[g], src, bytes, cudaMemcpyDefault, bt->stream));
  CK(cudaStreamSynchronize(bt->stream));
  return FLUTAS_OK;
}

int flutas_gb300_batch_get(void *batch, int g, double *dst) {
  flutas_batch *bt;
  TRY(check_batch(batch, &bt));
  if (g < 0 || g >= bt->ng || !dst) return fail(FLUTAS_EINVAL, "batch_get: bad arguments");
  const Geo &G = bt->grids[g].g;
  const size_t bytes = sizeof(double) * (size_t)(G.nx + 2) * (G.ny + 2) * (G.nz + 2);
  CK(cudaMemcpyAsync(dst, bt->x[g], bytes, cudaMemcpyDefault, bt->stream));
  CK(cudaStreamSynchronize(bt->stream));
  return FLUTAS_OK;
}

int flutas_gb300_batch_report(void *batch, char *buf, int len) {
  flutas_batch *bt;
  TRY(check_batch(batch, &bt));
  if (!buf || len <= 0) return fail(FLUTAS_EINVAL, "batch_report: bad buffer");
  std::string r = bt->report;
  if (bt->exec && !bt->per_pass && bt->stats && bt->p_err.p) {
    // the last solve's queue: items worked, tiles skipped (converged grids), waits and their polls
    unsigned long long st[12] = {};
    CK(cudaStreamSynchronize(bt->stream));
    CK(cudaMemcpy(st, (char *)bt->p_err.p + sizeof(int) * 4, sizeof(st), cudaMemcpyDeviceToHost));
    char line[512];
    const double nb = bt->grid_p > 0 ? 1e6 * bt->grid_p : 1.0;  // ms a block, averaged over the blocks
    snprintf(line, sizeof line, "queue: %d blocks, %llu items worked, %llu tiles skipped, %llu waits, %llu polls; "
             "ms a block x0 %.2f y %.2f z %.2f yi %.2f xi0 %.2f xr %.2f xi1 %.2f sched %.2f\n", bt->grid_p, st[0],
             st[1], st[2], st[3], st[4] / nb, st[5] / nb, st[6] / nb, st[7] / nb, st[8] / nb, st[9] / nb, st[10] / nb,
             st[11] / nb);
    r += line;
  }
  snprintf(buf, (size_t)len, "%s", r.c_str());
  return FLUTAS_OK;
}

int flutas_gb300_batch_destroy(void *batch) {
  flutas_batch *bt;
  TRY(check_batch(batch, &bt));
  cudaStreamSynchronize(bt->stream);
  batch_free(bt);
  return FLUTAS_OK;
}

}  // extern "C"
