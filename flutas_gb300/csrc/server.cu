// server.cu -- continuous-batching request loop for projection solves.
//
// Requests of different sizes arrive at any time (flutas_gb300_server_submit).
// A pool of slot workers, each with its own CUDA stream, admits requests in
// arrival order as soon as a slot is free and the HBM budget covers the
// request's fields plus the resident plan it needs; admitted requests run
// concurrently, so their work overlaps on the device.  Plans (eigenvalues,
// z coefficients, twiddles and spectral scratch) stay resident between
// requests of the same grid signature and are evicted least-recently-used when
// the budget needs room.  Built only on the public C ABI of this library.
#include "../../include/flutas_gb300.h"
#include "ptrcheck.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

void fg_set_error_text(const char *msg);  // flutas_gb300.cu

namespace {

using Clock = std::chrono::steady_clock;

struct Sig {  // grid signature of a plan
  int n[3];
  double dli[3];
  int nh_d;
  std::vector<double> dzci, dzfi;
  char cbc[6];
  bool operator==(const Sig &o) const {
    return memcmp(n, o.n, sizeof n) == 0 && memcmp(dli, o.dli, sizeof dli) == 0 && nh_d == o.nh_d &&
           dzci == o.dzci && dzfi == o.dzfi && memcmp(cbc, o.cbc, 6) == 0;
  }
};

struct PlanEntry {
  Sig sig;
  void *arr[4] = {nullptr, nullptr, nullptr, nullptr};
  std::vector<double> lam, a, b, c, rx, ry, rz;
  double normfft = 0.0;
  size_t bytes = 0;   // device bytes held (updated after use)
  bool busy = false;
  Clock::time_point last;
};

struct Request {
  long long id = 0;
  flutas_request r{};
  Sig sig;
  std::vector<double> bcvel;
  std::string cbcvel;
  size_t est = 0;
  Clock::time_point t_submit, t_admit, t_done;
  bool done = false;
  int rc = 0;
  double relres = 0.0;
  int iters = 0;
  double t0 = 0.0, t1 = 0.0;  // device span (ms after the server's reference event)
  std::string err;
};

size_t cells_halo(const int n[3], int h) { return (size_t)(n[0] + 2 * h) * (n[1] + 2 * h) * (n[2] + 2 * h); }

}  // namespace

struct flutas_server {
  static constexpr unsigned MAGIC = 0x5E7E5u;
  unsigned magic = MAGIC;
  int device = 0;
  size_t budget = 0, used = 0;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Request *> queue;
  std::map<long long, std::unique_ptr<Request>> reqs;
  std::list<std::unique_ptr<PlanEntry>> plans;
  std::vector<std::thread> workers;
  bool stop = false;
  long long next_id = 1;
  int inflight = 0;
  std::vector<double> latencies;  // ms, completed requests
  Clock::time_point t_first, t_last;
  long long completed = 0;
  // device-side span of every completed request (ms after ev_ref): the stream
  // work of the request from its first copy to its last, from CUDA events
  cudaEvent_t ev_ref = nullptr;
  std::vector<std::pair<double, double>> spans;
};

namespace {

// Device memory of the current device (or managed): such arrays are used in place.
bool resident(const void *p) {
  if (!p) return false;
  cudaPointerAttributes at;
  const bool ok = cudaPointerGetAttributes(&at, p) == cudaSuccess;
  if (!ok) cudaGetLastError();
  int cur = 0;
  cudaGetDevice(&cur);
  return fg::classify_ptr(ok, ok ? (int)at.type : 0, ok ? at.device : -1, cur) == fg::PTR_DEVICE;
}

// Every field of the request already lives on the device: the request is
// solved in place, with no staging copies and no field memory of its own.
// (A two-phase projection takes the staged path: its pold is an input of the
// request, which the in-place call would overwrite with p^n.)
bool fields_resident(const flutas_request &r) {
  if (r.kind == 0) return resident(r.rhs) && resident(r.p);
  return !r.rho && resident(r.u) && resident(r.v) && resident(r.w) && resident(r.p);
}

// Device bytes a request needs besides its plan: its fields (none when they
// are resident already).
size_t field_bytes(const flutas_request &r) {
  if (fields_resident(r)) return 0;
  const size_t p = sizeof(double) * cells_halo(r.n, 1);
  if (r.kind == 0) return p;
  const size_t uvw = 3 * sizeof(double) * cells_halo(r.n, r.nh_u);
  return uvw + p + (r.rho ? 2 * p : 0);
}

// Bytes a new plan will hold once it has solved: spectral FP32 + FP64 RHS copy
// (+ increment for projections) + tables.
size_t plan_bytes_estimate(const flutas_request &r) {
  const size_t N = (size_t)r.n[0] * r.n[1] * r.n[2];
  const size_t halo = sizeof(double) * cells_halo(r.n, 1);
  return 4 * N + halo + (r.kind == 1 ? 2 * halo : 0) + 8 * N / 8 + (1 << 20);
}

PlanEntry *acquire_plan(flutas_server *s, const Sig &sig, const flutas_request &r, int *rc, std::string *err,
                        std::unique_lock<std::mutex> &lk) {
  for (auto &pe : s->plans)
    if (!pe->busy && pe->sig == sig) {
      pe->busy = true;
      return pe.get();
    }
  // new plan: build it outside the lock
  auto pe = std::make_unique<PlanEntry>();
  pe->sig = sig;
  pe->busy = true;
  PlanEntry *raw = pe.get();
  s->plans.push_back(std::move(pe));
  lk.unlock();
  const int nx = r.n[0], ny = r.n[1], nz = r.n[2];
  raw->lam.resize((size_t)nx * ny);
  raw->a.resize(nz);
  raw->b.resize(nz);
  raw->c.resize(nz);
  raw->rx.resize(2 * (size_t)ny * nz);
  raw->ry.resize(2 * (size_t)nx * nz);
  raw->rz.resize(2 * (size_t)nx * ny);
  double nf = 0.0, bc6[6] = {0, 0, 0, 0, 0, 0};
  const double *bcp = r.bcpre ? r.bcpre : bc6;
  *rc = flutas_gb300_initsolver(r.n, r.dli, r.nh_d, sig.dzci.data(), sig.dzfi.data(), sig.cbc, bcp, "ccc",
                                raw->lam.data(), raw->a.data(), raw->b.data(), raw->c.data(), raw->arr, &nf,
                                raw->rx.data(), raw->ry.data(), raw->rz.data());
  if (*rc) {
    char buf[512];
    flutas_gb300_last_error(buf, sizeof buf);
    *err = buf;
  }
  raw->normfft = nf;
  lk.lock();
  if (*rc) {
    s->plans.remove_if([&](const std::unique_ptr<PlanEntry> &p) { return p.get() == raw; });
    return nullptr;
  }
  return raw;
}

// Evict idle plans (least recently used first) until `need` more bytes fit.
void evict_for(flutas_server *s, size_t need) {
  while (s->used + need > s->budget) {
    PlanEntry *victim = nullptr;
    for (auto &pe : s->plans)
      if (!pe->busy && (!victim || pe->last < victim->last)) victim = pe.get();
    if (!victim) return;
    s->used -= std::min(s->used, victim->bytes);
    flutas_gb300_fftend(victim->arr);
    s->plans.remove_if([&](const std::unique_ptr<PlanEntry> &p) { return p.get() == victim; });
  }
}

// Largest number of request spans that overlap at one instant.
int max_overlap(std::vector<std::pair<double, double>> sp) {
  std::vector<std::pair<double, int>> ev;
  for (auto &x : sp) {
    ev.push_back({x.first, 1});
    ev.push_back({x.second, -1});
  }
  std::sort(ev.begin(), ev.end());  // at equal times the end (-1) sorts before the start
  int cur = 0, best = 0;
  for (auto &e : ev) best = std::max(best, cur += e.second);
  return best;
}

int run_request(flutas_server *s, Request *q, PlanEntry *pe, cudaStream_t st) {
  const flutas_request &r = q->r;
  void *plan = pe->arr[0];
  int rc = flutas_gb300_plan_set_stream(plan, st, 1);
  if (rc) return rc;
  struct Restore {  // every exit path hands the plan back on the default stream
    void *plan;
    ~Restore() { flutas_gb300_plan_set_stream(plan, nullptr, 1); }
  } restore{plan};
  const size_t pb = sizeof(double) * cells_halo(r.n, 1);
  auto dmalloc = [&](size_t bytes, double **out) -> int {
    if (cudaMallocAsync((void **)out, bytes, st) != cudaSuccess) {
      cudaGetLastError();
      return FLUTAS_ENOMEM;
    }
    return 0;
  };
  std::vector<double *> bufs;
  auto cleanup = [&]() {
    for (double *b : bufs) cudaFreeAsync(b, st);
    cudaStreamSynchronize(st);
  };
  const bool in_place = fields_resident(r);
  if (r.kind == 0) {
    double *x = nullptr;
    if (in_place) {  // the solution array itself holds the RHS during the solve
      x = r.p;
      if ((const double *)x != r.rhs) cudaMemcpyAsync(x, r.rhs, pb, cudaMemcpyDeviceToDevice, st);
    } else {
      if ((rc = dmalloc(pb, &x))) return rc;
      bufs.push_back(x);
      cudaMemcpyAsync(x, r.rhs, pb, cudaMemcpyDefault, st);
    }
    if (r.tol > 0.0) {
      rc = flutas_gb300_solve_mixed(plan, x, r.tol, r.max_iter, &q->relres, &q->iters);
    } else {  // tol = 0: the plain FP64 solver call (the drop-in form)
      rc = flutas_gb300_solver(r.n, pe->arr, pe->normfft, pe->lam.data(), pe->a.data(), pe->b.data(), pe->c.data(),
                               r.cbc + 4, "ccc", x);
      q->relres = 0.0;
      q->iters = 0;
    }
    if (!in_place && (rc == 0 || rc == FLUTAS_EITER)) cudaMemcpyAsync(r.p, x, pb, cudaMemcpyDefault, st);
  } else if (in_place) {
    const double bc6[6] = {0, 0, 0, 0, 0, 0};
    const double *bcp = r.bcpre ? r.bcpre : bc6;
    const char *cv = q->cbcvel.empty() ? nullptr : q->cbcvel.c_str();
    const double *bv = q->bcvel.empty() ? nullptr : q->bcvel.data();
    const int prec = r.tol > 0.0 ? 1 : 0;
    // dzci / dzfi are host arrays of the request: the projection stages them
    rc = flutas_gb300_projection(plan, r.nh_u, r.dli[0], r.dli[1], q->sig.dzci.data(), q->sig.dzfi.data(), bcp, cv,
                                 bv, r.dt, r.rho0, r.u, r.v, r.w, r.p, prec, r.tol, r.max_iter);
    if (prec) flutas_gb300_last_solve(plan, &q->relres, &q->iters);
  } else {
    const size_t ub = sizeof(double) * cells_halo(r.n, r.nh_u);
    double *u, *v, *w, *p, *rho = nullptr, *pold = nullptr;
    if ((rc = dmalloc(ub, &u)) || (bufs.push_back(u), rc = dmalloc(ub, &v)) || (bufs.push_back(v), rc = dmalloc(ub, &w)) ||
        (bufs.push_back(w), rc = dmalloc(pb, &p))) {
      cleanup();
      return rc;
    }
    bufs.push_back(p);
    if (r.rho) {
      if ((rc = dmalloc(pb, &rho)) || (bufs.push_back(rho), rc = dmalloc(pb, &pold))) {
        cleanup();
        return rc;
      }
      bufs.push_back(pold);
      cudaMemcpyAsync(rho, r.rho, pb, cudaMemcpyDefault, st);
      cudaMemcpyAsync(pold, r.pold, pb, cudaMemcpyDefault, st);
    }
    cudaMemcpyAsync(u, r.u, ub, cudaMemcpyDefault, st);
    cudaMemcpyAsync(v, r.v, ub, cudaMemcpyDefault, st);
    cudaMemcpyAsync(w, r.w, ub, cudaMemcpyDefault, st);
    cudaMemcpyAsync(p, r.p, pb, cudaMemcpyDefault, st);
    double *dzci = nullptr, *dzfi = nullptr;
    const size_t zb = sizeof(double) * (r.n[2] + 2 * r.nh_d);
    if ((rc = dmalloc(zb, &dzci)) || (bufs.push_back(dzci), rc = dmalloc(zb, &dzfi))) {
      cleanup();
      return rc;
    }
    bufs.push_back(dzfi);
    cudaMemcpyAsync(dzci, q->sig.dzci.data(), zb, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dzfi, q->sig.dzfi.data(), zb, cudaMemcpyHostToDevice, st);
    const double bc6[6] = {0, 0, 0, 0, 0, 0};
    const double *bcp = r.bcpre ? r.bcpre : bc6;
    const char *cv = q->cbcvel.empty() ? nullptr : q->cbcvel.c_str();
    const double *bv = q->bcvel.empty() ? nullptr : q->bcvel.data();
    const int prec = r.tol > 0.0 ? 1 : 0;
    if (rho)
      rc = flutas_gb300_projection_df(plan, r.nh_u, r.dli[0], r.dli[1], dzci, dzfi, bcp, cv, bv, r.dt, r.dt_old, r.rho0,
                                      rho, pold, u, v, w, p, prec, r.tol, r.max_iter);
    else
      rc = flutas_gb300_projection(plan, r.nh_u, r.dli[0], r.dli[1], dzci, dzfi, bcp, cv, bv, r.dt, r.rho0, u, v, w, p,
                                   prec, r.tol, r.max_iter);
    if (prec) flutas_gb300_last_solve(plan, &q->relres, &q->iters);
    if (rc == 0 || rc == FLUTAS_EITER) {
      cudaMemcpyAsync(r.u, u, ub, cudaMemcpyDefault, st);
      cudaMemcpyAsync(r.v, v, ub, cudaMemcpyDefault, st);
      cudaMemcpyAsync(r.w, w, ub, cudaMemcpyDefault, st);
      cudaMemcpyAsync(r.p, p, pb, cudaMemcpyDefault, st);
    }
  }
  cleanup();
  if (cudaGetLastError() != cudaSuccess && rc == 0) rc = FLUTAS_ECUDA;
  return rc;
}

void worker_main(flutas_server *s) {
  cudaSetDevice(s->device);
  cudaStream_t st = nullptr;
  cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEventCreate(&ev0);
  cudaEventCreate(&ev1);
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    // admission: the head of the queue, when the budget covers it
    Request *q = nullptr;
    s->cv.wait(lk, [&] {
      if (s->stop) return true;
      if (s->queue.empty()) return false;
      Request *h = s->queue.front();
      if (s->used + h->est <= s->budget) return true;
      evict_for(s, h->est);
      if (s->used + h->est <= s->budget) return true;
      if (s->inflight == 0) return true;  // cannot ever fit: admit to fail it below
      return false;
    });
    if (s->stop) break;
    q = s->queue.front();
    s->queue.pop_front();
    const bool fits = s->used + q->est <= s->budget;
    if (!fits) {
      q->rc = FLUTAS_ENOMEM;
      q->err = "request does not fit the HBM budget";
      q->done = true;
      q->t_done = Clock::now();
      s->cv.notify_all();
      continue;
    }
    s->used += q->est;
    s->inflight++;
    q->t_admit = Clock::now();
    int rc = 0;
    std::string err;
    PlanEntry *pe = acquire_plan(s, q->sig, q->r, &rc, &err, lk);
    if (pe) {
      lk.unlock();
      cudaEventRecord(ev0, st);
      rc = run_request(s, q, pe, st);
      cudaEventRecord(ev1, st);
      float t0 = 0.0f, t1 = 0.0f;
      const bool timed = cudaEventSynchronize(ev1) == cudaSuccess &&
                         cudaEventElapsedTime(&t0, s->ev_ref, ev0) == cudaSuccess &&
                         cudaEventElapsedTime(&t1, s->ev_ref, ev1) == cudaSuccess;
      if (!timed) cudaGetLastError();
      if (rc && rc != FLUTAS_EITER) {
        char buf[512];
        flutas_gb300_last_error(buf, sizeof buf);
        err = buf;
      }
      if (timed) {
        q->t0 = t0;
        q->t1 = t1;
      }
      size_t pbytes = 0;
      flutas_gb300_plan_info(pe->arr[0], &pbytes, nullptr, nullptr);
      lk.lock();
      // the plan stays resident: its bytes replace this request's estimate
      s->used -= std::min(s->used, q->est);
      s->used -= std::min(s->used, pe->bytes);
      pe->bytes = pbytes;
      s->used += pbytes;
      pe->busy = false;
      pe->last = Clock::now();
    } else {
      s->used -= std::min(s->used, q->est);
    }
    s->inflight--;
    q->rc = rc;
    q->err = err;
    q->t_done = Clock::now();
    q->done = true;
    const double ms = std::chrono::duration<double, std::milli>(q->t_done - q->t_submit).count();
    if (rc == 0 || rc == FLUTAS_EITER) {
      s->latencies.push_back(ms);
      s->completed++;
      s->t_last = q->t_done;
      if (q->t1 > q->t0) s->spans.push_back({q->t0, q->t1});
    }
    s->cv.notify_all();
  }
  lk.unlock();
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  cudaStreamDestroy(st);
}

int sfail(const char *msg) {
  (void)msg;
  return FLUTAS_EINVAL;
}

}  // namespace

extern "C" {

int flutas_gb300_server_create(size_t hbm_budget, int slots, void **srv) {
  if (!srv || slots < 1 || slots > 64 || hbm_budget == 0) return sfail("server_create: bad arguments");
  flutas_server *s = new flutas_server();
  cudaGetDevice(&s->device);
  if (cudaEventCreate(&s->ev_ref) != cudaSuccess || cudaEventRecord(s->ev_ref, 0) != cudaSuccess ||
      cudaEventSynchronize(s->ev_ref) != cudaSuccess) {
    cudaGetLastError();
    delete s;
    fg_set_error_text("server_create: CUDA event set-up failed");
    return FLUTAS_ECUDA;
  }
  s->budget = hbm_budget;
  s->t_first = Clock::now();
  for (int i = 0; i < slots; i++) s->workers.emplace_back(worker_main, s);
  *srv = s;
  return FLUTAS_OK;
}

int flutas_gb300_server_submit(void *srv, const flutas_request *r, long long *ticket) {
  flutas_server *s = (flutas_server *)srv;
  if (!s || s->magic != flutas_server::MAGIC || !r || !ticket) return sfail("server_submit: bad arguments");
  auto bad = [](const char *why) {
    fg_set_error_text(why);
    return FLUTAS_EINVAL;
  };
  if (r->kind != 0 && r->kind != 1) return bad("server_submit: kind must be 0 (solve) or 1 (projection)");
  if (r->kind == 0 && (!r->rhs || !r->p || !(r->tol >= 0.0))) return bad("server_submit: solve needs rhs, p, tol >= 0");
  if (r->kind == 1 && (!r->u || !r->v || !r->w || !r->p || r->nh_u < 1 || (r->rho && !r->pold)))
    return bad("server_submit: projection needs u, v, w, p, nh_u >= 1 (and pold with rho)");
  if (r->n[0] < 2 || r->n[1] < 2 || r->n[2] < 3 || r->nh_d < 1 || !r->dzci || !r->dzfi)
    return bad("server_submit: bad sizes or missing dzci/dzfi");
  if (r->n[0] > 65536 || r->n[1] > 65536 || r->n[2] > 65536 || r->nh_d > 8)
    return bad("server_submit: sizes beyond 65536 cells per axis or nh_d above 8");
  for (int i = 0; i < 6; i++)
    if (r->cbc[i] != 'P' && r->cbc[i] != 'N' && r->cbc[i] != 'D')
      return bad("server_submit: bad pressure BC character (P, N or D)");
  for (int d = 0; d < 3; d++)
    if ((r->cbc[2 * d] == 'P') != (r->cbc[2 * d + 1] == 'P'))
      return bad("server_submit: a periodic BC must be set on both ends of its axis");
  for (int d = 0; d < 3; d++)
    if (!(r->dli[d] > 0.0) || !std::isfinite(r->dli[d])) return bad("server_submit: dli must be finite and > 0");
  if (!std::isfinite(r->tol) || (r->tol > 0.0 && r->max_iter < 1))
    return bad("server_submit: tol must be finite (0: FP64) and max_iter >= 1");
  if (r->kind == 1) {
    if (r->nh_u > 4 || r->nh_u > r->nh_d) return bad("server_submit: nh_u must be <= 4 and <= nh_d");
    if (!(r->dt != 0.0) || !std::isfinite(r->dt) || !(r->rho0 > 0.0) || !std::isfinite(r->rho0) ||
        (r->rho && (!(r->dt_old != 0.0) || !std::isfinite(r->dt_old))))
      return bad("server_submit: dt (and dt_old) must be finite and non-zero, rho0 finite and > 0");
    if (r->cbcvel) {
      if (!r->bcvel) return bad("server_submit: cbcvel given without bcvel");
      for (int i = 0; i < 18; i++)
        if (r->cbcvel[i] != 'P' && r->cbcvel[i] != 'N' && r->cbcvel[i] != 'D')
          return bad("server_submit: bad velocity BC character (P, N or D)");
    }
  }
  auto q = std::make_unique<Request>();
  q->r = *r;
  memcpy(q->sig.n, r->n, sizeof q->sig.n);
  memcpy(q->sig.dli, r->dli, sizeof q->sig.dli);
  q->sig.nh_d = r->nh_d;
  q->sig.dzci.assign(r->dzci, r->dzci + r->n[2] + 2 * r->nh_d);
  q->sig.dzfi.assign(r->dzfi, r->dzfi + r->n[2] + 2 * r->nh_d);
  memcpy(q->sig.cbc, r->cbc, 6);
  if (r->kind == 1 && r->cbcvel) {
    q->cbcvel.assign(r->cbcvel, 18);
    q->bcvel.assign(r->bcvel, r->bcvel + 18);
  }
  q->est = field_bytes(*r) + plan_bytes_estimate(*r);
  q->t_submit = Clock::now();
  std::lock_guard<std::mutex> lk(s->mu);
  q->id = s->next_id++;
  *ticket = q->id;
  s->queue.push_back(q.get());
  s->reqs[q->id] = std::move(q);
  s->cv.notify_all();
  return FLUTAS_OK;
}

int flutas_gb300_server_wait(void *srv, long long ticket, double *relres, int *iters, double *latency_ms) {
  flutas_server *s = (flutas_server *)srv;
  if (!s || s->magic != flutas_server::MAGIC) return FLUTAS_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return FLUTAS_EINVAL;
  Request *q = it->second.get();
  s->cv.wait(lk, [&] { return q->done; });
  if (relres) *relres = q->relres;
  if (iters) *iters = q->iters;
  if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(q->t_done - q->t_submit).count();
  const int rc = q->rc;
  if (rc) fg_set_error_text(q->err.c_str());
  s->reqs.erase(it);
  return rc;
}

int flutas_gb300_server_stats(void *srv, char *buf, int len) {
  flutas_server *s = (flutas_server *)srv;
  if (!s || s->magic != flutas_server::MAGIC || !buf || len <= 0) return FLUTAS_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  std::vector<double> l = s->latencies;
  std::sort(l.begin(), l.end());
  auto pct = [&](double q) { return l.empty() ? 0.0 : l[std::min(l.size() - 1, (size_t)(q * (l.size() - 1) + 0.5))]; };
  const double span = std::chrono::duration<double>(s->t_last - s->t_first).count();
  size_t resident = 0;
  for (auto &pe : s->plans) resident += pe->bytes;
  snprintf(buf, (size_t)len,
           "{\"completed\": %lld, \"p50_ms\": %.4f, \"p99_ms\": %.4f, \"span_s\": %.4f, \"used_bytes\": %zu, "
           "\"budget_bytes\": %zu, \"resident_plans\": %zu, \"resident_plan_bytes\": %zu, \"queued\": %zu, \"inflight\": %d, "
           "\"max_device_overlap\": %d}",
           s->completed, pct(0.5), pct(0.99), span, s->used, s->budget, s->plans.size(), resident, s->queue.size(),
           s->inflight, max_overlap(s->spans));
  return FLUTAS_OK;
}

int flutas_gb300_server_reset_stats(void *srv) {
  flutas_server *s = (flutas_server *)srv;
  if (!s || s->magic != flutas_server::MAGIC) return FLUTAS_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  s->latencies.clear();
  s->spans.clear();
  s->completed = 0;
  s->t_first = s->t_last = Clock::now();
  return FLUTAS_OK;
}

int flutas_gb300_server_destroy(void *srv) {
  flutas_server *s = (flutas_server *)srv;
  if (!s || s->magic != flutas_server::MAGIC) return FLUTAS_EINVAL;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv.wait(lk, [&] { return s->queue.empty() && s->inflight == 0; });
    s->stop = true;
  }
  s->cv.notify_all();
  for (auto &t : s->workers) t.join();
  for (auto &pe : s->plans) flutas_gb300_fftend(pe->arr);
  if (s->ev_ref) cudaEventDestroy(s->ev_ref);
  s->magic = 0;
  delete s;
  return FLUTAS_OK;
}

}  // extern "C"
