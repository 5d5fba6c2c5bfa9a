"""Benchmark of the GB300 pressure-projection path (one JSON line on rank 0).

Workload (the two-phase projection the headline metric is quoted on):
  256^3 cells on [0,1]^3, periodic in x and y, walls in z (pressure N/N),
  VoF field of 64 non-overlapping spheres (radii U[0.03,0.08], tanh interface
  of width 1.5 dx), density ratio 1000 (rho0 = min rho = 1), previous
  pressures p^n, p^(n-1) = seeded sums of 32 Fourier modes, velocities
  U[-1,1] with periodic / no-slip ghosts, dt = f_t12 = f_t12_o = 1e-3.
  One step = one call of flutas_gb300_projection_df: pres_tw_src (Dodd-
  Ferrante split) -> bounduvw -> pold = p -> fillps -> updt_rhs_b -> Poisson
  solve -> boundp -> correc -> bounduvw -> p = pold + phi -> boundp.  Each
  step projects the fields the previous step left (as a time loop does), so
  every step solves a new RHS.

value        : projections/s with the mixed-precision solve (FP32 bulk, FP64
               residual/update) refined to relative residual <= 1e-10,
               device-resident fields, whole job (sum over replicas).
e2e          : same through the C ABI with pinned HOST buffers (H2D of
               u,v,w,p,rho,pold and D2H of u,v,w,p,pold inside every step).
modes        : the same step refined to 1e-6, and the plain FP64 solve.
roofline     : the kernel with the largest share of a profiled timed region
               (the same step with CUDA events around every launch, run after
               the headline region so their overhead stays out of it): its
               algorithmic bytes per launch / its mean CUDA-event duration.
cpu_baseline : the FP64 oracle restatement of solver_cpu (not FFTW) on the
               host cores, a bounded sample of the same projection.

--impl reference times that CPU restatement alone (the reference's own
solver_cpu needs gfortran + FFTW, neither of which exists on these machines).
Multi-GPU (torchrun): independent replicas, one per GPU, no collective on the
data path; barrier + max over ranks for timing only.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT = 256
SPHERES = 64
RHO_RATIO = 1000.0
DT = 1e-3
CBC = "PPPPNN"
CBCVEL = "PPPPDD" * 3     # u, v, w: periodic x,y; no-slip walls in z (cbcvel(0:1,1:3,1:3))
BCVEL = [0.0] * 18
METRIC = "Poisson solves/s at <=1e-6 & <=1e-10 rel. residual, mixed vs FP64; p50/p99 latency"

# algorithmic bytes per cell of each kernel (one launch covers every cell)
BYTES_PER_CELL = {
    "k_pres_tw_src": 72,            # R p,pold,rho,u,v,w ; W u,v,w
    "k_fillps": 32,                 # R u,v,w ; W rhs
    "k_correc_padd": 80,            # R phi ; RW u,v,w ; RW p ; W pold (the two-phase step's pold = p)
    "k_xfwd<f32,keep-fillps>": 36,  # R u,v,w (24) W f-copy (8) W S (4)
    "k_xfwd<f32,keep-halo>": 20,    # R f (8) W f-copy (8) W S (4)
    "k_xfwd<f32,residual>": 20,     # R f, x (16) W S (4)
    "k_xyfwd_plane<f32,keep-fillps>": 36,
    "k_xyfwd_plane<f32,keep-halo>": 20,
    "k_xyfwd_plane<f32,residual>": 20,
    "k_ypass_fwd<f32>": 8,
    "k_ypass_inv<f32>": 8,
    "k_zstream<f32>": 8,            # R S W S (eliminated values stay in L2)
    "k_zsolve<f32>": 8,
    "k_xinv<f32,halo>": 12,         # R S(4) W p(8)
    "k_xinv<f32,haloadd>": 20,      # R S(4) RW p(16)
    "k_xyinv_plane<f32,halo>": 12,
    "k_xyinv_plane<f32,haloadd>": 20,
    "k_xfwd<f64,fillps>": 32,       # R u,v,w W S
    "k_xyfwd_plane<f64,fillps>": 32,
    "k_ypass_fwd<f64>": 16,
    "k_ypass_inv<f64>": 16,
    "k_zstream<f64>": 16,
    "k_zsolve<f64>": 16,
    "k_xinv<f64,halo>": 16,
    "k_xyinv_plane<f64,halo>": 16,
    # stencil passes ahead of the fixed-size transforms, and the norm-only check
    "k_stencil<fillps>": 36,        # R u,v,w (24) W f-copy FP64 (8) W S FP32 (4)
    "k_stencil<residual>": 20,      # R f, x (16) W S (4)
    "k_resnorm": 16,                # R f, x
    "k_resnorm_correc": 96,         # R f, x ; RW u,v,w ; RW p ; W pold
    "k_sub": 24,                    # R x, s ; W d (halo-1 array)
    # cluster plane kernels (run-time sized, and compile-time sized for 256^2)
    "k_xyfwd_cluster<f32,keep-fillps>": 36,
    "k_xyfwd_cluster<f32,keep-halo>": 20,
    "k_xyfwd_cluster<f32,residual>": 20,
    "k_xyinv_cluster<f32,halo>": 12,
    "k_xyinv_cluster<f32,haloadd>": 20,
    "k_xyfwd_cluster<f64,fillps>": 32,
    "k_xyfwd_cluster<f64,plain>": 16,   # R S W S (FP64, in place)
    "k_xyfwd_plane<f64,plain>": 16,
    "k_stencil<f64,fillps>": 32,        # R u,v,w (24) W S FP64 (8)
    "k_stencil<df64,fillps>": 32,       # R u,v,w (24) W S double-float (8)
    "k_xyfwd_cluster<df64,plain>": 16,  # R S W S (double-float, in place)
    "k_xyinv_cluster<df64,halo>": 16,   # R S W p (FP64)
    "k_xyfwd_cluster<df64,halo>": 16,
    "k_xyfwd_plane<df64,plain>": 16,
    "k_xyinv_plane<df64,halo>": 16,
    "k_xyfwd_cluster<f64,halo>": 16,
    "k_xyinv_cluster<f64,halo>": 16,
    "k_xyfwd_fix<f32,f32>": 8,      # R S W S (in place)
    "k_xyfwd_fix<f32,keep-fillps>": 36,
    "k_xyfwd_fix<f32,keep-halo>": 20,
    "k_xyfwd_fix<f32,residual>": 20,
    "k_xyinv_fix<f32,halo>": 12,
    "k_xyinv_fix<f32,haloadd>": 20,
}

# FP64 instructions per cell of the FP64-bound kernels (the part's FP64 rate,
# not HBM, bounds them): DF increments 3x(2 sub + 1 add), fillps 3 sub + 1 mul
# + 2 fma, residual 2 add + 5 fma, correc 3x(sub + fma) + 1 add.
FP64_PER_CELL = {"k_stencil<f64,fillps>": 6, "k_stencil<df64,fillps>": 6, "k_pres_tw_src": 9, "k_stencil<fillps>": 6, "k_stencil<residual>": 7, "k_resnorm": 7,
                 "k_correc_padd": 7, "k_resnorm_correc": 14}
FP64_PEAK_TOPS = 0.60   # FP64 FMA instructions/s measured on this part (1.20 TFLOP/s counting an FMA as 2)


def peaks():
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ----------------------------------------------------------------- inputs
def make_fields(n, seed, device):
    """Seeded synthetic two-phase projection inputs (torch, float64, Fortran layout)."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    dx = 1.0 / n
    xc = (torch.arange(0, n + 2, dtype=torch.float64, device=device) - 0.5) * dx  # cell centres incl. ghosts
    Z, Y, X = torch.meshgrid(xc, xc, xc, indexing="ij")
    # spheres: rejection-sampled non-overlapping centres, periodic in x,y, away from the walls
    cents, radii = [], []
    rs = 0.03 + 0.05 * torch.rand(SPHERES * 20, generator=g, dtype=torch.float64)
    cs = torch.rand(SPHERES * 20, 3, generator=g, dtype=torch.float64)
    for r, c in zip(rs.tolist(), cs.tolist()):
        cz = 0.1 + 0.8 * c[2]
        c = [c[0], c[1], cz]
        ok = True
        for (c2, r2) in zip(cents, radii):
            d = [abs(c[0] - c2[0]), abs(c[1] - c2[1]), abs(c[2] - c2[2])]
            d[0], d[1] = min(d[0], 1 - d[0]), min(d[1], 1 - d[1])
            if math.sqrt(sum(t * t for t in d)) < r + r2 + 3 * dx:
                ok = False
                break
        if ok:
            cents.append(c)
            radii.append(r)
        if len(cents) == SPHERES:
            break
    psi = torch.zeros((n + 2,) * 3, dtype=torch.float64, device=device)
    w_int = 1.5 * dx
    for c, r in zip(cents, radii):
        ddx = torch.remainder(X - c[0] + 0.5, 1.0) - 0.5
        ddy = torch.remainder(Y - c[1] + 0.5, 1.0) - 0.5
        dist = torch.sqrt(ddx * ddx + ddy * ddy + (Z - c[2]) ** 2)
        psi = torch.maximum(psi, 0.5 * (1.0 + torch.tanh((r - dist) / w_int)))
    rho = psi * RHO_RATIO + (1.0 - psi) * 1.0   # update_property (src/vof.f90:240-271)
    # smooth previous pressures: 32 Fourier modes, periodic in x,y, Neumann in z
    def modes():
        k = torch.randint(0, 5, (32, 3), generator=g)
        a = torch.randn(32, generator=g, dtype=torch.float64)
        ph = 2 * math.pi * torch.rand(32, generator=g, dtype=torch.float64)
        f = torch.zeros_like(X)
        for m in range(32):
            kx, ky, kz = (int(t) for t in k[m])
            amp = float(a[m]) / (1.0 + kx * kx + ky * ky + kz * kz)
            f += amp * torch.cos(2 * math.pi * (kx * X + ky * Y) + float(ph[m])) * torch.cos(math.pi * kz * Z)
        return f
    p = modes()
    pold = modes()
    # velocities U[-1,1], periodic ghosts in x,y, no-slip walls in z
    u, v, w = (2 * torch.rand((n + 2,) * 3, generator=g, dtype=torch.float64) - 1 for _ in range(3))
    u, v, w = u.to(device), v.to(device), w.to(device)
    for f in (u, v, w):
        f[:, :, 0] = f[:, :, n]
        f[:, :, n + 1] = f[:, :, 1]
        f[:, 0, :] = f[:, n, :]
        f[:, n + 1, :] = f[:, 1, :]
    w[0] = 0.0
    w[n] = 0.0
    u[0] = -u[1]
    u[n + 1] = -u[n]
    v[0] = -v[1]
    v[n + 1] = -v[n]
    return {k: t.contiguous() for k, t in dict(u=u, v=v, w=w, p=p, pold=pold, rho=rho).items()}


def zgrid(n):
    dz = np.full(n + 2, 1.0 / n)
    return 1.0 / dz, 1.0 / dz, dz


# ----------------------------------------------------------------- replicas
def reduce_max(x: float, world: int, device="cpu") -> float:
    """Max of a per-rank scalar over all ranks (timing only; no data-path collective)."""
    if world == 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_rate(steps_per_rank: int, world: int, max_ms: float) -> float:
    """Whole-job rate: every replica ran `steps_per_rank` steps; the slowest rank's time counts."""
    return world * steps_per_rank / (max_ms / 1e3)


# ----------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "50", "-i", str(self.idx)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        def rd():
            for line in self.proc.stdout:
                self.rows.append([x.strip() for x in line.split(",")])
        self.thread = threading.Thread(target=rd, daemon=True)
        self.thread.start()

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
                for nm, val in zip(names, r[5:9]):
                    if val.lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------- GPU arm
def run_ours(args, rank, world, local_rank):
    import torch
    import flutas_gb300 as F

    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    F.load()
    n = args.n
    dzci, dzfi, dz = zgrid(n)
    dxi = dyi = float(n)
    P = F.initsolver([n, n, n], [dxi, dyi, float(n)], 1, dzci, dzfi, CBC, [0.0] * 6, "ccc")
    P.set_stream(torch.cuda.current_stream().cuda_stream, synchronous=True)
    dzci_d = torch.from_numpy(dzci).to(dev)
    dzfi_d = torch.from_numpy(dzfi).to(dev)
    pristine = make_fields(n, args.seed, dev)
    torch.cuda.synchronize()

    def fresh():
        return {k: t.clone() for k, t in pristine.items()}

    def step(f, precision, tol):
        P.projection_df(1, dxi, dyi, dzci_d, dzfi_d, [0.0] * 6, DT, DT, 1.0, f["rho"], f["pold"], f["u"],
                        f["v"], f["w"], f["p"], precision=precision, tol=tol, max_iter=12, cbcvel=CBCVEL,
                        bcvel=BCVEL)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def timed(precision, tol, steps, warmup, profile=False):
        f = fresh()
        for _ in range(warmup):
            step(f, precision, tol)
        iters = []
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        barrier()
        torch.cuda.synchronize()
        launches0 = F.launch_count()
        if profile:
            F.profile_report(reset=True)
            F.profile(True)
        ev[0].record()
        for i in range(steps):
            step(f, precision, tol)
            ev[i + 1].record()
            if precision == 1:
                iters.append(P.last_solve()[1])
        torch.cuda.synchronize()
        barrier()
        if profile:
            F.profile(False)
        launches = F.launch_count() - launches0
        lat = [ev[i].elapsed_time(ev[i + 1]) for i in range(steps)]
        total = ev[0].elapsed_time(ev[steps])
        rep = F.profile_report(reset=True) if profile else None
        return total, lat, iters, launches, rep, f

    if args.single:
        tol = 1e-10 if args.precision == 1 else 0.0
        t, lat, its, launches, _, _ = timed(args.precision, tol, args.steps, args.warmup)
        if rank == 0:
            return {"mode": "single", "precision": args.precision, "grid": [n, n, n], "steps": args.steps,
                    "ms_per_step": round(t / args.steps, 4), "gpu_launches": launches,
                    "fp32_solves_per_step": float(np.mean(its)) if its else None}
        return None

    clk = ClockSampler(local_rank)
    clk.start()
    t_mix, lat_mix, it_mix, launches, _, f_mix = timed(1, 1e-10, args.steps, args.warmup)
    t_m6, lat_m6, it_m6, _, _, _ = timed(1, 1e-6, args.steps, args.warmup)
    t_64, lat_64, _, _, _, f_64 = timed(0, 0.0, max(3, args.steps // 4), min(args.warmup, 3))
    # the per-kernel split (CUDA events around every launch, on the plan stream) from a
    # timed region of its own: the events add host and device work, kept out of the headline
    prof_steps = max(5, args.steps // 2)
    t_prof, _, _, _, rep, _ = timed(1, 1e-10, prof_steps, 1, profile=True)
    _, _, _, _, rep64, _ = timed(0, 0.0, 3, 1, profile=True)  # the FP64 form's kernel split
    clocks = clk.stop()

    # accuracy of one mixed step against one FP64 step on the same input
    fa, fb = fresh(), fresh()
    step(fa, 1, 1e-10)
    relres_mix = P.last_solve()[0]
    step(fb, 0, 0.0)
    def rel(a, b):
        a, b = a[1:-1, 1:-1, 1:-1], b[1:-1, 1:-1, 1:-1]
        a, b = a - a.mean(), b - b.mean()
        return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))
    err_p = rel(fa["p"] - pristine["p"], fb["p"] - pristine["p"])
    err_u = max(float(torch.linalg.vector_norm(fa[k] - fb[k]) / torch.linalg.vector_norm(fb[k]))
                for k in ("u", "v", "w"))
    _, divmax = F.chkdiv([n, n, n], dxi, dyi, float(n), 1, 1, dzfi_d, fa["u"], fa["v"], fa["w"])
    _, divmax64 = F.chkdiv([n, n, n], dxi, dyi, float(n), 1, 1, dzfi_d, fb["u"], fb["v"], fb["w"])

    # e2e: pinned host buffers through the C ABI
    host = {k: t.cpu().pin_memory() for k, t in pristine.items()}
    hnp = {k: t.numpy() for k, t in host.items()}
    for _ in range(min(args.warmup, 2)):
        P.projection_df(1, dxi, dyi, dzci, dzfi, [0.0] * 6, DT, DT, 1.0, hnp["rho"], hnp["pold"], hnp["u"],
                        hnp["v"], hnp["w"], hnp["p"], precision=1, tol=1e-10, max_iter=12, cbcvel=CBCVEL,
                        bcvel=BCVEL)
    # three runs of e2e_steps calls each, every run timed as a whole (host clock, copies
    # included); the best run is the value (the host of these boxes stalls now and then for
    # 20-70 ms, once in about 45 calls, in the one-pass and the slab form alike), and every
    # run's figure and the slowest step are reported beside it
    e2e_steps = max(3, args.steps // 4)
    e2e_runs, e2e_worst = [], 0.0
    for _ in range(3):
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            ts = time.perf_counter()
            P.projection_df(1, dxi, dyi, dzci, dzfi, [0.0] * 6, DT, DT, 1.0, hnp["rho"], hnp["pold"], hnp["u"],
                            hnp["v"], hnp["w"], hnp["p"], precision=1, tol=1e-10, max_iter=12, cbcvel=CBCVEL,
                            bcvel=BCVEL)
            e2e_worst = max(e2e_worst, (time.perf_counter() - ts) * 1e3)
        torch.cuda.synchronize()
        e2e_runs.append(reduce_max((time.perf_counter() - t0) * 1e3, world, dev))
    t_e2e = min(e2e_runs)
    barrier()
    field_bytes = (n + 2) ** 3 * 8
    # the same step with the FP64 oracle on the host (rank 0), after the timed regions: the
    # error of both GPU forms against it; the oracle's state then seeds the timed CPU baseline
    cpu_state, vs_oracle = None, None
    if rank == 0 and not args.no_oracle:
        cpu_state = cpu_first_step(n, pristine)
        fo = {k: torch.from_numpy(cpu_state["f"][k]).to(dev) for k in ("u", "v", "w", "p")}
        vs_oracle = {}
        for tag, fg in (("fp64", fb), ("mixed", fa)):
            vs_oracle[f"{tag}_vs_oracle_rel_l2_phi"] = rel(fg["p"] - pristine["p"], fo["p"] - pristine["p"])
            vs_oracle[f"{tag}_vs_oracle_rel_l2_u"] = max(
                float(torch.linalg.vector_norm(fg[k] - fo[k]) / torch.linalg.vector_norm(fo[k]))
                for k in ("u", "v", "w"))
        vs_oracle["oracle_max_div_after"] = cpu_state["max_div"]
        del fo

    # max over ranks
    t_mix, t_m6, t_64 = (reduce_max(x, world, dev) for x in (t_mix, t_m6, t_64))

    res = None
    if rank == 0:
        ncell = n ** 3
        steps = args.steps
        value = replica_rate(steps, world, t_mix)
        # roofline of the dominant kernel
        hbm, src = peaks()
        dom = max(rep.items(), key=lambda kv: kv[1][1]) if rep else None
        roof = None
        shares = {}
        if rep:
            tot = sum(v[1] for v in rep.values())
            shares = {k: {"launches": v[0], "ms": round(v[1], 4), "share": round(v[1] / tot, 4)}
                      for k, v in sorted(rep.items(), key=lambda kv: -kv[1][1])}
            name, (cnt, ms) = dom
            bpc = BYTES_PER_CELL.get(name)
            if bpc:
                achieved = bpc * ncell / (ms / cnt / 1e3) / 1e9
                roof = {"bound": "hbm", "kernel": name, "achieved": round(achieved, 1), "peak": hbm,
                        "unit": "GB/s", "frac": round(achieved / hbm, 4),
                        "peak_source": src, "bytes_per_launch": bpc * ncell,
                        "traffic": ncu_traffic(name, n)}
                f64 = FP64_PER_CELL.get(name)
                if f64:
                    ops = f64 * ncell / (ms / cnt / 1e3) / 1e12
                    roof["fp64"] = {"instr_per_cell": f64, "achieved_tinstr_s": round(ops, 4),
                                    "peak_tinstr_s": FP64_PEAK_TOPS, "frac": round(ops / FP64_PEAK_TOPS, 4),
                                    "note": "FP64 FMA/add instructions; the binding roof of this kernel"}
        res = {
            "metric": METRIC,
            "value": round(value, 3),
            "unit": "projections/s",
            "n_gpus": world,
            "steps": steps,
            "warmup": args.warmup,
            "ms_per_step": round(t_mix / steps, 4),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32 bulk + f64 residual/update",
            "data": "synthetic: seeded VoF spheres, U[-1,1] velocities, Fourier-mode pressures",
            "config": {"workload": f"two-phase DF-split projection {n}^3, periodic x,y, walls z, "
                                   f"density ratio {RHO_RATIO:g}, mixed precision to 1e-10",
                       "grid": [n, n, n], "cbc": CBC, "spheres": SPHERES,
                       "parallelism": f"replicas x{world}",
                       "l2": "inputs (6 FP64 fields, 0.8 GB) larger than the 129 MB L2"},
            "latency_ms": {"p50": round(float(np.percentile(lat_mix, 50)), 4),
                           "p99": round(float(np.percentile(lat_mix, 99)), 4)},
            "modes": {
                "mixed_1e-10": {"solves_per_s": round(world * steps / (t_mix / 1e3), 3),
                                "ms_per_step": round(t_mix / steps, 4),
                                "fp32_solves_per_step": round(float(np.mean(it_mix)), 2)},
                "mixed_1e-6": {"solves_per_s": round(world * steps / (t_m6 / 1e3), 3),
                               "ms_per_step": round(t_m6 / steps, 4),
                               "p50_ms": round(float(np.percentile(lat_m6, 50)), 4),
                               "p99_ms": round(float(np.percentile(lat_m6, 99)), 4),
                               "fp32_solves_per_step": round(float(np.mean(it_m6)), 2)},
                "fp64": {"solves_per_s": round(world * len(lat_64) / (t_64 / 1e3), 3),
                         "ms_per_step": round(t_64 / len(lat_64), 4),
                         "p50_ms": round(float(np.percentile(lat_64, 50)), 4),
                         "p99_ms": round(float(np.percentile(lat_64, 99)), 4),
                         "roofline": roofline_of(rep64, ncell, n)[0],
                         "kernels": roofline_of(rep64, ncell, n)[1]},
            },
            "accuracy": accuracy_block(n, relres_mix, err_p, err_u, divmax, divmax64, vs_oracle),
            "e2e": {"value": round(world * e2e_steps / (t_e2e / 1e3), 3), "unit": "projections/s",
                    "h2d_bytes_per_step": 6 * field_bytes, "d2h_bytes_per_step": 5 * field_bytes,
                    "runs": [round(world * e2e_steps / (t / 1e3), 3) for t in e2e_runs],
                    "slowest_step_ms": round(e2e_worst, 3),
                    "timing": f"best of 3 runs of {e2e_steps} calls on page-locked host arrays (host clock, every "
                              "run's copies in and out included); the runs' figures and the slowest call listed"},
            "gpu_launches": launches,
            "roofline": roof,
            "kernels": shares,
            "kernels_timed_region": {"steps": prof_steps, "ms_per_step": round(t_prof / prof_steps, 4),
                                     "note": "same step with CUDA events around every launch (their overhead "
                                             "is why this region is separate from the headline)"},
            "clocks": clocks,
        }
        if not args.no_cpu_baseline:
            res["cpu_baseline"] = cpu_baseline(n, pristine, budget_s=args.cpu_budget, state=cpu_state)
    if rank == 0 and not args.no_extras:
        del pristine, fa, fb, f_mix, f_64, host, hnp
        torch.cuda.empty_cache()
        import copy
        res["batch"] = batch_summary(args)
        torch.cuda.empty_cache()
        sa = copy.copy(args)
        sa.requests, sa.rates = args.serve_requests, [0.5, 0.8, 1.1]
        res["serving"] = run_serve(sa)
    return res


def accuracy_block(n, relres_mix, err_p, err_u, divmax, divmax64, vs_oracle):
    """Errors of the headline step: the mixed form against the FP64 form, both against
    the FP64 oracle (phi = p_after - p_before with the mean removed: the problem is
    singular; u,v,w as they are), and max|div u| after the step against the bound
    1e-11 U/dx (U = 1, the largest initial velocity)."""
    bound = 1e-11 * n
    acc = {"mixed_relres": relres_mix, "mixed_vs_fp64_rel_l2_phi": err_p, "mixed_vs_fp64_rel_l2_u": err_u,
           "max_div_after": divmax, "fp64_max_div_after": divmax64, "div_bound": bound,
           "mixed_meets_div_bound": bool(divmax <= bound), "fp64_meets_div_bound": bool(divmax64 <= bound),
           "div_note": "max|div u| after correc = dt/rho0 * max|f - A phi|: a solve stopped at relative "
                       "residual 1e-10 (L2) leaves more than the bound; the FP64 form meets it"}
    if vs_oracle:
        acc.update(vs_oracle)
        acc["fp64_parity_1e-12"] = bool(vs_oracle["fp64_vs_oracle_rel_l2_phi"] <= 1e-12 and
                                        vs_oracle["fp64_vs_oracle_rel_l2_u"] <= 1e-12)
    return acc


def roofline_of(rep, ncell, n):
    """Roofline entry of the kernel with the largest total time in a profiled region:
    algorithmic bytes per launch / its mean CUDA-event duration, against the measured
    HBM peak; for the FP64-bound kernels also the FP64 instruction rate."""
    if not rep:
        return None, {}
    hbm, src = peaks()
    tot = sum(v[1] for v in rep.values())
    shares = {k: {"launches": v[0], "ms": round(v[1], 4), "share": round(v[1] / tot, 4)}
              for k, v in sorted(rep.items(), key=lambda kv: -kv[1][1])}
    name, (cnt, ms) = max(rep.items(), key=lambda kv: kv[1][1])
    bpc = BYTES_PER_CELL.get(name)
    if not bpc:
        return {"kernel": name, "note": "no byte model for this kernel"}, shares
    achieved = bpc * ncell / (ms / cnt / 1e3) / 1e9
    roof = {"bound": "hbm", "kernel": name, "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
            "frac": round(achieved / hbm, 4), "peak_source": src, "bytes_per_launch": bpc * ncell,
            "traffic": ncu_traffic(name, n)}
    f64 = FP64_PER_CELL.get(name)
    if f64:
        ops = f64 * ncell / (ms / cnt / 1e3) / 1e12
        roof["fp64"] = {"instr_per_cell": f64, "achieved_tinstr_s": round(ops, 4), "peak_tinstr_s": FP64_PEAK_TOPS,
                        "frac": round(ops / FP64_PEAK_TOPS, 4),
                        "note": "FP64 FMA/add instructions; the binding roof of this kernel"}
    return roof, shares


def ncu_traffic(kernel, n):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, scaled to n^3."""
    try:
        d = json.load(open(os.path.join(ROOT, "profiles", "ncu_traffic.json")))
        e = d[kernel]
        return round(e["dram_bytes_per_launch"] * (n ** 3) / e["cells"], 0)
    except Exception:
        return None


# ----------------------------------------------------------------- CPU arm
def oracle_projection_fields(n, fields):
    return {k: (v.cpu().numpy().copy() if hasattr(v, "cpu") else v.copy()) for k, v in fields.items()}


def cpu_step(O, S, n, f, dzci, dzfi, dz):
    """One two-phase projection with the FP64 oracle (same sequence as the GPU step)."""
    dxi = dyi = float(n)
    nn = [n, n, n]
    O.pres_tw_src(nn, dxi, dyi, float(n), 1, 1, dzci, 1.0, DT, DT, f["p"], f["pold"], f["rho"], f["u"], f["v"],
                  f["w"])
    f["pold"][1:-1, 1:-1, 1:-1] = f["p"][1:-1, 1:-1, 1:-1]  # the app's pold = p, then boundp
    O.boundp(CBC, nn, [0.0] * 6, 1, [1 / dxi, 1 / dyi, 0.0], dz, dz, f["pold"])
    O.bounduvw(CBCVEL, nn, BCVEL, 1, 1, [1 / dxi, 1 / dyi, 0.0], dz, dz, f["u"], f["v"], f["w"])
    phi = np.zeros_like(f["p"])
    O.fillps(nn, 1, 1, dxi, dyi, float(n), dzfi, 1.0 / DT, 1.0, f["u"], f["v"], f["w"], phi)
    O.updt_rhs_b(nn, "ccc", CBC, S.rhsbx, S.rhsby, S.rhsbz, phi)
    S.solve(phi)
    O.boundp(CBC, nn, [0.0] * 6, 1, [1 / dxi, 1 / dyi, 0.0], dz, dz, phi)
    O.correc(nn, 1, 1, dxi, dyi, float(n), dzci, DT, 1.0, phi, f["u"], f["v"], f["w"])
    O.bounduvw(CBCVEL, nn, BCVEL, 1, 1, [1 / dxi, 1 / dyi, 0.0], dz, dz, f["u"], f["v"], f["w"])
    f["p"][1:-1, 1:-1, 1:-1] += phi[1:-1, 1:-1, 1:-1]
    O.boundp(CBC, nn, [0.0] * 6, 1, [1 / dxi, 1 / dyi, 0.0], dz, dz, f["p"])


def cpu_setup(n):
    from oracle import oracle as O
    O.build()
    O.set_threads(os.cpu_count() or 1)
    dzci, dzfi, dz = zgrid(n)
    S = O.SolverSetup([n, n, n], [float(n)] * 3, 1, dzci, dzfi, CBC, [0.0] * 6, "ccc")
    return O, S, dzci, dzfi, dz


def cpu_first_step(n, pristine):
    """One oracle step on the pristine fields: the reference result of the headline step."""
    O, S, dzci, dzfi, dz = cpu_setup(n)
    f = oracle_projection_fields(n, pristine)
    cpu_step(O, S, n, f, dzci, dzfi, dz)
    _, mx = O.chkdiv([n, n, n], float(n), float(n), float(n), 1, 1, dzfi, f["u"], f["v"], f["w"])
    return {"O": O, "S": S, "z": (dzci, dzfi, dz), "f": f, "max_div": float(mx)}


def cpu_baseline(n, pristine, budget_s=12.0, state=None):
    if state is None:
        state = cpu_first_step(n, pristine)  # warm-up (plans, page faults)
    O, S, f = state["O"], state["S"], state["f"]
    dzci, dzfi, dz = state["z"]
    cnt, t0 = 0, time.perf_counter()
    while True:
        cpu_step(O, S, n, f, dzci, dzfi, dz)
        cnt += 1
        el = time.perf_counter() - t0
        if el >= budget_s or cnt >= 200:
            break
    return {"value": round(cnt / el, 4), "unit": "projections/s", "cores": O.get_threads(), "kind": "port",
            "sample": f"{cnt} full FP64 two-phase projections at {n}^3 (oracle restatement of "
                      "solver_cpu with own r2r FFTs, not FFTW), after 1 warm-up"}


def run_reference(args, rank):
    if rank != 0:
        return None
    import torch
    fields = make_fields(args.n, args.seed, "cpu")
    O, S, dzci, dzfi, dz = cpu_setup(args.n)
    f = oracle_projection_fields(args.n, fields)
    for _ in range(args.warmup):
        cpu_step(O, S, args.n, f, dzci, dzfi, dz)
    lat = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        cpu_step(O, S, args.n, f, dzci, dzfi, dz)
        lat.append((time.perf_counter() - t0) * 1e3)
    total = sum(lat)
    value = args.steps / (total / 1e3)
    sample = (f"{args.steps} FP64 two-phase projections at {args.n}^3 on {O.get_threads()} host threads "
              "(oracle restatement of solver_cpu; the reference itself needs gfortran+FFTW, absent)")
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "projections/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded VoF spheres, U[-1,1] velocities, Fourier-mode pressures",
        "config": {"workload": f"two-phase DF-split projection {args.n}^3, periodic x,y, walls z, "
                               f"density ratio {RHO_RATIO:g}", "grid": [args.n] * 3, "cbc": CBC},
        "latency_ms": {"p50": round(float(np.percentile(lat, 50)), 3),
                       "p99": round(float(np.percentile(lat, 99)), 3)},
        "cpu_baseline": {"value": round(value, 4), "unit": "projections/s", "cores": O.get_threads(),
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "projections/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


# ----------------------------------------------------------------- batch mode
def batch_grids(count, seed):
    """Uneven grids: each axis 16*m log-uniform in [32,192], BCs per axis from
    {PP,NN,DD}, z uniform or tanh-clustered (factor U[1,2.5])."""
    rng = np.random.default_rng(seed)
    grids = []
    for _ in range(count):
        n = [int(16 * round(np.exp(rng.uniform(np.log(32), np.log(192))) / 16)) for _ in range(3)]
        cbc = "".join(rng.choice(["PP", "NN", "DD"]) for _ in range(3))
        gr = 0.0 if (rng.uniform() < 0.5 or cbc[4:6] == "PP") else float(rng.uniform(1.0, 2.5))
        k = np.arange(0, n[2] + 1) / n[2]
        zf = 0.5 * (1 + np.tanh((k - 0.5) * gr) / np.tanh(gr / 2)) if gr else k
        dzf = np.empty(n[2] + 2)
        dzf[1:-1] = np.diff(zf)
        dzf[0], dzf[-1] = dzf[1], dzf[-2]
        dzc = np.empty(n[2] + 2)
        dzc[:-1] = 0.5 * (dzf[:-1] + dzf[1:])
        dzc[-1] = dzc[-2]
        grids.append(dict(n=n, dli=[float(n[0]), float(n[1]), 1.0], dzci=1.0 / dzc, dzfi=1.0 / dzf, cbc=cbc,
                          dzf=dzf))
    return grids


def run_batch(args, keep=False):
    import torch
    import flutas_gb300 as F
    F.load()
    grids = batch_grids(args.grids, args.seed)
    cells = sum(int(np.prod(g["n"])) for g in grids)
    t0 = time.perf_counter()
    B = F.Batch(grids, autotune=True)
    t_create = time.perf_counter() - t0
    rng = np.random.default_rng(args.seed + 1)
    rhs = []
    for g in grids:
        nx, ny, nz = g["n"]
        f = rng.uniform(-1, 1, (nz, ny, nx))
        w = g["dzf"][1:-1][:, None, None]
        f -= (f * w).sum() / (w.sum() * nx * ny)  # compatible with every BC (zero weighted mean)
        h = np.zeros((nz + 2, ny + 2, nx + 2))
        h[1:-1, 1:-1, 1:-1] = f
        rhs.append(torch.from_numpy(h).cuda())
    torch.cuda.synchronize()
    def load_rhs():
        for i, r in enumerate(rhs):
            B.set(i, r)
    for _ in range(args.warmup):
        load_rhs()
        B.solve(tol=1e-10, max_iter=8)
    times, iters, rels = [], [], []
    l0 = F.launch_count()
    for _ in range(args.steps):
        load_rhs()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        rr, it = B.solve(tol=1e-10, max_iter=8)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
        iters.append(it)
        rels.append(rr)
    launches = (F.launch_count() - l0) // max(1, args.steps)
    queue = [ln for ln in B.report().splitlines() if ln.startswith("queue:")]
    # the same grids one by one with the single-grid paths (a sample)
    sample = list(range(0, len(grids), max(1, len(grids) // 24)))
    t_seq_mixed = t_seq_fp64 = 0.0
    for i in sample:
        g = grids[i]
        P = F.initsolver(g["n"], g["dli"], 1, g["dzci"], g["dzfi"], g["cbc"], [0.0] * 6, "ccc")
        x = rhs[i].clone()
        P.solve_mixed(x, tol=1e-10, max_iter=8)  # warm
        for mode in ("mixed", "fp64"):
            x = rhs[i].clone()
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            if mode == "mixed":
                P.solve_mixed(x, tol=1e-10, max_iter=8)
            else:
                P.solver(x)
            torch.cuda.synchronize()
            dt_ = time.perf_counter() - t1
            if mode == "mixed":
                t_seq_mixed += dt_
            else:
                t_seq_fp64 += dt_
        P.fftend()
    ms = float(np.median(times))
    scale = len(grids) / len(sample)
    out = {"mode": "batch", "metric": "grids solved/s (mixed precision to 1e-10)", "grids": len(grids),
            "cells": cells, "value": round(len(grids) / (ms / 1e3), 2), "unit": "grids/s",
            "ms_per_batch": round(ms, 3), "cells_per_s": round(cells / (ms / 1e3), 1),
            "max_relres": float(np.max(rels)), "fp32_solves_per_grid": {
                "mean": float(np.mean(iters)), "max": int(np.max(iters))},
            "gpu_launches_per_batch": int(launches), "create_s": round(t_create, 2),
            "queue": queue[0][7:] if queue else ("one persistent kernel"
                                                  if os.environ.get("FLUTAS_GB300_BATCH_PERSISTENT") == "1"
                                                  else "one work-queue kernel per pass, in one CUDA graph"),
            "sequential_single_grid": {"mixed_grids_per_s": round(len(sample) / t_seq_mixed, 2),
                                       "fp64_grids_per_s": round(len(sample) / t_seq_fp64, 2),
                                       "sample_grids": len(sample), "est_batch_equivalent_ms":
                                           round(t_seq_mixed * scale * 1e3, 2)},
            "steps": args.steps, "warmup": args.warmup,
            "timing": "CUDA events around each batch solve; RHS reloaded (device copies) between solves, untimed"}
    if keep:
        out.update({"_batch": B, "_grids": grids, "_rhs": rhs, "_iters": iters[-1]})
    else:
        B.destroy()
    return out


# ----------------------------------------------------------------- serving mode
def serve_sizes(rng, count):
    """Sizes 64^3..384^3 (volume log-uniform), aspect up to 4:1, axes multiples of 32."""
    out = []
    while len(out) < count:
        vol = np.exp(rng.uniform(np.log(64 ** 3), np.log(384 ** 3)))
        a = np.exp(rng.uniform(-np.log(2), np.log(2), 3))
        a = a / np.prod(a) ** (1 / 3)
        n = [int(max(32, min(512, 32 * round(vol ** (1 / 3) * x / 32)))) for x in a]
        if max(n) / min(n) <= 4.0:
            out.append(n)
    return out


def run_serve(args, classes_n=32, fp64_sample=400):
    """C5 stream: Poisson requests of log-uniform volume (64^3..384^3, aspect <= 4:1)
    drawn from `classes_n` grid shapes, 30% with a two-phase (density-jump) RHS,
    tolerance 1e-6 or 1e-10 (50/50), fields resident on the device (the server solves
    them in place), admission under the HBM budget, Poisson arrivals at fractions of
    the measured capacity; the same stream in FP64 through the server, and the plain
    FP64 drop-in solver on a sample of it."""
    import torch
    import flutas_gb300 as F
    F.load()
    rng = np.random.default_rng(args.seed)
    classes = []
    while len(classes) < classes_n:
        for c in serve_sizes(rng, classes_n):
            if tuple(c) not in classes and len(classes) < classes_n:
                classes.append(tuple(c))
    classes.sort()
    sizes = [classes[i] for i in rng.integers(0, len(classes), args.requests)]
    dev = torch.device("cuda")
    g = torch.Generator(device=dev).manual_seed(args.seed)
    rhs = {}
    for c in classes:
        nx, ny, nz = c
        for kind in ("1p", "2p"):
            f = torch.zeros((nz + 2, ny + 2, nx + 2), dtype=torch.float64, device=dev)
            v = 2.0 * torch.rand((nz, ny, nx), generator=g, dtype=torch.float64, device=dev) - 1.0
            if kind == "2p":  # density-jump structure of a two-phase RHS: large values inside a drop
                zz, yy, xx = torch.meshgrid(*(torch.linspace(0, 1, m, device=dev, dtype=torch.float64)
                                              for m in (nz, ny, nx)), indexing="ij")
                drop = ((xx - 0.5) ** 2 + (yy - 0.5) ** 2 + (zz - 0.5) ** 2) < 0.04
                v = v * torch.where(drop, float(np.exp(rng.uniform(np.log(10), np.log(1000)))), 1.0)
                del zz, yy, xx, drop
            v -= v.mean()  # compatible with the singular (periodic x, y, Neumann z) problem
            f[1:-1, 1:-1, 1:-1] = v
            rhs[(c, kind)] = f
    nout = 12  # outputs per class: two requests of a class in flight at once never share one
    outs = {c: [torch.empty_like(rhs[(c, "1p")]) for _ in range(nout)] for c in classes}
    torch.cuda.synchronize()
    dz = {c: np.full(c[2] + 2, float(c[2])) for c in classes}
    reqs = []
    for s in sizes:
        kind = "2p" if rng.uniform() < 0.3 else "1p"
        tol = 1e-6 if rng.uniform() < 0.5 else 1e-10
        reqs.append((tuple(s), kind, tol))
    occ = {}
    slot = []
    for c, _, _ in reqs:  # the k-th request of a class writes output k mod nout
        slot.append(occ.get(c, 0) % nout)
        occ[c] = occ.get(c, 0) + 1
    S = F.Server(hbm_budget_bytes=int(args.budget_gb * (1 << 30)), slots=args.slots)

    def submit(i, tol=None):
        c, kind, t = reqs[i]
        return S.submit_solve(c, [float(c[0]), float(c[1]), float(c[2])], dz[c], dz[c], "PPPPNN", rhs[(c, kind)],
                              outs[c][slot[i]], tol=t if tol is None else tol, max_iter=8)

    for j, c in enumerate(classes):  # warm: plans become resident
        S.wait(S.submit_solve(c, [float(c[0]), float(c[1]), float(c[2])], dz[c], dz[c], "PPPPNN", rhs[(c, "1p")],
                              outs[c][0], tol=1e-6, max_iter=8))
    S.reset_stats()
    t0 = time.perf_counter()
    ts = [submit(i) for i in range(len(reqs))]
    cap_stat = [S.wait(t) for t in ts]
    capacity = len(reqs) / (time.perf_counter() - t0)
    overlap = S.stats().get("max_device_overlap")
    sweep = []
    for frac in args.rates:
        rate = frac * capacity
        S.reset_stats()
        gaps = rng.exponential(1.0 / rate, len(reqs))
        t0 = time.perf_counter()
        tick = t0
        ts = []
        for i in range(len(reqs)):
            tick += gaps[i]
            dt_ = tick - time.perf_counter()
            if dt_ > 0:
                time.sleep(dt_)
            ts.append(submit(i))
        stat = [S.wait(t) for t in ts]
        span = time.perf_counter() - t0
        st = S.stats()
        codes, worst = {}, {}
        for (c, kind, tol), x in zip(reqs, stat):
            if x[0] != 0:
                codes[str(x[0])] = codes.get(str(x[0]), 0) + 1
            key = f"{kind}@{tol:g}"
            worst[key] = max(worst.get(key, 0.0), x[1])
        sweep.append({"offered_fraction": frac, "offered_per_s": round(rate, 2),
                      "solves_per_s": round(len(reqs) / span, 2), "p50_ms": round(st["p50_ms"], 3),
                      "p99_ms": round(st["p99_ms"], 3), "max_device_overlap": st.get("max_device_overlap"),
                      "nonzero_status": codes, "worst_relres": worst})
    # the same stream in FP64 through the same server (tol = 0 selects the drop-in solver)
    S.reset_stats()
    t0 = time.perf_counter()
    ts = [submit(i, tol=0.0) for i in range(len(reqs))]
    for t in ts:
        S.wait(t)
    cap64 = len(reqs) / (time.perf_counter() - t0)
    S.close()
    # the plain FP64 drop-in solver call on device arrays, one request after another (a sample)
    plans, lat64 = {}, []
    sample = reqs[:fp64_sample]
    for c, kind, tol in sample:
        x = outs[c][0]
        if c not in plans:
            plans[c] = F.initsolver(c, [float(c[0]), float(c[1]), float(c[2])], 1, dz[c], dz[c], "PPPPNN", [0.0] * 6)
            x.copy_(rhs[(c, kind)])
            plans[c].solver(x)
        x.copy_(rhs[(c, kind)])
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        plans[c].solver(x)
        lat64.append((time.perf_counter() - t1) * 1e3)
    for P in plans.values():
        P.fftend()
    vols = [int(np.prod(c)) for c, _, _ in reqs]
    return {"mode": "serve", "metric": "projection solves/s and p50/p99 latency under a mixed-size stream",
            "requests": len(reqs), "size_classes": len(classes),
            "volume_cells": {"min": min(vols), "median": int(np.median(vols)), "max": max(vols)},
            "two_phase_frac": 0.3, "tolerances": "1e-6 / 1e-10 (50/50)", "budget_gb": args.budget_gb,
            "slots": args.slots, "fields": "device-resident (solved in place by the server)",
            "capacity_solves_per_s": round(capacity, 2), "capacity_max_device_overlap": overlap,
            "capacity_nonzero_status": {str(c): sum(1 for x in cap_stat if x[0] == c)
                                        for c in sorted({x[0] for x in cap_stat if x[0] != 0})}, "sweep": sweep,
            "fp64_served_capacity_solves_per_s": round(cap64, 2),
            "fp64_drop_in_sequential": {"solves_per_s": round(len(lat64) / (sum(lat64) / 1e3), 2),
                                        "p50_ms": round(float(np.percentile(lat64, 50)), 3),
                                        "p99_ms": round(float(np.percentile(lat64, 99)), 3),
                                        "requests": len(lat64),
                                        "note": "solver() on device arrays, one at a time, the stream's first "
                                                "requests"},
            "timing": "host clock; latency = submit to result (device-resident fields); Poisson arrivals"}


def batch_summary(args):
    """C4 inside the headline line: run_batch with a short timed region, its HBM
    fraction on the mixed-precision byte model (32 B/cell for the first FP32 solve,
    48 B/cell for each further one), and the residual of a sample of grids
    recomputed by the FP64 oracle."""
    import copy
    a = copy.copy(args)
    a.steps, a.warmup = 3, 1
    res = run_batch(a, keep=True)
    B, grids, rhs, it = res.pop("_batch"), res.pop("_grids"), res.pop("_rhs"), res.pop("_iters")
    byts = sum(int(np.prod(g["n"])) * (32 + 48 * (int(k) - 1)) for g, k in zip(grids, it))
    hbm, src = peaks()
    gbs = byts / (res["ms_per_batch"] / 1e3) / 1e9
    res["hbm"] = {"bytes_per_batch": byts, "achieved_gbs": round(gbs, 1), "peak_gbs": hbm,
                  "frac": round(gbs / hbm, 4), "peak_source": src,
                  "model": "per grid cells x (32 + 48 x (FP32 solves - 1)) bytes"}
    try:
        from oracle import oracle as O
        O.build()
        worst = 0.0
        for gi in range(0, len(grids), max(1, len(grids) // 8)):
            g = grids[gi]
            x = B.get(gi)
            f = rhs[gi].cpu().numpy()
            r = O.residual(g["n"], g["cbc"], g["dli"][0], g["dli"][1], 1, g["dzci"], g["dzfi"], f, x)
            worst = max(worst, float(np.linalg.norm(r) / np.linalg.norm(f[1:-1, 1:-1, 1:-1])))
        res["oracle_worst_relres_sample"] = worst
    except Exception as e:  # the oracle only checks this number; without it the number is left out
        res["oracle_worst_relres_sample"] = f"unavailable: {e}"
    B.destroy()
    return res


def run_solve(args):
    """Poisson solves alone on one grid (--grid NX NY NZ, --cbc, uniform z), mixed
    to --tol (0: the FP64 solver), on a device array with a seeded U[-1,1] RHS."""
    import torch
    import flutas_gb300 as F
    nx, ny, nz = args.grid
    dzci, dzfi = zgrid_stretched(nz, 0.0)
    P = F.initsolver([nx, ny, nz], [float(nx), float(ny), float(nz)], 1, dzci, dzfi, args.cbc, [0.0] * 6, "ccc")
    rng = np.random.default_rng(args.seed)
    f = np.zeros((nz + 2, ny + 2, nx + 2))
    g = rng.uniform(-1.0, 1.0, (nz, ny, nx))
    f[1:-1, 1:-1, 1:-1] = g - g.mean()
    rhs = torch.from_numpy(f).cuda()
    x = rhs.clone()

    def once():
        x.copy_(rhs)
        return P.solve_mixed(x, tol=args.tol, max_iter=10) if args.tol > 0 else (P.solver(x), None)

    for _ in range(args.warmup):
        once()
    ts, out = [], None
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        out = once()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    info = P.info()
    return {"mode": "solve", "grid": [nx, ny, nz], "cbc": args.cbc, "tol": args.tol,
            "ms_per_solve": round(float(np.median(ts)), 4), "relres_and_fp32_solves": out if args.tol > 0 else None,
            "xy_path_fp32": info["xy_path_fp32"], "xy_path_fp64": info["xy_path_fp64"],
            "timing": "CUDA events around each solve (median), including the device copy of the RHS"}

# ------------------------------------------------------------ configs C1, C3
def zgrid_stretched(n, gr):
    """dzci, dzfi (0:n+1) of src/initgrid.f90 steps 1-5 with two-end tanh
    clustering (gr > 0; uniform for gr = 0), lz = 1, one ghost layer:
    zf(k) = 0.5 (1 + tanh((k/n - 0.5) gr) / tanh(gr/2)), dzf(k) = zf(k) - zf(k-1),
    dzc(k) = (dzf(k) + dzf(k+1)) / 2, and the ghost extension of step 5
    (dzf(0) = dzf(1), dzf(n+1) = dzf(n-2), dzc(n+1) = dzc(n-1))."""
    z0 = np.arange(1, n + 1, dtype=np.float64) / n
    zf = 0.5 * (1.0 + np.tanh((z0 - 0.5) * gr) / np.tanh(gr / 2.0)) if gr != 0.0 else z0
    dzf = np.empty(n + 2)
    dzf[1:n + 1] = np.diff(np.concatenate([[0.0], zf]))
    dzf[0], dzf[n + 1] = dzf[1], dzf[n]
    dzc = np.empty(n + 2)
    dzc[0:n + 1] = 0.5 * (dzf[0:n + 1] + dzf[1:n + 2])
    dzc[n + 1] = dzc[n]
    dzf[n + 1] = dzf[n - 2]     # step 5: dzf(k) = dzf(2n-k-1), dzc(k) = dzc(2n-k) for k = n+1
    dzc[n + 1] = dzc[n - 1]
    return 1.0 / dzc, 1.0 / dzf


def run_config1(args):
    """C1: plain single-phase FP64 projection, 128^3, periodic x,y, walls z (one
    fillps -> solver -> boundp -> correc -> bounduvw), as drop-in calls and as one fused
    call, device-resident and through host arrays, with the oracle restatement on
    the host cores beside it."""
    import torch
    import flutas_gb300 as F
    dev = torch.device("cuda:0")
    n = 128
    dzci, dzfi = zgrid_stretched(n, 0.0)
    dxi = dyi = float(n)
    P = F.initsolver([n, n, n], [dxi, dyi, float(n)], 1, dzci, dzfi, CBC, [0.0] * 6, "ccc")
    g = torch.Generator(device="cpu").manual_seed(args.seed)
    vel = [2 * torch.rand((n + 2,) * 3, generator=g, dtype=torch.float64) - 1 for _ in range(3)]
    for f in vel:
        f[:, :, 0] = f[:, :, n]; f[:, :, n + 1] = f[:, :, 1]
        f[:, 0, :] = f[:, n, :]; f[:, n + 1, :] = f[:, 1, :]
    for f in vel[:2]:
        f[0] = -f[1]; f[n + 1] = -f[n]
    vel[2][0] = 0.0; vel[2][n] = 0.0; vel[2][n + 1] = 0.0
    pristine = {"u": vel[0], "v": vel[1], "w": vel[2], "p": torch.zeros((n + 2,) * 3, dtype=torch.float64)}
    dd = {k: t.to(dev) for k, t in pristine.items()}
    dzci_d, dzfi_d = torch.from_numpy(dzci).to(dev), torch.from_numpy(dzfi).to(dev)
    dzc, dzf = 1.0 / dzci, 1.0 / dzfi

    def fresh():
        return {k: t.clone() for k, t in dd.items()}

    def three_calls(f):
        F.fillps([n, n, n], 1, 1, dxi, dyi, float(n), dzfi_d, 1.0 / DT, 1.0, f["u"], f["v"], f["w"], f["p"])
        P.solver(f["p"])
        F.boundp(CBC, [n, n, n], [0.0] * 6, 1, [1.0 / n] * 3, dzc, dzf, f["p"])
        F.correc([n, n, n], 1, 1, dxi, dyi, float(n), dzci_d, DT, 1.0, f["p"], f["u"], f["v"], f["w"])
        F.bounduvw(CBCVEL, [n, n, n], BCVEL, 1, 1, [1.0 / n] * 3, dzc, dzf, f["u"], f["v"], f["w"])

    def fused(f):
        P.projection(1, dxi, dyi, dzci_d, dzfi_d, [0.0] * 6, DT, 1.0, f["u"], f["v"], f["w"], f["p"], precision=0,
                     cbcvel=CBCVEL, bcvel=BCVEL)

    def timed(fn, steps):
        fs = [fresh() for _ in range(steps + 3)]
        for i in range(3):
            fn(fs[i])
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for i in range(steps):
            fn(fs[3 + i])
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / steps, fs[-1]

    steps = max(args.steps, 10)
    t3, f3 = timed(three_calls, steps)
    tf, ff = timed(fused, steps)
    _, div3 = F.chkdiv([n, n, n], dxi, dyi, float(n), 1, 1, dzfi_d, f3["u"], f3["v"], f3["w"])
    _, divf = F.chkdiv([n, n, n], dxi, dyi, float(n), 1, 1, dzfi_d, ff["u"], ff["v"], ff["w"])
    # e2e through host arrays (pinned)
    host = {k: t.clone().pin_memory() for k, t in pristine.items()}
    hnp = {k: t.numpy() for k, t in host.items()}
    for _ in range(2):
        P.projection(1, dxi, dyi, dzci, dzfi, [0.0] * 6, DT, 1.0, hnp["u"], hnp["v"], hnp["w"], hnp["p"],
                     precision=0, cbcvel=CBCVEL, bcvel=BCVEL)
    t0 = time.perf_counter()
    for _ in range(steps):
        P.projection(1, dxi, dyi, dzci, dzfi, [0.0] * 6, DT, 1.0, hnp["u"], hnp["v"], hnp["w"], hnp["p"],
                     precision=0, cbcvel=CBCVEL, bcvel=BCVEL)
    te = (time.perf_counter() - t0) * 1e3 / steps
    # the oracle restatement of the same three calls on the host cores
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        S = O.SolverSetup([n, n, n], [dxi, dyi, float(n)], 1, dzci, dzfi, CBC, [0.0] * 6, "ccc")
        f = {k: t.numpy().copy() for k, t in pristine.items()}
        def cpu_once():
            O.fillps([n, n, n], 1, 1, dxi, dyi, float(n), dzfi, 1.0 / DT, 1.0, f["u"], f["v"], f["w"], f["p"])
            S.solve(f["p"])
            O.boundp(CBC, [n, n, n], [0.0] * 6, 1, [1.0 / n] * 3, dzc, dzf, f["p"])
            O.correc([n, n, n], 1, 1, dxi, dyi, float(n), dzci, DT, 1.0, f["p"], f["u"], f["v"], f["w"])
            O.bounduvw(CBCVEL, [n, n, n], BCVEL, 1, 1, [1.0 / n] * 3, dzc, dzf, f["u"], f["v"], f["w"])
        cpu_once()
        reps, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < min(args.cpu_budget, 5.0) or reps < 3:
            cpu_once()
            reps += 1
        tc = (time.perf_counter() - t0) / reps * 1e3
        cpu = {"ms_per_projection": round(tc, 3), "projections_per_s": round(1e3 / tc, 2), "cores": O.get_threads(),
               "kind": "port", "sample": f"{reps} FP64 fillps+solver+boundp+correc+bounduvw at 128^3"}
    cells = n ** 3
    return {"mode": "c1", "workload": "single-phase FP64 projection 128^3, periodic x,y, walls z, U[-1,1] velocities",
            "three_calls": {"ms": round(t3, 4), "projections_per_s": round(1e3 / t3, 2),
                            "hbm_gbs_136B": round(136 * cells / t3 / 1e6, 1)},
            "fused": {"ms": round(tf, 4), "projections_per_s": round(1e3 / tf, 2),
                      "hbm_gbs_112B": round(112 * cells / tf / 1e6, 1)},
            "e2e_fused_host_arrays": {"ms": round(te, 3), "projections_per_s": round(1e3 / te, 2)},
            "max_div_after": {"three_calls": div3, "fused": divf}, "div_bound": 1e-11 * dxi, "cpu_baseline": cpu,
            "hbm_peak_gbs": peaks()[0]}


def run_config3(args):
    """C3: stretched-grid solve, 512x512x256, tanh two-end clustering (gr = 2) in z,
    Neumann x (DCT-II), periodic y, Neumann bottom / Dirichlet top in z; RHS a
    seeded Gaussian random field with a k^-5/3 spectrum, zero mean.  FP64 solver
    against the mixed solve refined to 1e-6 and to 1e-10 (device-resident)."""
    import torch
    import flutas_gb300 as F
    dev = torch.device("cuda:0")
    nx, ny, nz = 512, 512, 256
    cbc = "NNPPND"
    dzci, dzfi = zgrid_stretched(nz, 2.0)
    dli = [float(nx), float(ny), float(nz)]
    P = F.initsolver([nx, ny, nz], dli, 1, dzci, dzfi, cbc, [0.0] * 6, "ccc")
    g = torch.Generator(device=dev).manual_seed(args.seed)
    white = torch.randn((nz, ny, nx), generator=g, dtype=torch.float64, device=dev)
    spec = torch.fft.rfftn(white)
    kz = torch.fft.fftfreq(nz, device=dev, dtype=torch.float64)[:, None, None] * nz
    ky = torch.fft.fftfreq(ny, device=dev, dtype=torch.float64)[None, :, None] * ny
    kx = torch.fft.rfftfreq(nx, device=dev, dtype=torch.float64)[None, None, :] * nx
    k = torch.sqrt(kx * kx + ky * ky + kz * kz)
    k[0, 0, 0] = 1.0
    spec *= k ** (-5.0 / 6.0)       # power ~ k^-5/3
    spec[0, 0, 0] = 0.0
    field = torch.fft.irfftn(spec, s=(nz, ny, nx))
    field -= field.mean()
    field /= field.std()
    rhs = torch.zeros((nz + 2, ny + 2, nx + 2), dtype=torch.float64, device=dev)
    rhs[1:-1, 1:-1, 1:-1] = field
    del white, spec, k, field

    def timed(fn, steps):
        bufs = [rhs.clone() for _ in range(2)]
        out = None
        for i in range(3):
            bufs[i % 2].copy_(rhs)
            out = fn(bufs[i % 2])
        ts, extra = [], []
        for i in range(steps):
            b = bufs[i % 2]
            b.copy_(rhs)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            out = fn(b)
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
            extra.append(out)
        return float(np.median(ts)), b, extra[-1]

    steps = max(args.steps // 2, 8)
    t64, p64, _ = timed(lambda b: P.solver(b), steps)
    p64 = p64.clone()
    res = {}
    for tol in (1e-6, 1e-10):
        tm, pm, (rr, its) = timed(lambda b: P.solve_mixed(b, tol=tol, max_iter=10), steps)
        d = pm[1:-1, 1:-1, 1:-1] - p64[1:-1, 1:-1, 1:-1]
        err = float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(p64[1:-1, 1:-1, 1:-1]))
        res[f"mixed_{tol:g}"] = {"ms": round(tm, 4), "solves_per_s": round(1e3 / tm, 2), "relres": rr,
                                 "fp32_solves": its, "rel_l2_vs_fp64": err}
    info = P.info()
    return {"mode": "c3", "workload": "Poisson solve 512x512x256, tanh-stretched z (gr 2), BC NN/PP/ND, k^-5/3 RHS",
            "fp64": {"ms": round(t64, 4), "solves_per_s": round(1e3 / t64, 2),
                     "hbm_gbs_48B": round(48 * nx * ny * nz / t64 / 1e6, 1)},
            **res, "xy_path_fp32": info["xy_path_fp32"], "xy_path_fp64": info["xy_path_fp64"],
            "timing": "CUDA events per solve (median), RHS reloaded untimed"}

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-oracle", action="store_true", help="skip the oracle step that checks the headline step")
    ap.add_argument("--no-extras", action="store_true",
                    help="leave the batch (512 grids) and serving (request stream) summaries out of the headline line")
    ap.add_argument("--serve-requests", type=int, default=4000,
                    help="requests of the serving summary in the headline line")
    ap.add_argument("--single", action="store_true",
                    help="only the headline mode (for profiler captures): W warm-up + K steps, no extra modes, "
                         "no e2e, no CPU baseline")
    ap.add_argument("--precision", type=int, default=1, help="with --single: 1 mixed to 1e-10, 0 FP64")
    ap.add_argument("--mode", choices=["projection", "batch", "serve", "c1", "c3", "solve"], default="projection",
                    help="projection: the headline two-phase step; batch: 512 uneven grids in one graph; "
                         "serve: Poisson request stream through the continuous-batching server")
    ap.add_argument("--grids", type=int, default=512)
    ap.add_argument("--requests", type=int, default=4000)
    ap.add_argument("--slots", type=int, default=4)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--rates", type=float, nargs="+", default=[0.5, 0.8, 1.0, 1.2])
    ap.add_argument("--grid", type=int, nargs=3, default=[256, 256, 32], help="--mode solve: nx ny nz")
    ap.add_argument("--cbc", default="PPPPNN", help="--mode solve: pressure BCs")
    ap.add_argument("--tol", type=float, default=1e-10, help="--mode solve: mixed tolerance (0: FP64 solver)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "ours" and args.mode != "projection":
        res = {"batch": run_batch, "serve": run_serve, "c1": run_config1, "c3": run_config3,
               "solve": run_solve}[args.mode](args)
    elif args.impl == "reference":
        res = run_reference(args, rank)
    else:
        if world > 1:
            import torch
            torch.cuda.set_device(local_rank)
            torch.distributed.init_process_group("nccl")
        res = run_ours(args, rank, world, local_rank)
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
