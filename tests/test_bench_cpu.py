"""CPU tests of bench.py: the reference arm's JSON line (the contract the
driver reads) and the time-stepping semantics of the projection step.

The CPU step (oracle restatement) performs the same sequence as the GPU step,
including the app's `pold = p` (src/apps/two_phase_inc_isot/
main__two_phase_inc_isot.f90:655-674).  Without it the Dodd-Ferrante
extrapolation 2p - pold feeds on itself and |p| doubles every step.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "24",
                        "--steps", "2", "--warmup", "3"], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["warmup"] >= 3 and d["steps"] == 2
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["unit"] == d["unit"]


def test_repeated_steps_stay_bounded(oracle):
    """Twenty CPU projection steps on the bench's kind of fields: with pold = p each
    step, |p| grows at most slowly (it doubled every step without it)."""
    sys.path.insert(0, ROOT)
    import bench
    n = 16
    O, S, dzci, dzfi, dz = bench.cpu_setup(n)
    rng = np.random.default_rng(5)
    shp = (n + 2,) * 3
    f = {"u": rng.uniform(-1, 1, shp), "v": rng.uniform(-1, 1, shp), "w": rng.uniform(-1, 1, shp),
         "p": rng.standard_normal(shp), "pold": rng.standard_normal(shp),
         "rho": np.where(rng.uniform(0, 1, shp) > 0.7, 1000.0, 1.0)}
    peak = []
    for _ in range(20):
        p_n = f["p"].copy()
        bench.cpu_step(O, S, n, f, dzci, dzfi, dz)
        # pold now holds p^n: the interior copy, with boundp's ghosts
        assert np.array_equal(f["pold"][1:-1, 1:-1, 1:-1], p_n[1:-1, 1:-1, 1:-1])
        peak.append(np.abs(f["p"]).max())
    assert np.all(np.isfinite(f["p"]))
    # no advection: p accumulates the corrections, but sub-exponentially (doubling per step
    # would give a factor 1024 between steps 10 and 20)
    assert peak[19] < 8 * peak[9], peak


def test_accuracy_block_states_parity_and_the_div_bound():
    """The headline's accuracy block says, in so many words, whether each form meets
    max|div u| <= 1e-11 U/dx and whether the FP64 form is within 1e-12 of the oracle."""
    sys.path.insert(0, ROOT)
    import bench
    vs = {"fp64_vs_oracle_rel_l2_phi": 3e-14, "fp64_vs_oracle_rel_l2_u": 1e-15,
          "mixed_vs_oracle_rel_l2_phi": 2e-12, "mixed_vs_oracle_rel_l2_u": 4e-9, "oracle_max_div_after": 1e-12}
    a = bench.accuracy_block(256, 1.5e-12, 2e-12, 4e-9, 5.0e-9, 1.1e-12, vs)
    assert a["div_bound"] == 256e-11
    assert a["mixed_meets_div_bound"] is False and a["fp64_meets_div_bound"] is True
    assert a["fp64_parity_1e-12"] is True and a["oracle_max_div_after"] == 1e-12
    b = bench.accuracy_block(256, 1e-13, 0, 0, 1e-9, 1e-12, None)
    assert b["mixed_meets_div_bound"] is True and "fp64_parity_1e-12" not in b


def test_cpu_first_step_is_the_oracle_step(oracle):
    """The oracle step the bench compares the GPU forms with: one cpu_step on the
    pristine fields, and the max|div u| it leaves within the bound."""
    sys.path.insert(0, ROOT)
    import bench
    n = 16
    fields = {k: t.numpy() for k, t in bench.make_fields(n, 3, "cpu").items()}
    st = bench.cpu_first_step(n, fields)
    O, S, dzci, dzfi, dz = bench.cpu_setup(n)
    f = {k: a.copy() for k, a in fields.items()}
    bench.cpu_step(O, S, n, f, dzci, dzfi, dz)
    for k in ("u", "v", "w", "p", "pold"):
        assert np.array_equal(st["f"][k], f[k]), k
    assert st["max_div"] <= 1e-11 * n
