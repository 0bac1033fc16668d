"""Long runs of the production-size workloads to their final radius, opt-in.

Config 2 (MA, 2048 x 4 x 512 bins, 0.5-80 MeV, 4e51 erg/s): mixed precision
and double-float against FP64 at r = 1500 km, for the inverted (dm2 < 0) and
normal (dm2 > 0) hierarchy (src/Parser.cpp:99-100), from r = 50 km (the
stiff 10 -> 50 km stretch alone takes about 1e7 iterations, several GPU-hours
at this size).  The runs end at exactly Rn, so they are compared at the same
radius whatever steps each took: max |dP_ee(E)| over every nu_e beam and the
max per-beam survival-probability error (src/IO_f.cpp:341-351).

The batched sweep (xflat_gb300.sweep, config 4): its eight smallest
instances (124 K to 242 K bins each, mixed hierarchies and luminosities) run
from r = 50 km to their final radius of 600 km as one double-float batch and
one FP64 batch, compared the same way at 600 km.

Bars: double-float within 1e-5 of FP64 (the accuracy target of the faster
variants).  A batch
instance that misses it free-running is examined: FP64's own accepted steps
replayed in double-float, and FP64 with the tolerance moved by 1e-4 relative;
on such an ill-conditioned trajectory the replayed difference must stay
below a tenth of that FP64 tolerance sensitivity (measured on GB300 for
instance 58: replayed 6.3e-5 against a sensitivity of 1.7e-3, where instance
7's is 6.0e-6).  Mixed precision is recorded, not asserted (it is not expected to hold 1e-5 through long runs:
see tests/test_gpu_full_run.py).  Set XF_LONG_RUNS=1 to run (about 20
GPU-minutes); XF_LONG_RUNS_OUT=<file> saves the numbers as JSON;
XF_LONG_RUNS_ONLY (comma-separated: inverted, normal, batch) selects parts."""
import json
import os

import numpy as np
import pytest

import xflat_gb300 as xg
from helpers import derive, replay_inputs

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(os.environ.get("XF_LONG_RUNS") != "1",
                                 reason="runs to 1500 km take ~20 GPU-minutes: set XF_LONG_RUNS=1")]

RESULTS = {}
ONLY = [x for x in os.environ.get("XF_LONG_RUNS_ONLY", "").split(",") if x]


def _selected(part):
    if ONLY and part not in ONLY:
        pytest.skip("not selected by XF_LONG_RUNS_ONLY")


def pee(psi):
    x = psi[0::4]
    return x[:, 0] ** 2 + x[:, 1] ** 2


def _save():
    out = os.environ.get("XF_LONG_RUNS_OUT")
    if out:
        with open(out, "w") as f:
            json.dump(RESULTS, f, indent=1, sort_keys=True)


@pytest.mark.parametrize("hierarchy,dm2", [("inverted", "-3E-3"), ("normal", "3E-3")])
def test_config2_to_1500km(hierarchy, dm2):
    _selected(hierarchy)
    runs = {}
    for prec in ("fp64", "df", "mixed"):
        text = derive("config1_ma.txt", R0=50, dr="1.5e-4", Rn=1500, dm2=dm2, precision=prec)
        s = xg.Simulation(xg.Config.from_text(text))
        o = s.evolutionLoop(max_iters=-1, device_control=True)
        assert o["status"] == 0 and o["r_end"] == 1500.0, o
        runs[prec] = (o, pee(s.get_state(0)), s.survival().copy())
        s.close()
    res = {"r_km": [50.0, 1500.0], "bins": 2048 * 4 * 512}
    for prec, (o, p, sv) in runs.items():
        res[prec] = {"iterations": o["iterations"], "accepted": o["accepted"], "seconds": o["device_ms"] * 1e-3}
        if prec != "fp64":
            res[prec]["max_dPee_vs_fp64"] = float(np.max(np.abs(p - runs["fp64"][1])))
            res[prec]["max_dsurvival_vs_fp64"] = float(np.max(np.abs(sv - runs["fp64"][2])))
    RESULTS["config2_" + hierarchy] = res
    _save()
    assert res["df"]["max_dPee_vs_fp64"] <= 1e-5
    assert res["df"]["max_dsurvival_vs_fp64"] <= 1e-5


def test_batched_sweep_subset_to_600km():
    _selected("batch")
    from xflat_gb300.sweep import sweep_configs
    sizes = [xg.Config.from_text(t) for t in sweep_configs(seed=4, n=64)]
    pick = sorted(range(64), key=lambda i: sizes[i].abins * sizes[i].ebins)[:8]
    texts = {p: [derive(sweep_configs(seed=4, n=64, precision=p)[i], R0=50, dr="1.5e-4") for i in pick]
             for p in ("fp64", "df")}
    runs = {}
    for prec, ts in texts.items():
        b = xg.Batch([xg.Config.from_text(t) for t in ts])
        r = b.run(max_iters=-1)
        assert all(x == 600.0 for x in r["r_end"]), r["r_end"]
        runs[prec] = (r, [b.get_state(i) for i in range(len(ts))])
        b.close()
    d = [float(np.max(np.abs(pee(a) - pee(c)))) for a, c in zip(runs["fp64"][1], runs["df"][1])]
    # an instance that misses the bar free-running is examined on the single-instance paths: FP64's
    # own accepted steps replayed in double-float (the arithmetic alone), and FP64 itself with the
    # tolerance moved by 1e-4 relative (how well the method determines P_ee on that trajectory)
    checked = {}
    for k, i in enumerate(pick):
        if d[k] <= 1e-5:
            continue
        a = xg.Simulation(xg.Config.from_text(texts["fp64"][k]))
        oa = a.evolutionLoop(max_iters=-1, device_control=True, log_cap=2000000)
        c = xg.Simulation(xg.Config.from_text(texts["df"][k]))
        rb, dr = replay_inputs(texts["fp64"][k], oa["log"][:oa["accepted"]])
        c.replay(rb, dr)
        e = xg.Simulation(xg.Config.from_text(derive(texts["fp64"][k], eps0="1.0001E-9")))
        e.evolutionLoop(max_iters=-1, device_control=True)
        checked[str(i)] = {"replayed_dPee": float(np.max(np.abs(pee(a.get_state(0)) - pee(c.get_state(0))))),
                           "fp64_tolerance_sensitivity": float(np.max(np.abs(pee(a.get_state(0)) - pee(e.get_state(0)))))}
    RESULTS["batch_subset_600km"] = {
        "instances": pick, "r_km": [50.0, 600.0],
        "iterations_fp64": list(runs["fp64"][0]["iterations"]), "iterations_df": list(runs["df"][0]["iterations"]),
        "seconds_fp64": runs["fp64"][0]["seconds"], "seconds_df": runs["df"][0]["seconds"],
        "free_running_dPee": d, "examined": checked}
    _save()
    for i, c in checked.items():
        # double-float's deviation must stay well inside the method's own uncertainty there
        assert c["replayed_dPee"] <= max(1e-5, 0.1 * c["fp64_tolerance_sensitivity"]), (i, c)
