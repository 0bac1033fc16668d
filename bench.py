#!/usr/bin/env python
"""Benchmark of the per-radius-step hot path on GB300.

One "step" is one stepper iteration (the three-point stage schedule, the error
estimate and the accept/reject/dr control of src/Nmr.cpp:153-249) over every
bin of the workload.  The workload is the plain-FP64 MA bulb run at production
size: 2048 angle bins x 4 particles x 512 energy bins (0.5-80 MeV, 4e51 erg/s,
inverted hierarchy), 4,194,304 bins, started at r = 50 km with seeded noise.
Throughput is bin-iterations per second (beam * energy * steps / s), counting
rejected iterations as the reference's own counter does (src/Nmr.cpp:246).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank runs an independent replica on its own GPU
(the path is one simulation per GPU; there is no collective on the data path);
rank 0 prints one JSON line with the whole-job aggregate.
"""
import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "beam·energy·steps/s on 1 GB300: FP64 vs mixed vs batched; max|ΔP_ee| vs FP64"
UNIT = "beam·energy·steps/s"
WORKLOAD_CFG = os.path.join(ROOT, "xflat_gb300", "configs", "config1_ma.txt")
R_START, DR_START = 50.0, 1.5e-4
WORKLOAD = ("MA bulb, FP64: 2048 angle x 4 particle x 512 energy bins (0.5-80 MeV), L=4e51 erg/s, IH, "
            "tol 1e-9, from r=50 km, seeded noise 1e-7")
# Algorithmic FP operations per bin of each phase kernel, from the reference's
# stage arithmetic (add/mul counted singly, sqrt/sin/cos/div as one each):
# phase A = S2 + S6 (2 x evolveBinsHvv: 2 x (61 + 4 special)), phase B = S4/S5 +
# S8 (47 + 61 + 8 special), phase C = S10/S11 + calcErrHvv (47 + 35 + 4
# special); 332 per bin-iteration in total.
PHASE_OPS = {"A": 130, "B": 116, "C": 86}
# Algorithmic HBM bytes per bin of each phase kernel (FP64 state, 32 B per
# bin): A reads psi0, writes psi1, psi3; B reads psi0, psi1, writes psi1, psi4;
# C reads psi3, psi4, psi1, writes psi4.
PHASE_BYTES = {"A": 96, "B": 128, "C": 128}
PHASE_KERNEL = {"A": "k_phaseA", "B": "k_phaseB", "C": "k_phaseC"}


def workload_text(path=WORKLOAD_CFG, **over):
    text = open(path).read()
    for k, v in over.items():
        text, n = re.subn(r"^%s=.*$" % re.escape(k), "%s= %s" % (k, v), text, flags=re.M)
        if n != 1:
            raise ValueError(k)
    return text


def aggregate_replicas(units, seconds):
    """Whole-job throughput of independent replicas: the units all ranks
    processed over the slowest rank's time."""
    t = max(seconds)
    return sum(units) / t if t > 0 else float("nan"), t


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        if self.path and os.path.exists(self.path):
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    rows.append(dict(sm=float(parts[1]), smmax=float(parts[2]), power=float(parts[3]),
                                     hw=parts[5], hwt=parts[6], swt=parts[7], swp=parts[8]))
                except ValueError:
                    continue
            os.remove(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        reasons = []
        for key, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"), ("swt", "sw_thermal_slowdown"),
                          ("swp", "sw_power_cap")):
            if any(r[key].lower() == "active" for r in rows):
                reasons.append(name)
        return {"sm_mhz": statistics.median(r["sm"] for r in rows), "sm_max_mhz": max(r["smmax"] for r in rows),
                "power_w_max": max(r["power"] for r in rows), "reasons": reasons, "samples": len(rows)}


def profiled_traffic(phase):
    """DRAM bytes per launch of a phase kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "%s_config1.md" % PHASE_KERNEL[phase])
    if not os.path.exists(path):
        return None
    m = re.search(r"dram_bytes_per_launch:\s*([0-9.eE+]+)", open(path).read())
    return float(m.group(1)) if m else None


def pinned_empty(n):
    """Pinned host buffer (float64) for the end-to-end leg."""
    try:
        import torch
        t = torch.empty(n, dtype=torch.float64, pin_memory=True)
        return t.numpy(), True
    except Exception:
        import numpy as np
        return np.empty(n), False


def cpu_baseline(text, r0, dr0, target_s=15.0):
    """The oracle's C restatement (oracle/_build/xfport, OpenMP on every host
    core) on a bounded sample of the same workload."""
    exe = os.path.join(ROOT, "oracle", "_build", "xfport")
    if not os.path.exists(exe):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "port"], check=True, capture_output=True)
    cores = os.cpu_count() or 1
    env = dict(os.environ, OMP_NUM_THREADS=str(cores), OMP_PROC_BIND="close")
    fd, path = tempfile.mkstemp(suffix=".txt")
    with os.fdopen(fd, "w") as f:
        f.write(text)
    try:
        def run(n):
            out = subprocess.run([exe, path, "--iters", str(n), "--r0", repr(r0), "--dr", repr(dr0)], env=env,
                                 capture_output=True, text=True, check=True)
            return json.loads(out.stdout.strip().splitlines()[-1])
        probe = run(2)
        per_it = probe["seconds"] / max(1, probe["iterations"])
        n = int(max(3, min(2000, target_s / max(per_it, 1e-6))))
        res = run(n)
    finally:
        os.remove(path)
    return {"value": res["bin_iter_per_s"], "unit": UNIT, "cores": res["threads"], "kind": "port",
            "sample": "%d stepper iterations of the same workload from r=%g km (%.1f s of CPU time)"
                      % (res["iterations"], r0, res["seconds"])}


def workload_config():
    """The `config` of both arms' lines: the same workload, the same start."""
    return {"workload": WORKLOAD, "bins": 2048 * 4 * 512, "r0_km": R_START, "dr0_km": DR_START,
            "start": "seeded noise state (seed 1, amplitude 1e-7) at r0; every timed run starts there",
            "l2": "inputs larger than L2 (four 134 MB state buffers)"}


def reference_arm(args, rank):
    """CPU implementation of the path on this host's cores: the reference built
    from its own sources (oracle/_ref) where it exists and runs, else the
    oracle's C restatement of it.  Like the GPU arm, the warm-up and the timed
    run each start from the workload's start state at r0."""
    if rank != 0:
        return 0
    text = workload_text(R0=R_START, dr=DR_START)
    cores = os.cpu_count() or 1
    env = dict(os.environ, OMP_NUM_THREADS=str(cores), OMP_PROC_BIND="close")
    ref_exe = os.path.join(ROOT, "oracle", "_ref", "xflat_ref_ma")
    kind = "port"
    fd, path = tempfile.mkstemp(suffix=".txt")
    os.close(fd)

    def run(n):
        nonlocal kind
        if os.path.exists(ref_exe):
            with open(path, "w") as f:
                f.write(re.sub(r"^Ts=.*$", "Ts= %d" % n, text, flags=re.M))
            try:
                out = subprocess.run([ref_exe, path, "--noise", "1", "1e-7"], env=env, capture_output=True, text=True,
                                     check=True)
                kind = "reference"
                d = json.loads(out.stdout.strip().splitlines()[-1])
                return d["iterations"], d["seconds"], d["beams"] * d["ebins"]
            except (subprocess.CalledProcessError, OSError, ValueError):
                pass
        exe = os.path.join(ROOT, "oracle", "_build", "xfport")
        if not os.path.exists(exe):
            subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "port"], check=True, capture_output=True)
        with open(path, "w") as f:
            f.write(text)
        out = subprocess.run([exe, path, "--iters", str(n)], env=env, capture_output=True, text=True, check=True)
        kind = "port"
        d = json.loads(out.stdout.strip().splitlines()[-1])
        return d["iterations"], d["seconds"], d["bins"]

    try:
        run(max(1, args.warmup))
        it, secs, bins = run(args.steps)
    finally:
        os.remove(path)
    value = bins * it / secs
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": it, "warmup": args.warmup,
        "ms_per_step": 1e3 * secs / it, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic", "impl": "reference", "config": workload_config(),
        "parallelism": "OpenMP over angle bins, host cores",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": "%d stepper iterations of the workload from r0, loop wall time" % it},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def pee(psi):
    """P_ee(E) = |a(E)|^2 of the nu_e beams (particle index 0)."""
    x = psi[0::4]
    return x[:, 0] ** 2 + x[:, 1] ** 2


def set_precision(text, prec):
    return re.sub(r"^precision=.*$", "precision= " + prec, text, flags=re.M)


def replay_inputs(r0, log):
    """(r_before, dr) of a run's accepted steps, in order (r += dr, src/Nmr.cpp:229)."""
    import numpy as np
    rb = np.concatenate([[r0], log[:-1, 1]]) if len(log) else np.zeros(0)
    return rb, log[:, 2].copy()


def accuracy_vs(xg, text, prec, psi_start, r0, log, psi_ref, surv_ref):
    """The run forced onto the FP64 run's accepted steps in precision `prec`
    (xf_replay): max |dP_ee(E)| over every nu_e beam and max per-beam
    survival-probability error (the src/IO_f.cpp:341-351 quantity) against
    FP64 at the same radius.  Always computed, whatever steps the free-running
    variant took."""
    import numpy as np
    m = xg.Simulation(xg.Config.from_text(set_precision(text, prec)))
    m.set_state(psi_start)
    rb, dr = replay_inputs(r0, log)
    m.replay(rb, dr)
    out = {"max_dPee_vs_fp64": float(np.max(np.abs(pee(m.get_state(0)) - pee(psi_ref)))),
           "max_dsurvival_vs_fp64": float(np.max(np.abs(m.survival() - surv_ref))),
           "compared_on": "the FP64 run's %d accepted steps replayed" % len(rb)}
    m.close()
    return out


def timed_run(xg, text, psi_start, r0, dr0, steps, warmup, log=False, options=None):
    """Device-controlled run of `steps` iterations from (r0, dr0) and the
    start state, after `warmup` iterations from the same start, in the
    library's default launch form (a persistent cooperative launch where that
    is faster); then the same steps again with per-phase CUDA events (the
    graph-launched form), for the phase times."""
    sim = xg.Simulation(xg.Config.from_text(text))
    for k, v in (options or {}).items():
        sim.lib.xf_set_option(sim.h, k.encode(), float(v))
    sim.set_state(psi_start)
    sim.evolutionLoop(max_iters=max(3, warmup), device_control=True, iters_per_launch=16, r0=r0, dr0=dr0)
    sim.set_state(psi_start)
    sim.evolutionLoop(max_iters=steps, device_control=True, iters_per_launch=16, r0=r0, dr0=dr0, time_phases=True)
    sim.set_state(psi_start)
    out = sim.evolutionLoop(max_iters=steps, device_control=True, iters_per_launch=16, r0=r0, dr0=dr0,
                            log_cap=steps if log else 0)
    return sim, out


VARIANT_WORKLOAD = {
    "mixed": "precision= mixed (FP32 rotations and compensated FP32 state; FP64 moment reduction, error estimate, "
             "control, renormalisation)",
    "df": "precision= df (every state, propagator, average and moment in double-float FP32 pairs; FP64 block "
          "reduction and control)",
}


def variant_leg(xg, prec, text, psi_start, r0, dr0, steps, bins, log64, psi64, surv64, st64, warmup=3):
    """The same K steps from the same state in another precision: speed of the
    free run, accuracy on FP64's own accepted steps."""
    m, out = timed_run(xg, set_precision(text, prec), psi_start, r0, dr0, steps, warmup)
    ms, _ = m.phase_times()
    m.close()
    res = {"value": bins * out["iterations"] / (out["device_ms"] * 1e-3), "unit": UNIT,
           "ms_per_step": out["device_ms"] / max(1, out["iterations"]), "phases_ms": dict(zip("ABC", map(float, ms))),
           "iterations": out["iterations"], "accepted": out["accepted"], "accepted_fp64": st64["accepted"],
           "speedup_vs_fp64": None, "workload": VARIANT_WORKLOAD[prec]}
    res.update(accuracy_vs(xg, text, prec, psi_start, r0, log64, psi64, surv64))
    return res


def shape_leg(xg, name, text, r0, dr0, steps, warmup):
    """FP64, mixed and double-float on one workload shape: ms per iteration and
    bin-iterations per second of each, accuracy of the others against FP64 on
    FP64's accepted steps."""
    sim = xg.Simulation(xg.Config.from_text(text))
    psi0 = sim.get_state(0).copy()
    bins = sim.nbeams * sim.ebins
    sim.close()
    s64, o64 = timed_run(xg, text, psi0, r0, dr0, steps, warmup, log=True)
    psi64, surv64 = s64.get_state(0).copy(), s64.survival().copy()
    s64.close()
    out = {"workload": name, "bins": bins, "r0_km": r0, "r_end_km": o64["r_end"], "iterations": o64["iterations"],
           "fp64": {"ms_per_step": o64["device_ms"] / max(1, o64["iterations"]),
                    "value": bins * o64["iterations"] / (o64["device_ms"] * 1e-3)}}
    for prec in ("mixed", "df"):
        v = variant_leg(xg, prec, text, psi0, r0, dr0, steps, bins, o64["log"], psi64, surv64, o64, warmup)
        v["speedup_vs_fp64"] = v["value"] / out["fp64"]["value"]
        out[prec] = v
    return out


def long_window_leg(xg, iters):
    """Double-float (and mixed) against FP64 over a long free-running window of
    the config-0 physics (256 x 4 x 64 bins from r = 50 km): the step
    sequences and max |dP_ee(E)| at the end, replayed on FP64's steps where
    the free runs' step counts differ."""
    import numpy as np
    text = workload_text(os.path.join(ROOT, "xflat_gb300", "configs", "config0_ma.txt"), R0=50, dr="1.5e-4")
    a = xg.Simulation(xg.Config.from_text(text))
    psi0 = a.get_state(0).copy()
    oa = a.evolutionLoop(max_iters=iters, device_control=True, log_cap=iters)
    pa, sa = a.get_state(0).copy(), a.survival().copy()
    a.close()
    out = {"workload": "config-0 physics, 256 x 4 x 64 bins, free-running from r = 50 km",
           "iterations": oa["iterations"], "r_km": [50.0, oa["r_end"]], "fp64_seconds": oa["device_ms"] * 1e-3}
    for prec in ("df", "mixed"):
        b = xg.Simulation(xg.Config.from_text(set_precision(text, prec)))
        ob = b.evolutionLoop(max_iters=iters, device_control=True)
        same = (ob["iterations"], ob["accepted"]) == (oa["iterations"], oa["accepted"]) and ob["r_end"] == oa["r_end"]
        res = {"accepted": ob["accepted"], "accepted_fp64": oa["accepted"], "same_step_sequence_end": same,
               "seconds": ob["device_ms"] * 1e-3}
        if same:
            res["max_dPee_vs_fp64"] = float(np.max(np.abs(pee(b.get_state(0)) - pee(pa))))
            res["max_dsurvival_vs_fp64"] = float(np.max(np.abs(b.survival() - sa)))
            res["compared_on"] = "free runs ending at the same radius after the same steps"
        else:
            res.update(accuracy_vs(xg, text, prec, psi0, 50.0, oa["log"][:oa["accepted"]], pa, sa))
        b.close()
        out[prec] = res
    return out


def batched_leg(xg, steps):
    """The batched parameter sweep (64 independent MA instances from a seed,
    xflat_gb300.sweep): double-float, mixed precision and FP64 in one batch
    each, and the same 64 instances run back to back through the
    single-simulation FP64 path."""
    import numpy as np
    from xflat_gb300.sweep import sweep_configs
    out = {"workload": "64 MA instances (seed 4): angle bins U{128..2048}, energy bins U{32..512} (1-60 MeV), "
                       "L log-U[1e50,1e52] erg/s, NH/IH p=1/2, lambda0 log-U[1e2,1e4] /km, from r=10 km",
           "steps_per_instance": steps}
    states = {}
    for prec in ("df", "mixed", "fp64"):
        b = xg.Batch([xg.Config.from_text(t) for t in sweep_configs(seed=4, n=64, precision=prec)])
        r = b.run(max_iters=steps)
        units = sum(nb * ne * i for (nb, ne), i in zip(b.dims, r["iterations"]))
        out["bins"] = sum(nb * ne for nb, ne in b.dims)
        t = b.tuning()
        out["batched_" + prec] = {"value": units / r["seconds"], "unit": UNIT, "seconds": r["seconds"],
                                  "tile": {"warps_per_block": t["warps"], "beams_per_warp": t["beams_per_warp"],
                                           "launch": "persistent" if t["persistent"] else "graphs",
                                           "candidates_ms": {"%s %dx%d" % ("persistent" if p else "graphs", w, bp):
                                                             round(ms, 3) for w, bp, p, ms in t["candidates"]}}}
        states[prec] = ([b.get_state(i)[0::4, :2] for i in range(len(b.dims))], list(r["accepted"]))
        b.close()
    units, ms = 0, 0.0
    for t in sweep_configs(seed=4, n=64, precision="fp64"):
        s = xg.Simulation(xg.Config.from_text(t))
        o = s.evolutionLoop(max_iters=steps, device_control=True)
        units += s.nbeams * s.ebins * o["iterations"]
        ms += o["device_ms"]
        s.close()
    out["fp64_back_to_back"] = {"value": units / (ms * 1e-3), "unit": UNIT}
    for prec in ("df", "mixed"):
        out["speedup_batched_%s_vs_fp64_back_to_back" % prec] = (out["batched_" + prec]["value"] /
                                                                 out["fp64_back_to_back"]["value"])
        d, diverged = [], 0
        for a, c, na, nc in zip(states["fp64"][0], states[prec][0], states["fp64"][1], states[prec][1]):
            if na != nc:
                diverged += 1
                continue
            d.append(np.max(np.abs((a[:, 0] ** 2 + a[:, 1] ** 2) - (c[:, 0] ** 2 + c[:, 1] ** 2))))
        out["max_dPee_batched_%s_vs_fp64" % prec] = float(max(d)) if d else None
        out["instances_compared_" + prec] = len(d)
        out["instances_with_other_step_count_" + prec] = diverged
    return out


def whole_run_record():
    """The opt-in whole-run test's measured result (tests/test_gpu_full_run.py),
    committed in profiles/whole_run_config0.md as a line `record: {json}`:
    recorded, not measured by this run."""
    path = os.path.join(ROOT, "profiles", "whole_run_config0.md")
    if not os.path.exists(path):
        return None
    m = re.search(r"^record: (\{.*\})\s*$", open(path).read(), re.M)
    if not m:
        return None
    rec = json.loads(m.group(1))
    rec["source"] = "profiles/whole_run_config0.md (tests/test_gpu_full_run.py on a GB300; not measured by this run)"
    return rec


def ours(args, rank, world, dist):
    import numpy as np
    import xflat_gb300 as xg

    lib = xg.load()
    text = workload_text(R0=R_START, dr=DR_START)
    sim = xg.Simulation(xg.Config.from_text(text))
    bins = sim.nbeams * sim.ebins
    state_bytes = bins * 4 * 8
    psi_start = sim.get_state(0).copy()

    # --- warm-up, then the timed region: K device-controlled iterations from the
    # start state at r0 with the inputs resident in HBM (4 state buffers of 134
    # MB each: larger than L2)
    sim.evolutionLoop(max_iters=max(3, args.warmup), device_control=True, iters_per_launch=16)
    sim.set_state(psi_start)
    if dist:
        dist.barrier()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clocks:
        # FP64 at this size runs graph-launched phases; their CUDA events give the phase times
        st = sim.evolutionLoop(max_iters=args.steps, device_control=True, iters_per_launch=min(16, args.steps),
                               r0=R_START, dr0=DR_START, time_phases=True, log_cap=args.steps)
    if dist:
        dist.barrier()
    phase_ms, phase_n = sim.phase_times()
    secs = st["device_ms"] * 1e-3
    units = bins * st["iterations"]
    psi_fp64_end = sim.get_state(0).copy()
    surv_fp64 = sim.survival()
    log64 = st["log"][:st["accepted"]]

    # --- end to end through the C ABI with host buffers: state H2D from pinned
    # memory (xf_set_state), the loop through xf_run, state D2H into pinned
    # memory (xf_get_state), all inside the host-clock timed region; the byte
    # counts add the copies xf_run reports.  The headline runs xf_run as the
    # integration module calls it when no files are written (device-controlled
    # stepping: the control block comes back once per launch of 16
    # iterations); the host-driven form (the reference's loop structure: per
    # iteration r, dr and the three matter terms H2D, Max_err D2H) is reported
    # beside it.
    host_psi, pinned = pinned_empty(bins * 4)
    host_psi[:] = psi_start.reshape(-1)
    out = pinned_empty(bins * 4)[0]

    def end_to_end(device_control):
        t0 = time.perf_counter()
        sim.set_state(host_psi)
        e = sim.evolutionLoop(max_iters=args.steps, device_control=device_control, r0=R_START, dr0=DR_START)
        sim.get_state(0, out=out)
        return time.perf_counter() - t0, e

    e2e_s, e = end_to_end(True)
    e2e_units = bins * e["iterations"]
    hd_s, ehd = end_to_end(False)
    hd_value = bins * ehd["iterations"] / hd_s
    sim.close()

    # --- aggregation over replicas
    if dist:
        import torch
        t = torch.tensor([secs, e2e_s, float(units), float(e2e_units)], dtype=torch.float64)
        gathered = [torch.zeros_like(t) for _ in range(world)]
        dist.all_gather(gathered, t)
        g = [x.tolist() for x in gathered]
        value, tmax = aggregate_replicas([x[2] for x in g], [x[0] for x in g])
        e2e_value, _ = aggregate_replicas([x[3] for x in g], [x[1] for x in g])
    else:
        value, tmax = aggregate_replicas([units], [secs])
        e2e_value, _ = aggregate_replicas([e2e_units], [e2e_s])
    if rank != 0:
        return 0

    # --- the same K steps in the other precisions (speed of the free runs,
    # accuracy on FP64's accepted steps), normal hierarchy, the other
    # workload shapes, a long window, the batched sweep
    variants = {"fp64": {"value": value, "unit": UNIT}}
    whole = whole_run_record()
    for prec in ("mixed", "df"):
        v = variant_leg(xg, prec, text, psi_start, R_START, DR_START, args.steps, bins, log64, psi_fp64_end,
                        surv_fp64, st)
        v["speedup_vs_fp64"] = v["value"] / value
        variants[prec] = v
    if whole:
        # recorded by the opt-in whole-run test, not measured by this run (see "whole_run")
        variants["df"]["whole_run_max_dPee_vs_fp64"] = whole.get("df_vs_fp64_max_dPee")
    extra = {}
    if not args.quick:
        nh = workload_text(R0=R_START, dr=DR_START, dm2="3E-3")
        extra["normal_hierarchy"] = shape_leg(
            xg, "as the FP64 line with normal hierarchy (dm2 = +3e-3 eV^2)", nh, R_START, DR_START,
            min(args.steps, 50), 3)
        extra["config0_shape"] = shape_leg(
            xg, "config-0 physics, 256 x 4 x 64 bins (65,536; 1e51 erg/s), from r = 10 km: latency-bound",
            workload_text(os.path.join(ROOT, "xflat_gb300", "configs", "config0_ma.txt")), 10.0, 1e-3,
            2000, 10)
        extra["maa_config3"] = shape_leg(
            xg, "MAA 256 polar x 64 azimuthal x 4 x 128 energy bins (8.39 M; 1e51 erg/s, IH), from r = 50 km",
            workload_text(os.path.join(ROOT, "xflat_gb300", "configs", "config3_maa.txt"), R0=50, dr="1e-4"),
            50.0, 1e-4, min(args.steps, 40), 3)
        extra["long_window"] = long_window_leg(xg, args.window)
    batched = batched_leg(xg, args.batch_steps) if args.batch_steps > 0 else None

    # --- roofline of the dominant phase kernel against the live FP64 FMA peak
    peak = lib_peak(lib)
    totals = {p: phase_ms[i] * phase_n[i] for i, p in enumerate("ABC")}
    dom = max(totals, key=totals.get)
    di = "ABC".index(dom)
    avg_s = phase_ms[di] * 1e-3
    achieved = PHASE_OPS[dom] * bins / avg_s / 1e12
    hbm_achieved = PHASE_BYTES[dom] * bins / avg_s / 1e9
    traffic = profiled_traffic(dom)
    peaks = {}
    pk_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk_path):
        peaks = json.load(open(pk_path))
    hbm_peak = peaks.get("hbm_gbs")

    cpu = cpu_baseline(text, R_START, DR_START) if not args.skip_cpu else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": st["iterations"],
        "warmup": max(3, args.warmup), "ms_per_step": 1e3 * tmax / max(1, st["iterations"]),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(),
        "run": {"precision": "fp64", "stepping": "device-controlled", "accepted": st["accepted"],
                "r_range_km": [R_START, st["r_end"]], "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None, "traffic": traffic, "kernel": PHASE_KERNEL[dom],
                     "peak_source": "FP64 FMA throughput measured live by xf_probe_fp64_peak",
                     "traffic_source": "ncu capture summarised in profiles/%s_config1.md" % PHASE_KERNEL[dom],
                     "ops_per_bin": PHASE_OPS[dom],
                     "hbm_view": {"achieved_gbs": hbm_achieved, "peak_gbs": hbm_peak,
                                  "frac": hbm_achieved / hbm_peak if hbm_peak else None,
                                  "algorithmic_bytes_per_bin": PHASE_BYTES[dom]}},
        "phases_ms": {p: phase_ms[i] for i, p in enumerate("ABC")},
        "variants": variants, "workloads": extra, "batched": batched, "whole_run": whole,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": (state_bytes + e["h2d_bytes"]) /
                max(1, e["iterations"]), "d2h_bytes_per_step": (state_bytes + e["d2h_bytes"]) /
                max(1, e["iterations"]), "pinned": pinned,
                "loop": "xf_run, device-controlled stepping (16 iterations per graph launch)",
                "host_driven": {"value": hd_value, "unit": UNIT, "iterations": ehd["iterations"],
                                "h2d_bytes_per_step": (state_bytes + ehd["h2d_bytes"]) / max(1, ehd["iterations"]),
                                "d2h_bytes_per_step": (state_bytes + ehd["d2h_bytes"]) / max(1, ehd["iterations"]),
                                "loop": "host-driven, the reference's loop structure (rank 0)"}},
        "gpu_launches": st["kernel_launches"],
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


def lib_peak(lib):
    import ctypes
    v = ctypes.c_double()
    rc = lib.xf_probe_fp64_peak(60.0, ctypes.byref(v))
    return v.value if rc == 0 else None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--skip-cpu", action="store_true", help="omit the CPU-baseline leg")
    ap.add_argument("--batch-steps", type=int, default=24, help="iterations per instance of the batched legs (0 = skip)")
    ap.add_argument("--window", type=int, default=100000,
                    help="iterations of the long double-float/mixed vs FP64 window at the config-0 shape")
    ap.add_argument("--quick", action="store_true", help="omit the other workload shapes and the long window")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        return reference_arm(args, rank)
    if world > 1:
        # one process per GPU: pin this rank to its device before CUDA starts
        os.environ["CUDA_VISIBLE_DEVICES"] = os.environ.get("LOCAL_RANK", str(rank))
        import torch.distributed as dist
        dist.init_process_group("gloo")
    else:
        dist = None
    try:
        return ours(args, rank, world, dist)
    finally:
        if dist:
            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
