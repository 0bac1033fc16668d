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


def reference_arm(args, rank):
    """CPU implementation of the path on this host's cores: the reference built
    from its own sources (oracle/_ref) where it exists and runs, else the
    oracle's C restatement of it."""
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
        "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": WORKLOAD, "bins": bins, "parallelism": "OpenMP over angle bins, host cores"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": "%d stepper iterations of the workload, loop wall time" % it},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def ours(args, rank, world, dist):
    import numpy as np
    import xflat_gb300 as xg

    lib = xg.load()
    text = workload_text(R0=R_START, dr=DR_START)
    sim = xg.Simulation(xg.Config.from_text(text))
    bins = sim.nbeams * sim.ebins
    state_bytes = bins * 4 * 8

    # --- warm-up, then the timed region: K device-controlled iterations with the
    # inputs resident in HBM (4 state buffers of 134 MB each: larger than L2)
    w = sim.evolutionLoop(max_iters=max(3, args.warmup), device_control=True, iters_per_launch=16)
    r0, dr0 = w["r_end"], w["dr_end"]
    psi_start = sim.get_state(0).copy()
    if dist:
        dist.barrier()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clocks:
        st = sim.evolutionLoop(max_iters=args.steps, device_control=True, iters_per_launch=min(16, args.steps),
                               r0=r0, dr0=dr0, time_phases=True)
    if dist:
        dist.barrier()
    phase_ms, phase_n = sim.phase_times()
    secs = st["device_ms"] * 1e-3
    units = bins * st["iterations"]
    psi_fp64_end = sim.get_state(0).copy()
    surv_fp64 = sim.survival()

    # --- mixed precision (FP32 rotations and compensated FP32 state, FP64
    # reductions/control) and double-float (every operation in FP32 pairs) on
    # the same workload: same start state, same K steps
    mixed = variant_leg(xg, "mixed", text, psi_start, r0, dr0, args.steps, bins, psi_fp64_end, surv_fp64, st)
    dfl = variant_leg(xg, "df", text, psi_start, r0, dr0, args.steps, bins, psi_fp64_end, surv_fp64, st)
    batched = batched_leg(xg, args.batch_steps) if args.batch_steps > 0 else None

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
    sim.get_state(0, out=host_psi)
    out = pinned_empty(bins * 4)[0]

    def end_to_end(device_control):
        t0 = time.perf_counter()
        sim.set_state(host_psi)
        e = sim.evolutionLoop(max_iters=args.steps, device_control=device_control, r0=r0, dr0=dr0)
        sim.get_state(0, out=out)
        return time.perf_counter() - t0, e

    e2e_s, e = end_to_end(True)
    e2e_units = bins * e["iterations"]
    hd_s, ehd = end_to_end(False)
    hd_value = bins * ehd["iterations"] / hd_s

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

    cpu = cpu_baseline(text, r0, dr0) if not args.skip_cpu else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": st["iterations"],
        "warmup": max(3, args.warmup), "ms_per_step": 1e3 * tmax / max(1, st["iterations"]),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "bins": bins, "precision": "fp64", "stepping": "device-controlled",
                   "accepted": st["accepted"], "r_range_km": [r0, st["r_end"]],
                   "l2": "inputs larger than L2 (four 134 MB state buffers per replica)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None, "traffic": traffic, "kernel": PHASE_KERNEL[dom],
                     "peak_source": "FP64 FMA throughput measured live by xf_probe_fp64_peak",
                     "ops_per_bin": PHASE_OPS[dom],
                     "hbm_view": {"achieved_gbs": hbm_achieved, "peak_gbs": hbm_peak,
                                  "frac": hbm_achieved / hbm_peak if hbm_peak else None,
                                  "algorithmic_bytes_per_bin": PHASE_BYTES[dom]}},
        "phases_ms": {p: phase_ms[i] for i, p in enumerate("ABC")},
        "variants": {"fp64": {"value": value, "unit": UNIT}, "mixed": mixed, "df": dfl, "batched": batched},
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


def pee(psi):
    """P_ee(E) = |a(E)|^2 of the nu_e beams (particle index 0)."""
    x = psi[0::4]
    return x[:, 0] ** 2 + x[:, 1] ** 2


VARIANT_WORKLOAD = {
    "mixed": "same as the FP64 line, precision= mixed (FP32 rotations and compensated FP32 state; "
             "FP64 moment reduction, error estimate, control, renormalisation)",
    "df": "same as the FP64 line, precision= df (every state, propagator, average and moment in double-float "
          "FP32 pairs; FP64 block reduction and control)",
}


def variant_leg(xg, prec, text, psi_start, r0, dr0, steps, bins, psi_fp64_end, surv_fp64, st64):
    """Run of the same K steps from the same state in another precision;
    accuracy against the FP64 run: max |dP_ee(E)| over every nu_e beam and max
    per-beam survival-probability error (src/IO_f.cpp:341-351 quantity)."""
    import numpy as np
    m = xg.Simulation(xg.Config.from_text(text.replace("precision= fp64", "precision= " + prec)))
    m.set_state(psi_start)
    out = m.evolutionLoop(max_iters=steps, device_control=True, iters_per_launch=min(16, steps), r0=r0, dr0=dr0)
    res = {"value": bins * out["iterations"] / (out["device_ms"] * 1e-3), "unit": UNIT,
           "ms_per_step": out["device_ms"] / max(1, out["iterations"]), "iterations": out["iterations"],
           "accepted": out["accepted"], "accepted_fp64": st64["accepted"], "workload": VARIANT_WORKLOAD[prec]}
    if out["accepted"] == st64["accepted"]:
        res["max_dPee_vs_fp64"] = float(np.max(np.abs(pee(m.get_state(0)) - pee(psi_fp64_end))))
        res["max_dsurvival_vs_fp64"] = float(np.max(np.abs(m.survival() - surv_fp64)))
    m.close()
    return res


def batched_leg(xg, steps):
    """The batched parameter sweep (64 independent MA instances from a seed,
    xflat_gb300.sweep): mixed precision and FP64 in one batch each, and the same
    64 instances run back to back through the single-simulation FP64 path."""
    import numpy as np
    from xflat_gb300.sweep import sweep_configs
    out = {"workload": "64 MA instances (seed 4): angle bins U{128..2048}, energy bins U{32..512} (1-60 MeV), "
                       "L log-U[1e50,1e52] erg/s, NH/IH p=1/2, lambda0 log-U[1e2,1e4] /km, from r=10 km",
           "steps_per_instance": steps}
    states = {}
    for prec in ("mixed", "fp64"):
        b = xg.Batch([xg.Config.from_text(t) for t in sweep_configs(seed=4, n=64, precision=prec)])
        r = b.run(max_iters=steps)
        units = sum(nb * ne * i for (nb, ne), i in zip(b.dims, r["iterations"]))
        out["bins"] = sum(nb * ne for nb, ne in b.dims)
        out["batched_" + prec] = {"value": units / r["seconds"], "unit": UNIT, "tile_warps": b.tile_shape()[0],
                                  "seconds": r["seconds"]}
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
    out["speedup_batched_mixed_vs_fp64_back_to_back"] = out["batched_mixed"]["value"] / out["fp64_back_to_back"]["value"]
    d = []
    for a, c, na, nc in zip(states["fp64"][0], states["mixed"][0], states["fp64"][1], states["mixed"][1]):
        if na == nc:
            d.append(np.max(np.abs((a[:, 0] ** 2 + a[:, 1] ** 2) - (c[:, 0] ** 2 + c[:, 1] ** 2))))
    out["max_dPee_batched_mixed_vs_fp64"] = float(max(d)) if d else None
    out["instances_compared"] = len(d)
    return out


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
