"""Generate the golden fixtures in tests/golden/ from the reference itself.

The reference's own hot-path sources are compiled by ``oracle/Makefile`` (target
``ref``) into ``oracle/_ref/xflat_ref_{ma,maa,sa}``; this script runs those binaries
on small configurations derived from the workload configs and stores what they
print into compressed ``.npz`` files:

* ``log``    accepted steps (iteration index, radius after the step, dr used),
             as recorded through the reference's dumpToFile hook
             (src/Nmr.cpp:238);
* ``final``  the state after the last accepted step, in the NetCDF psi layout
             [beam][comp][ebin] (the seeded initial state is regenerated from
             ``meta.seed``/``meta.noise_amp``; ``stage_psi0`` holds it verbatim);
* ``probe_*`` energy tables, matter terms, angle tables and the Hamiltonian at
             the three stage points on the initial state (src/NBeam.cpp:138-209,
             src/Matt.cpp:58-64, src/Phy_MA.cpp:172-227/455-474,
             src/Phy_MAA.cpp:194-241/571-621, src/Phy_SA.cpp:121-147/259-281);
* ``stage_*`` every stage buffer after one forced iteration (src/Nmr.cpp:153-206).

Run it from the repository root, in a checkout that has the reference sources:

    python tests/golden/make_golden.py [--ref /path/to/reference]
"""
import argparse
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CONFIGS = os.path.join(ROOT, "xflat_gb300", "configs")

# name, base config, key overrides, noise amp, outputs
CASES = [
    ("ma_small_r10", "config0_ma.txt", dict(Abins=16, Ebins=16, R0=10, dr=1e-3, Ts=300), 1e-7, "replay probe"),
    ("ma_small_r50", "config0_ma.txt", dict(Abins=16, Ebins=16, R0=50, dr=1e-4, Ts=300), 1e-7, "replay"),
    ("ma_small_r290", "config0_ma.txt", dict(Abins=16, Ebins=16, R0=290, dr=1e-2, Ts=400), 1e-7, "replay"),
    ("ma_ragged_nh", "config0_ma.txt", dict(Abins=13, Ebins=21, R0=20, dr=1e-5, Ts=200, dm2="3E-3"), 1e-7,
     "replay probe stages"),
    ("ma_nomatter", "config0_ma.txt", dict(Abins=16, Ebins=16, R0=30, dr=1e-4, Ts=200, hasMatter=0), 1e-7,
     "replay probe"),
    ("ma_c0shape", "config0_ma.txt", dict(R0=10, dr=1e-8, Ts=200), 1e-7, "replay probe"),
    ("ma_stage_r10", "config0_ma.txt", dict(Abins=16, Ebins=16, R0=10, dr=1.3e-8, Ts=1), 1e-7, "stages probe"),
    ("maa_small_r10", "config3_maa.txt", dict(Abins=16, Pbins=8, Ebins=16, R0=10, dr=1e-3, Ts=150), 1e-6,
     "replay probe"),
    ("maa_small_r50", "config3_maa.txt", dict(Abins=16, Pbins=8, Ebins=16, R0=50, dr=1e-4, Ts=150), 1e-6,
     "replay stages"),
    ("maa_ragged", "config3_maa.txt", dict(Abins=9, Pbins=5, Ebins=19, R0=12, dr=1e-6, Ts=100), 1e-6,
     "replay probe stages"),
    ("ma_c1shape_probe", "config1_ma.txt", dict(Ts=0), 1e-7, "probe"),
    ("maa_c3shape_probe", "config3_maa.txt", dict(Ts=0), 1e-6, "probe"),
    ("sa_r10", "sa_bulb.txt", dict(Ebins=64, R0=10, dr=1e-3, Ts=600), 1e-7, "replay probe stages"),
    ("sa_r60", "sa_bulb.txt", dict(R0=60, dr=1e-3, Ts=1500), 1e-7, "replay probe"),
    ("sa_ragged", "sa_bulb.txt", dict(Abins=7, Ebins=37, R0=25, dr=1e-5, Ts=400, dm2="3E-3"), 1e-7,
     "replay probe stages"),
]
EXES = {"MA": "xflat_ref_ma", "MAA": "xflat_ref_maa", "SA": "xflat_ref_sa"}
SEED = 1


def derive_config(base_text, overrides):
    text = base_text
    for k, v in overrides.items():
        text, n = re.subn(r"^%s=.*$" % re.escape(k), "%s= %s" % (k, v), text, flags=re.M)
        if n != 1:
            raise ValueError("key %s not found exactly once" % k)
    return text


def read_probe(path):
    out = {}
    with open(path, "rb") as f:
        while True:
            name = f.read(32)
            if len(name) < 32:
                break
            n = int(np.frombuffer(f.read(8), dtype=np.int64)[0])
            out[name.rstrip(b"\0").decode()] = np.frombuffer(f.read(8 * n), dtype=np.float64).copy()
    return out


def run_case(name, base, overrides, amp, outputs, refdir, tmp):
    text = derive_config(open(os.path.join(CONFIGS, base)).read(), overrides)
    cfg_path = os.path.join(tmp, name + ".txt")
    open(cfg_path, "w").write(text)
    exe = os.path.join(refdir, EXES[re.search(r"^geometry=\s*(\S+)", text, re.M).group(1).upper()])
    pre = os.path.join(tmp, name)
    cmd = [exe, cfg_path, "--noise", str(SEED), repr(amp), "--state-out", pre + "_final.bin", "--log", pre + "_log.bin"]
    if "probe" in outputs:
        cmd += ["--probe", pre + "_probe.bin"]
    if "stages" in outputs:
        one = re.sub(r"^Ts=.*$", "Ts= 1", text, flags=re.M)
        one_path = os.path.join(tmp, name + "_one.txt")
        open(one_path, "w").write(one)
        subprocess.run([exe, one_path, "--noise", str(SEED), repr(amp), "--stages", pre + "_stg"], check=True,
                       capture_output=True, env=dict(os.environ, OMP_NUM_THREADS="4"))
    res = subprocess.run(cmd, check=True, capture_output=True, text=True, env=dict(os.environ, OMP_NUM_THREADS="4"))
    summary = json.loads(res.stdout.strip().splitlines()[-1])
    arrays = {"config": np.frombuffer(text.encode(), dtype=np.uint8)}
    meta = dict(name=name, seed=SEED, noise_amp=amp, summary=summary, outputs=outputs,
                generator="oracle/_ref built by oracle/Makefile from the reference sources")
    nb, ne = summary["beams"], summary["ebins"]
    if "replay" in outputs:
        arrays["log"] = np.fromfile(pre + "_log.bin").reshape(-1, 3)
        arrays["final"] = np.fromfile(pre + "_final.bin")
    if "probe" in outputs:
        for k, v in read_probe(pre + "_probe.bin").items():
            arrays["probe_" + k] = v
    if "stages" in outputs:
        for k in ("psi0", "psi1", "psi3", "psi4", "esum4", "err"):
            arrays["stage_" + k] = np.fromfile("%s_stg_%s.bin" % (pre, k))
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
    print(name, summary)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("XFLAT_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference"),
                    help="reference checkout (default: XFLAT_REFERENCE, else `reference` beside the repository)")
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref", "REF=" + args.ref, "-j8"], check=True,
                   capture_output=True)
    refdir = os.path.join(ROOT, "oracle", "_ref")
    with tempfile.TemporaryDirectory() as tmp:
        for case in CASES:
            if args.only and case[0] != args.only:
                continue
            run_case(*case, refdir=refdir, tmp=tmp)


if __name__ == "__main__":
    sys.exit(main())
