"""Generate tests/golden/c0_full_ref.npz: the reference's own run of the whole
config-0 workload (xflat_gb300/configs/config0_ma.txt: MA 256 angle x 64
energy bins, 10 -> 300 km, tolerance 1e-9, noise seed 1 at amplitude 1e-7),
for the full-run test (tests/test_gpu_full_run.py).

The reference's hot-path sources are compiled by ``oracle/Makefile`` (target
``ref``) into ``oracle/_ref/xflat_ref_ma``; this script runs it to the end of
the run (about 1.1e7 stepper iterations, about 5 hours on 8 cores) and keeps
P_ee(E) = ar^2 + ai^2 of every nu_e beam (particle 0 of each angle bin) of
the final state, the final radius and the reference's iteration counts.

    python tests/golden/make_full_run.py [--threads N]
    python tests/golden/make_full_run.py --state final_state.bin --stdout run.log

The second form packs the output of a run made earlier with
``xflat_ref_ma config0_ma.txt --noise 1 1e-7 --state-out final_state.bin``
(its standard output saved as run.log).
"""
import argparse
import json
import os
import re
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CONFIG = os.path.join(ROOT, "xflat_gb300", "configs", "config0_ma.txt")
EXE = os.path.join(ROOT, "oracle", "_ref", "xflat_ref_ma")
OUT = os.path.join(HERE, "c0_full_ref.npz")
ABINS, EBINS = 256, 64


def pack(state_path, stdout_text):
    psi = np.fromfile(state_path, dtype="<f8").reshape(ABINS * 4, 4, EBINS)
    x = psi[0::4]
    pee = x[:, 0] ** 2 + x[:, 1] ** 2
    stats = json.loads([ln for ln in stdout_text.splitlines() if ln.startswith("{")][-1])
    m = re.search(r"at radius\(Km\):\s*([0-9.eE+-]+)", stdout_text)
    if not m:
        raise SystemExit("the run's output has no final radius")
    np.savez_compressed(OUT, pee=pee, r_end=float(m.group(1)), iterations=int(stats["iterations"]),
                        accepted=int(stats["accepted"]), seconds=float(stats["seconds"]),
                        config=open(CONFIG).read(), seed=1, noise_amp=1e-7)
    print("wrote %s: r_end %s, %d iterations, %d accepted" % (OUT, m.group(1), stats["iterations"],
                                                              stats["accepted"]))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--state", help="final state of an earlier run (raw float64, NetCDF psi layout)")
    ap.add_argument("--stdout", help="standard output of that run")
    args = ap.parse_args()
    if args.state:
        pack(args.state, open(args.stdout).read())
        return
    if not os.path.exists(EXE):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref", "-j8"], check=True)
    env = dict(os.environ, OMP_NUM_THREADS=str(args.threads), OMP_PROC_BIND="close")
    with tempfile.TemporaryDirectory() as tmp:
        state = os.path.join(tmp, "final_state.bin")
        res = subprocess.run([EXE, CONFIG, "--noise", "1", "1e-7", "--state-out", state], env=env,
                             capture_output=True, text=True, check=True)
        pack(state, res.stdout)


if __name__ == "__main__":
    main()
