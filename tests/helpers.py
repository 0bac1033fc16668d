"""Shared helpers for the tests: golden fixtures, derived configs, checks."""
import json
import os
import re
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLDEN = os.path.join(HERE, "golden")
CONFIGS = os.path.join(ROOT, "xflat_gb300", "configs")


def golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    out = {k: z[k] for k in z.files}
    out["config"] = bytes(out["config"]).decode()
    out["meta"] = json.loads(bytes(out["meta"]).decode())
    return out


def golden_names(kind):
    """Window fixtures of make_golden.py with output `kind` (the whole-run
    fixture of make_full_run.py carries no meta and is read by its own test)."""
    names = []
    for f in sorted(os.listdir(GOLDEN)):
        if f.endswith(".npz"):
            g = np.load(os.path.join(GOLDEN, f))
            if "meta" not in g.files:
                continue
            meta = json.loads(bytes(g["meta"]).decode())
            if kind in meta["outputs"].split():
                names.append(f[:-4])
    return names


def derive(base, **kv):
    """Config text from a workload config with key overrides."""
    text = open(os.path.join(CONFIGS, base)).read() if not base.startswith("#") and "\n" not in base else base
    for k, v in kv.items():
        text, n = re.subn(r"^%s=.*$" % re.escape(k), "%s= %s" % (k, v), text, flags=re.M)
        assert n == 1, k
    return text


def key(text, k, cast=float):
    return cast(re.search(r"^%s=\s*(\S+)" % re.escape(k), text, re.M).group(1))


class TempConfig:
    """Writes config text to a temporary file (for the C restatement, which reads files)."""

    def __init__(self, text):
        fd, self.path = tempfile.mkstemp(suffix=".txt")
        with os.fdopen(fd, "w") as f:
            f.write(text)

    def __enter__(self):
        return self.path

    def __exit__(self, *a):
        os.remove(self.path)


def replay_inputs(text, log):
    """Recovers the exact (r_before, dr) doubles of the accepted steps: the
    reference accumulates r += dr (src/Nmr.cpp:229)."""
    r = key(text, "R0")
    rb = []
    for k in range(len(log)):
        rb.append(r)
        r = r + log[k, 2]
        assert r == log[k, 1], "radius sequence is not the accumulated one"
    return np.array(rb), log[:, 2].copy()


def polarization(psi):
    """Per-bin polarization vector P = (2 Re rho01, -2 Im rho01, 2 rho00) with rho
    from NBeam::density (src/NBeam.cpp:314-322); psi: [beam][4][e]."""
    ar, ai, br, bi = psi[:, 0], psi[:, 1], psi[:, 2], psi[:, 3]
    r00 = .5 * ((ar * ar + ai * ai) - (br * br + bi * bi))
    r01r = ar * br + ai * bi
    r01i = ai * br - ar * bi
    return np.stack([2 * r01r, -2 * r01i, 2 * r00], -1)


def pol_rel_err(a, b):
    """Max over bins of |P_a - P_b| / |P_b| (every beam's polarization vector)."""
    pa, pb = polarization(a), polarization(b)
    return float(np.max(np.linalg.norm(pa - pb, axis=-1) / np.linalg.norm(pb, axis=-1)))


def noise_state(nbeams, ne, seed, amp):
    """numpy statement of the seeded initial state (splitmix64 keyed on seed,
    beam, ebin): pure flavor states of src/NBeam.cpp:246-276 plus noise."""
    M = np.uint64(0xFFFFFFFFFFFFFFFF)

    def sm(x):
        x = (x + np.uint64(0x9E3779B97F4A7C15)) & M
        z = x
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & M
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & M
        return z ^ (z >> np.uint64(31))

    b = np.arange(nbeams, dtype=np.uint64)[:, None]
    e = np.arange(ne, dtype=np.uint64)[None, :]
    with np.errstate(over="ignore"):
        def u(k):
            h = sm(np.uint64(seed) ^ sm((b << np.uint64(24)) ^ (e << np.uint64(1)) ^ np.uint64(k)))
            return (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        eps = (u(0) - 0.5) * amp
        eta = (u(1) - 0.5) * amp
    one = np.sqrt(1. - eps * eps - eta * eta)
    nu = (np.arange(nbeams) % 4 < 2)[:, None]
    psi = np.zeros((nbeams, 4, ne))
    psi[:, 0] = np.where(nu, one, eps)
    psi[:, 2] = np.where(nu, eps, one)
    psi[:, 3] = eta
    return psi
