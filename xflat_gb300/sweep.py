"""Seeded parameter sweep of independent MA bulb instances (the batched
workload): per instance, angle bins uniform in {128..2048}, energy bins uniform
in {32..512} (1-60 MeV), each species' luminosity log-uniform in
[1e50, 1e52] erg/s, normal or inverted hierarchy with probability 1/2, and a
matter potential lambda(R) = lambda0 (R/r)^3 with lambda0 log-uniform in
[1e2, 1e4] km^-1; integrated from 10 to 600 km.  Returns config texts in the
reference's key format."""
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BASE = os.path.join(HERE, "configs", "config0_ma.txt")

# sqrt2 * GF * Ye * 4.2e45 with the reference's truncated constants
# (src/Matt.cpp:24-35, include/Util.h:15-22): lambda(10 km) per unit gs.
_SQRT2, _GF = 1.41421356237, 1.16637E-11 * 3.893793036626876e-32


def lambda_per_gs(Ye=0.5, Mns=1.4, S=100.):
    return _SQRT2 * _GF * Ye * 4.2E+45 * (Mns / 1.4) ** 3 * (100. / S) ** 4


def _set(text, key, value):
    text, n = re.subn(r"^%s=.*$" % re.escape(key), "%s= %s" % (key, value), text, flags=re.M)
    if n != 1:
        raise KeyError(key)
    return text


def sweep_configs(seed=4, n=64, precision="fp64", rn=600.0, abins=(128, 2048), ebins=(32, 512), base=BASE):
    rng = np.random.default_rng(seed)
    text0 = open(base).read()
    out = []
    for i in range(n):
        t = text0
        t = _set(t, "Abins", int(rng.integers(abins[0], abins[1] + 1)))
        t = _set(t, "Ebins", int(rng.integers(ebins[0], ebins[1] + 1)))
        for key in ("Lve", "Lv_e", "Lvt", "Lv_t"):
            t = _set(t, key, "%.6e" % (10.0 ** rng.uniform(50.0, 52.0)))
        t = _set(t, "dm2", "3E-3" if rng.random() < 0.5 else "-3E-3")
        lam0 = 10.0 ** rng.uniform(2.0, 4.0)
        t = _set(t, "gs", "%.10g" % (lam0 / lambda_per_gs()))
        t = _set(t, "Rn", rn)
        t = _set(t, "precision", precision)
        t = _set(t, "seed", seed * 1000 + i)
        out.append(t)
    return out
