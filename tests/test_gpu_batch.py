"""Batched path: independent MA (and SA) instances of uneven shapes advanced by
shared launches with per-instance step control, against the same instances run
alone."""
import numpy as np
import pytest

import xflat_gb300 as xg
from xflat_gb300.sweep import sweep_configs
from helpers import derive, pol_rel_err

pytestmark = pytest.mark.gpu


def _small_sweep(precision="fp64", n=4):
    return sweep_configs(seed=7, n=n, precision=precision, abins=(3, 40), ebins=(5, 70))


def test_batch_equals_instances_run_alone():
    texts = _small_sweep()
    b = xg.Batch([xg.Config.from_text(t) for t in texts])
    out = b.run(max_iters=60)
    for i, t in enumerate(texts):
        s = xg.Simulation(xg.Config.from_text(t))
        o = s.evolutionLoop(max_iters=60, device_control=True)
        assert (o["iterations"], o["accepted"]) == (out["iterations"][i], out["accepted"][i])
        assert abs(o["r_end"] - out["r_end"][i]) <= 1e-12 * o["r_end"]
        # same arithmetic, moments summed in a different (fixed) order
        assert pol_rel_err(b.get_state(i), s.get_state(0)) <= 1e-10


def test_batch_uneven_budgets_and_radii():
    texts = _small_sweep()
    texts[1] = derive(texts[1], Rn="10.0000003")    # finishes by radius
    b = xg.Batch([xg.Config.from_text(t) for t in texts])
    out = b.run(max_iters=60)
    r = out["r_end"]
    assert r[1] == pytest.approx(10.0000003, abs=1e-12)
    assert out["iterations"][1] < 60
    assert all(out["iterations"][i] == 60 for i in (0, 2, 3))
    w, ms = b.tile_shape()
    assert w in (2, 4, 8) and np.all(ms > 0)


def test_batch_mixed_vs_fp64():
    b64 = xg.Batch([xg.Config.from_text(t) for t in _small_sweep("fp64")])
    b32 = xg.Batch([xg.Config.from_text(t) for t in _small_sweep("mixed")])
    o64 = b64.run(max_iters=80)
    o32 = b32.run(max_iters=80)
    for i in range(4):
        if o64["accepted"][i] != o32["accepted"][i]:
            continue
        a, c = b64.get_state(i), b32.get_state(i)
        pee = lambda x: x[0::4, 0] ** 2 + x[0::4, 1] ** 2
        assert np.max(np.abs(pee(a) - pee(c))) <= 1e-5


def test_batch_rejects_mixed_geometry():
    texts = _small_sweep(n=2)
    texts[1] = texts[1].replace("geometry= MA", "geometry= MAA")
    with pytest.raises(xg.XflatError):
        xg.Batch([xg.Config.from_text(t) for t in texts])


def test_batch_with_sa_instances():
    """SA instances share the MA-shaped kernels, so they batch with MA ones."""
    texts = _small_sweep(n=3)
    texts.append(derive("sa_bulb.txt", Ebins=48, R0=10, dr="1e-3"))
    texts.append(derive("sa_bulb.txt", Ebins=5, R0=60, dr="1e-3"))
    b = xg.Batch([xg.Config.from_text(t) for t in texts])
    out = b.run(max_iters=60)
    for i in (3, 4):
        s = xg.Simulation(xg.Config.from_text(texts[i]))
        o = s.evolutionLoop(max_iters=60, device_control=True)
        assert (o["iterations"], o["accepted"]) == (out["iterations"][i], out["accepted"][i])
        assert pol_rel_err(b.get_state(i), s.get_state(0)) <= 1e-10
