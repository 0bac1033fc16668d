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
    t = b.tuning()
    # 9 graph-launched shapes and 3 persistent ones (FP64)
    assert len(t["candidates"]) == 12 and all(c[3] > 0 for c in t["candidates"])
    assert (t["warps"], t["beams_per_warp"], t["persistent"]) == min(t["candidates"], key=lambda c: c[3])[:3]


@pytest.mark.parametrize("warps,bpw", [(2, 4), (8, 2)])
def test_batch_tile_shapes_agree(warps, bpw):
    """Every tile shape gives the same decisions and states (the per-instance
    reductions are summed in an order fixed by the shape, so states agree to
    rounding)."""
    texts = _small_sweep()
    b = xg.Batch([xg.Config.from_text(t) for t in texts])
    ref = b.run(max_iters=40)
    ref_states = [b.get_state(i) for i in range(len(texts))]
    c = xg.Batch([xg.Config.from_text(t) for t in texts])
    assert c.lib.xf_batch_set_persistent(c.h, 0, 1) == 0
    assert c.lib.xf_batch_set_shape(c.h, warps, bpw) == 0
    out = c.run(max_iters=40)
    assert list(out["accepted"]) == list(ref["accepted"])
    for i in range(len(texts)):
        assert pol_rel_err(c.get_state(i), ref_states[i]) <= 1e-10


def test_batch_mixed_vs_fp64():
    b64 = xg.Batch([xg.Config.from_text(t) for t in _small_sweep("fp64")])
    b32 = xg.Batch([xg.Config.from_text(t) for t in _small_sweep("mixed")])
    o64 = b64.run(max_iters=80)
    o32 = b32.run(max_iters=80)
    # every instance is compared: the step sequences must agree for the
    # comparison to be at equal radii
    assert list(o64["accepted"]) == list(o32["accepted"])
    np.testing.assert_allclose(o32["r_end"], o64["r_end"], rtol=1e-9)
    for i in range(4):
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


def test_batch_df_equals_instances_run_alone():
    """Double-float instances in a batch: the single-simulation double-float
    path's decisions and states (moments summed in the batch's order)."""
    texts = [t.replace("precision= fp64", "precision= df") for t in _small_sweep()]
    b = xg.Batch([xg.Config.from_text(t) for t in texts])
    out = b.run(max_iters=60)
    for i, t in enumerate(texts):
        s = xg.Simulation(xg.Config.from_text(t))
        o = s.evolutionLoop(max_iters=60, device_control=True)
        assert (o["iterations"], o["accepted"]) == (out["iterations"][i], out["accepted"][i])
        assert pol_rel_err(b.get_state(i), s.get_state(0)) <= 1e-10


def test_batch_df_vs_fp64():
    b64 = xg.Batch([xg.Config.from_text(t) for t in _small_sweep("fp64")])
    b2 = xg.Batch([xg.Config.from_text(t) for t in _small_sweep("df")])
    o64 = b64.run(max_iters=80)
    o2 = b2.run(max_iters=80)
    assert list(o64["accepted"]) == list(o2["accepted"])
    np.testing.assert_allclose(o2["r_end"], o64["r_end"], rtol=1e-9)
    for i in range(4):
        a, c = b64.get_state(i), b2.get_state(i)
        pee = lambda x: x[0::4, 0] ** 2 + x[0::4, 1] ** 2
        assert np.max(np.abs(pee(a) - pee(c))) <= 1e-8


@pytest.mark.parametrize("prec,bpw", [("fp64", 1), ("df", 2)])
def test_batch_persistent_equals_graphs(prec, bpw):
    """The batch as one cooperative launch per 8 iterations (grid barriers
    between the stages) against the per-stage graph launches with the same
    tile shape: the same decisions and states bit for bit."""
    texts = _small_sweep(prec)
    a = xg.Batch([xg.Config.from_text(t) for t in texts])
    assert a.lib.xf_batch_set_persistent(a.h, 0, 1) == 0
    assert a.lib.xf_batch_set_shape(a.h, 8, bpw) == 0
    b = xg.Batch([xg.Config.from_text(t) for t in texts])
    assert b.lib.xf_batch_set_persistent(b.h, 1, bpw) == 0
    oa, ob = a.run(max_iters=60), b.run(max_iters=60)
    assert list(oa["iterations"]) == list(ob["iterations"]) and list(oa["accepted"]) == list(ob["accepted"])
    for i in range(len(texts)):
        assert np.array_equal(a.get_state(i), b.get_state(i))


def test_batch_persistent_rejects_mixed():
    b = xg.Batch([xg.Config.from_text(t) for t in _small_sweep("mixed", n=2)])
    assert b.lib.xf_batch_set_persistent(b.h, 1, 1) == xg._abi.XF_EUNSUPPORTED
