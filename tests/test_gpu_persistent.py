"""Persistent device-controlled loop (option "persistent": one cooperative
launch per k iterations, the phases separated by grid barriers) against the
graph-launched loop, and the bounded barrier waits.

Bars: the same accepted steps, logs and final states bit for bit (the grid and
therefore every reduction order are the same); a barrier wait that cannot end
returns XF_ETIMEOUT within its limit and leaves the handle usable."""
import ctypes

import numpy as np
import pytest

import xflat_gb300 as xg
from helpers import derive

pytestmark = pytest.mark.gpu


def _sim(text, **opts):
    s = xg.Simulation(xg.Config.from_text(text))
    for k, v in opts.items():
        assert s.lib.xf_set_option(s.h, k.encode(), float(v)) == 0, k
    return s


@pytest.mark.parametrize("base,over,prec", [
    ("config0_ma.txt", dict(Abins=64, Ebins=64, R0=20, dr="1e-5"), "fp64"),
    ("config0_ma.txt", dict(Abins=256, Ebins=64, R0=50, dr="1e-4"), "fp64"),
    ("config0_ma.txt", dict(Abins=64, Ebins=64, R0=20, dr="1e-5"), "df"),
    ("config3_maa.txt", dict(Abins=16, Pbins=8, Ebins=32, R0=15, dr="1e-6"), "fp64"),
    ("config3_maa.txt", dict(Abins=16, Pbins=8, Ebins=32, R0=15, dr="1e-6"), "df"),
    ("sa_bulb.txt", dict(R0=10, dr="1e-3"), "fp64"),
])
def test_persistent_equals_graph_loop(base, over, prec):
    text = derive(base, precision=prec, **over)
    a = _sim(text, persistent=0)
    b = _sim(text, persistent=1)
    oa = a.evolutionLoop(max_iters=300, device_control=True, log_cap=300)
    ob = b.evolutionLoop(max_iters=300, device_control=True, log_cap=300)
    assert (oa["iterations"], oa["accepted"]) == (ob["iterations"], ob["accepted"])
    np.testing.assert_array_equal(oa["log"], ob["log"])
    assert np.array_equal(a.get_state(0), b.get_state(0))
    # one cooperative launch per 16 iterations instead of four kernels per
    # iteration (plus the set-up's moment kernel)
    assert ob["kernel_launches"] <= (300 + 15) // 16 + 1 < oa["kernel_launches"]


def test_persistent_ends_at_the_radius():
    text = derive("config0_ma.txt", Abins=32, Ebins=32, R0=20, dr="1e-5", Rn="20.001")
    a = _sim(text, persistent=0)
    b = _sim(text, persistent=1)
    oa = a.evolutionLoop(max_iters=100000, device_control=True)
    ob = b.evolutionLoop(max_iters=100000, device_control=True)
    assert ob["r_end"] == oa["r_end"] == 20.001
    assert (oa["iterations"], oa["accepted"]) == (ob["iterations"], ob["accepted"])


def test_barrier_wait_runs_out_and_the_handle_recovers():
    """Each barrier waits for one arrival beyond the grid, which never comes:
    the launch ends after the 50 ms limit with XF_ETIMEOUT, nothing traps, and
    the same handle then runs normally."""
    text = derive("config0_ma.txt", Abins=32, Ebins=32, R0=20, dr="1e-5")
    s = _sim(text, persistent=1, barrier_timeout_ms=50, debug_barrier_extra=1)
    psi0 = s.get_state(0).copy()
    with pytest.raises(xg.XflatError) as e:
        s.evolutionLoop(max_iters=32, device_control=True)
    assert e.value.status == xg._abi.XF_ETIMEOUT
    assert b"barrier" in s.lib.xf_last_error(s.h)
    # the state was not touched (the first barrier precedes every phase)
    assert np.array_equal(s.get_state(0), psi0)
    assert s.lib.xf_set_option(s.h, b"debug_barrier_extra", 0.0) == 0
    out = s.evolutionLoop(max_iters=64, device_control=True, log_cap=64)
    ref = _sim(text, persistent=0)
    oref = ref.evolutionLoop(max_iters=64, device_control=True, log_cap=64)
    assert (out["iterations"], out["accepted"]) == (oref["iterations"], oref["accepted"])
    np.testing.assert_array_equal(out["log"], oref["log"])
    assert np.array_equal(s.get_state(0), ref.get_state(0))


def test_persistent_options_are_checked():
    s = _sim(derive("config0_ma.txt", Abins=4, Ebins=8))
    assert s.lib.xf_set_option(s.h, b"barrier_timeout_ms", 0.0) == xg._abi.XF_EINVAL
    assert s.lib.xf_set_option(s.h, b"debug_barrier_extra", -1.0) == xg._abi.XF_EINVAL
    assert s.lib.xf_set_option(s.h, b"persistent", 1.0) == 0
    assert s.lib.xf_set_option(s.h, b"persistent", -1.0) == 0
    assert s.lib.xf_set_option(s.h, b"persistent", 2.0) == xg._abi.XF_EINVAL
