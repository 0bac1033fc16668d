"""Parity of the FP64 CUDA path with the reference (golden fixtures made by the
reference itself) and with the oracle at the workload shapes.  Bar: every
beam's polarization vector within 1e-10 relative when forced to the
reference's accepted step sequence (floating point; tolerance stated per test)."""
import numpy as np
import pytest

import xflat_gb300 as xg
from helpers import TempConfig, derive, golden, golden_names, key, noise_state, pol_rel_err, replay_inputs
from oracle.port import Port

pytestmark = pytest.mark.gpu

POL_TOL = 1e-10


def _sim(text):
    return xg.Simulation(xg.Config.from_text(text))


@pytest.mark.parametrize("name", golden_names("probe"))
def test_tables_angles_and_hamiltonian_vs_reference(name):
    g = golden(name)
    sim = _sim(g["config"])
    t = sim.tables()
    np.testing.assert_allclose(t["fv"].reshape(-1), g["probe_fv"], rtol=1e-14, atol=0)
    np.testing.assert_allclose(t["hvac"], g["probe_hvac"], rtol=1e-14, atol=0)
    r, dr = key(g["config"], "R0"), key(g["config"], "dr")
    c, s, d, l = sim.calcAngleBins(r, dr)
    if "probe_rpt" in g:
        # SA: dl = dr/2, dr, dr/2 exactly; the weight slot holds D(r) at the
        # reference's stage radii (src/Phy_SA.cpp:121-147, 250-256)
        np.testing.assert_array_equal(l.reshape(-1), g["probe_dl"])
        R = key(g["config"], "Rv") / g["probe_rpt"]
        np.testing.assert_allclose(d.reshape(-1), .5 * (1. - np.sqrt(1. - R * R)) ** 2, rtol=1e-14, atol=0)
        assert not c.any() and not s.any()
    else:
        # device sqrt and division are correctly rounded; contraction differs (see oracle tests)
        np.testing.assert_allclose(c.reshape(-1), g["probe_cos"], rtol=2e-13, atol=0)
        np.testing.assert_allclose(d.reshape(-1), g["probe_dcos"], rtol=2e-13, atol=0)
        np.testing.assert_allclose(l.reshape(-1), g["probe_dl"], rtol=2e-13, atol=0)
        if "probe_sin" in g:
            np.testing.assert_allclose(s.reshape(-1), g["probe_sin"], rtol=2e-13, atol=0)
    sim.set_noise(g["meta"]["seed"], g["meta"]["noise_amp"])
    for pt in range(3):
        h = sim.calc_Hvv(0, pt, r, dr).reshape(-1)
        ref = g["probe_hvv%d" % pt]
        # the moment sums are reduced in a different order than the reference's serial loop
        assert np.max(np.abs(h - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("name", golden_names("replay"))
def test_replay_reference_step_sequence(name):
    g = golden(name)
    sim = _sim(g["config"])
    sim.set_state(noise_state(sim.nbeams, sim.ebins, g["meta"]["seed"], g["meta"]["noise_amp"]))
    rb, dr = replay_inputs(g["config"], g["log"])
    sim.replay(rb, dr)
    err = pol_rel_err(sim.get_state(0), g["final"].reshape(sim.state_shape))
    assert err <= POL_TOL, err


@pytest.mark.parametrize("name", golden_names("stages"))
def test_one_iteration_every_stage_buffer(name):
    g = golden(name)
    sim = _sim(g["config"])
    sim.lib.xf_set_option(sim.h, b"debug_psi3", 1.0)
    sim.set_noise(g["meta"]["seed"], g["meta"]["noise_amp"])
    r, dr = key(g["config"], "R0"), key(g["config"], "dr")
    me = sim.step(r, dr)
    ref_me = np.sqrt(g["stage_err"].max())
    # Max_err is a difference of nearly equal states: relative precision ~ ulp/Max_err
    assert abs(me - ref_me) <= 1e-6 * ref_me
    for k in (1, 3, 4):
        ref = g["stage_psi%d" % k].reshape(sim.state_shape)
        assert np.max(np.abs(sim.get_state(k) - ref)) < 1e-13, k


def _port_and_sim(text, seed, amp):
    with TempConfig(text) as path:
        port = Port(path)
    port.noise(seed, amp)
    sim = _sim(text)
    sim.set_state(port.get_state(0))
    return port, sim


def test_config0_shape_window_vs_oracle():
    """Config-0 shape (256 x 64), 60 free-running oracle steps from 10 km replayed."""
    text = derive("config0_ma.txt", dr="1e-8")
    port, sim = _port_and_sim(text, 1, 1e-7)
    out = port.run(r0=10.0, dr0=1e-8, max_iters=60, log_cap=100)
    rb, dr = replay_inputs(text, out["log"])
    sim.replay(rb, dr)
    assert pol_rel_err(sim.get_state(0), port.get_state(0)) <= POL_TOL


def test_config1_shape_iteration_vs_oracle():
    """Config-1 shape (2048 x 512 energies, 4.19M bins): one iteration at 50 km,
    every stage buffer and the step error."""
    text = derive("config1_ma.txt", R0=50, dr="1e-4")
    port, sim = _port_and_sim(text, 1, 1e-7)
    sim.lib.xf_set_option(sim.h, b"debug_psi3", 1.0)
    me_c = port.iterate(50.0, 1e-4)
    me_g = sim.step(50.0, 1e-4)
    assert abs(me_g - me_c) <= 1e-5 * me_c
    for k in (1, 3, 4):
        assert np.max(np.abs(sim.get_state(k) - port.get_state(k))) < 1e-12, k


def test_config3_maa_shape_iterations_vs_oracle():
    """Config-3 MAA shape (256 x 64 azimuth x 128 energies, 8.4M bins): two
    accepted iterations at 12 km."""
    text = derive("config3_maa.txt", R0=12, dr="1e-7")
    port, sim = _port_and_sim(text, 3, 1e-6)
    r = 12.0
    for _ in range(2):
        me_c = port.iterate(r, 1e-7)
        me_g = sim.step(r, 1e-7)
        assert abs(me_g - me_c) <= 1e-5 * me_c
        port.accept()
        sim.accept()
        r += 1e-7
    assert pol_rel_err(sim.get_state(0), port.get_state(0)) <= POL_TOL


@pytest.mark.parametrize("geom,over", [
    ("config0_ma.txt", dict(Abins=7, Ebins=45, R0=15, dr="1e-6")),
    ("config0_ma.txt", dict(Abins=1, Ebins=1, R0=40, dr="1e-4")),
    ("config3_maa.txt", dict(Abins=3, Pbins=7, Ebins=33, R0=15, dr="1e-6")),
])
def test_ragged_and_minimal_shapes(geom, over):
    text = derive(geom, **over)
    port, sim = _port_and_sim(text, 5, 1e-6)
    out = port.run(max_iters=30, log_cap=100)
    port2 = None
    sim.lib.xf_set_option(sim.h, b"debug_psi3", 0.0)
    rb, dr = replay_inputs(text, out["log"])
    sim.set_state(noise_state(sim.nbeams, sim.ebins, 5, 1e-6))
    sim.replay(rb, dr)
    assert pol_rel_err(sim.get_state(0), port.get_state(0)) <= POL_TOL


def test_free_running_loop_vs_oracle():
    text = derive("config0_ma.txt", Abins=32, Ebins=32)
    port, sim = _port_and_sim(text, 1, 1e-7)
    a = port.run(max_iters=300, log_cap=1000)
    b = sim.evolutionLoop(max_iters=300, log_cap=1000)
    assert b["iterations"] == a["iterations"] and b["accepted"] == a["accepted"]
    np.testing.assert_array_equal(b["log"][:, 0], a["log"][:, 0])
    np.testing.assert_allclose(b["log"][:, 2], a["log"][:, 2], rtol=1e-5)


def test_device_control_equals_host_loop():
    """The GPU-resident controller takes exactly the host loop's decisions."""
    text = derive("config0_ma.txt", Abins=32, Ebins=64)
    s1 = _sim(text)
    s2 = _sim(text)
    a = s1.evolutionLoop(max_iters=250, log_cap=1000)
    b = s2.evolutionLoop(max_iters=250, log_cap=1000, device_control=True, iters_per_launch=16)
    assert (a["iterations"], a["accepted"]) == (b["iterations"], b["accepted"])
    np.testing.assert_array_equal(a["log"], b["log"])
    assert a["r_end"] == b["r_end"] and a["dr_end"] == b["dr_end"]
    assert np.array_equal(s1.get_state(0), s2.get_state(0))
    # copies the loops report: host-driven r, dr, hm H2D (40 B) and Max_err D2H
    # (8 B) per iteration (its log is written on the host); device control one
    # control-block copy per launch of 16 iterations, plus the log (24 B per
    # record)
    it = a["iterations"]
    assert a["h2d_bytes"] >= 40 * it and a["d2h_bytes"] >= 8 * it
    ctl = b["d2h_bytes"] - 24 * b["log_len"]
    assert 0 < b["h2d_bytes"] < 40 * it and 0 < ctl
    # the same 48 iterations in 3 and in 6 launches: 3 more control-block copies
    c = s2.evolutionLoop(max_iters=48, device_control=True, iters_per_launch=16)
    d = s2.evolutionLoop(max_iters=48, device_control=True, iters_per_launch=8)
    assert c["iterations"] == d["iterations"] == 48
    assert c["h2d_bytes"] == d["h2d_bytes"]
    extra = d["d2h_bytes"] - c["d2h_bytes"]
    assert extra > 0 and extra % 3 == 0 and c["d2h_bytes"] >= extra


def test_bitwise_reproducible():
    text = derive("config0_ma.txt")
    outs = []
    for _ in range(2):
        s = _sim(text)
        s.evolutionLoop(max_iters=20, device_control=True)
        outs.append(s.get_state(0))
    assert np.array_equal(outs[0], outs[1])


def test_launch_shapes_agree():
    text = derive("config0_ma.txt", Abins=64, Ebins=96)
    ref = None
    for threads, blocks in [(256, 0), (128, 0), (64, 7), (32, 1)]:
        s = _sim(text)
        assert s.lib.xf_set_option(s.h, b"threads", float(threads)) == 0
        assert s.lib.xf_set_option(s.h, b"blocks", float(blocks)) == 0
        s.evolutionLoop(max_iters=40)
        st = s.get_state(0)
        if ref is None:
            ref = st
        else:
            assert pol_rel_err(st, ref) <= 1e-12


def test_nan_state_reports_status():
    text = derive("config0_ma.txt", Abins=4, Ebins=8)
    s = _sim(text)
    psi = s.get_state(0)
    psi[3, 0, 2] = np.nan
    s.set_state(psi)
    assert np.isnan(s.step(10.0, 1e-8))
    out = s.evolutionLoop(max_iters=5)
    assert out["status"] == xg._abi.XF_ENAN


def test_argument_errors():
    s = _sim(derive("config0_ma.txt", Abins=4, Ebins=8))
    with pytest.raises(xg.XflatError):
        s.get_state(2)
    with pytest.raises(xg.XflatError):
        s.set_state(np.zeros(5))
    assert s.lib.xf_set_option(s.h, b"threads", 48.0) == xg._abi.XF_EINVAL
    assert s.lib.xf_set_option(s.h, b"nonsense", 1.0) == xg._abi.XF_EINVAL


def test_survival_probabilities():
    """Probability-file quantity sum_e fv (ar^2 + ai^2) with the fv of particle
    p % 2 (src/IO_f.cpp:341-351)."""
    s = _sim(derive("config0_ma.txt", Abins=8, Ebins=16))
    psi = s.get_state(0)
    fv = s.tables()["fv"]
    sv = s.survival()
    ref = np.einsum("bpe,pe->bp", (psi[:, 0] ** 2 + psi[:, 1] ** 2).reshape(8, 4, 16), fv[[0, 1, 0, 1]])
    np.testing.assert_allclose(sv, ref, rtol=1e-14)


@pytest.mark.parametrize("name", ["sa_r10", "sa_r60"])
def test_sa_free_running_vs_reference(name):
    """Single-angle geometry on the MA-shaped kernels, device-controlled loop:
    the reference's own accept/reject sequence (src/Phy_SA.cpp + src/Nmr.cpp),
    dr to the precision the step-error cancellation allows."""
    g = golden(name)
    sim = _sim(g["config"])
    assert (sim.nbeams, sim.abins, sim.pbins) == (4, 1, 1)
    sim.set_noise(g["meta"]["seed"], g["meta"]["noise_amp"])
    out = sim.evolutionLoop(max_iters=g["meta"]["summary"]["iterations"], log_cap=100000, device_control=True)
    log = g["log"]
    assert out["accepted"] == len(log)
    np.testing.assert_array_equal(out["log"][:, 0], log[:, 0])
    np.testing.assert_allclose(out["log"][:, 2], log[:, 2], rtol=1e-5)


def test_sa_ignores_abins():
    """SA has one trajectory whatever Abins says (src/Phy_SA.cpp:150-184)."""
    a = _sim(derive("sa_bulb.txt", Abins=1, Ebins=40))
    b = _sim(derive("sa_bulb.txt", Abins=300, Ebins=40))
    assert a.nbeams == b.nbeams == 4
    for s in (a, b):
        s.set_noise(1, 1e-7)
        s.evolutionLoop(max_iters=50)
    assert np.array_equal(a.get_state(0), b.get_state(0))
