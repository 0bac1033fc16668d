"""The oracle (C restatement, oracle/xf_port.c) pinned against outputs of the
reference itself (tests/golden/, generated by tests/golden/make_golden.py from
the reference's own sources).  CPU only."""
import numpy as np
import pytest

from helpers import TempConfig, golden, golden_names, key, noise_state, pol_rel_err, replay_inputs
from oracle.port import Port


def _port(g):
    with TempConfig(g["config"]) as path:
        return Port(path)


@pytest.mark.parametrize("name", golden_names("stages"))
def test_noise_generator_matches_reference_harness(name):
    g = golden(name)
    p = _port(g)
    psi0 = g["stage_psi0"].reshape(p.shape)
    ref = noise_state(p.nbeams, p.ebins, g["meta"]["seed"], g["meta"]["noise_amp"])
    assert np.array_equal(psi0, ref)
    p.noise(g["meta"]["seed"], g["meta"]["noise_amp"])
    assert np.array_equal(p.get_state(0), ref)


@pytest.mark.parametrize("name", golden_names("probe"))
def test_tables_and_matter(name):
    g = golden(name)
    p = _port(g)
    t = p.tables()
    # floating point, order of operations restated; the compilers' FMA
    # contraction choices differ, hence ulp-level tolerances
    np.testing.assert_allclose(t["fv"].reshape(-1), g["probe_fv"], rtol=1e-14, atol=0)
    np.testing.assert_allclose(t["hvac"], g["probe_hvac"], rtol=1e-14, atol=0)
    np.testing.assert_allclose(t["Ev"], g["probe_Ev"], rtol=1e-14, atol=0)
    np.testing.assert_allclose(t["LE"], g["probe_LE"], rtol=1e-14, atol=0)
    r, dr = key(g["config"], "R0"), key(g["config"], "dr")
    hm = [p.hm(r), p.hm(r + .5 * dr), p.hm(r + dr)]
    np.testing.assert_allclose(hm, g["probe_hm"], rtol=1e-15, atol=0)


@pytest.mark.parametrize("name", golden_names("probe"))
def test_angle_tables_and_hamiltonian(name):
    g = golden(name)
    p = _port(g)
    r, dr = key(g["config"], "R0"), key(g["config"], "dr")
    c, s, d, l = p.probe(r, dr)
    if "probe_rpt" in g:
        # SA keeps the stage radii and dl = dr/2, dr, dr/2 (src/Phy_SA.cpp:121-147);
        # the port reports the dilution factor D(r) in the weight slot
        assert np.array_equal(g["probe_rpt"], [r, r + .5 * dr, r + dr])
        np.testing.assert_array_equal(l.reshape(-1), g["probe_dl"])
        R = key(g["config"], "Rv") / g["probe_rpt"]
        np.testing.assert_allclose(d.reshape(-1), .5 * (1. - np.sqrt(1. - R * R)) ** 2, rtol=1e-14, atol=0)
        assert not c.any() and not s.any()
    else:
        np.testing.assert_allclose(c.reshape(-1), g["probe_cos"], rtol=2e-13, atol=0)  # cancellation in 1 - r2 (1 - u) near the limb: rel. err ~ ulp / (2 cos^2)
        np.testing.assert_allclose(d.reshape(-1), g["probe_dcos"], rtol=2e-13, atol=0)
        np.testing.assert_allclose(l.reshape(-1), g["probe_dl"], rtol=2e-13, atol=0)
    if "probe_sin" in g:
        np.testing.assert_allclose(s.reshape(-1), g["probe_sin"], rtol=1e-15, atol=0)
    p.noise(g["meta"]["seed"], g["meta"]["noise_amp"])
    np.testing.assert_allclose(p.get_esum(0).reshape(-1), g["probe_esum0"], rtol=1e-13, atol=1e-17)
    for pt in range(3):
        h = p.calc_hvv(0, pt).reshape(-1)
        ref = g["probe_hvv%d" % pt]
        scale = np.max(np.abs(ref))
        assert np.max(np.abs(h - ref)) <= 1e-12 * scale


@pytest.mark.parametrize("name", golden_names("stages"))
def test_one_iteration_stage_buffers(name):
    g = golden(name)
    p = _port(g)
    p.noise(g["meta"]["seed"], g["meta"]["noise_amp"])
    r, dr = key(g["config"], "R0"), key(g["config"], "dr")
    me = p.iterate(r, dr)
    assert abs(me - np.sqrt(g["stage_err"].max())) <= 1e-6 * me
    for k in (1, 3, 4):
        ref = g["stage_psi%d" % k].reshape(p.shape)
        assert np.max(np.abs(p.get_state(k) - ref)) < 1e-13
    np.testing.assert_allclose(p.get_esum(4).reshape(-1), g["stage_esum4"], rtol=1e-11, atol=1e-16)


@pytest.mark.parametrize("name", golden_names("replay"))
def test_replay_of_reference_step_sequence(name):
    """Forced to the reference's accepted step sequence, every beam's
    polarization vector agrees to 1e-12 relative."""
    g = golden(name)
    p = _port(g)
    p.noise(g["meta"]["seed"], g["meta"]["noise_amp"])
    rb, dr = replay_inputs(g["config"], g["log"])
    p.replay(rb, dr)
    final = g["final"].reshape(p.shape)
    assert pol_rel_err(p.get_state(0), final) <= 1e-12


@pytest.mark.parametrize("name", ["ma_small_r10", "ma_small_r50", "maa_small_r10", "ma_nomatter", "sa_r10", "sa_r60"])
def test_free_running_loop_matches_reference(name):
    """The free-running loop takes the same accept/reject decisions; dr agrees
    to the precision the step-error cancellation allows."""
    g = golden(name)
    p = _port(g)
    p.noise(g["meta"]["seed"], g["meta"]["noise_amp"])
    out = p.run(max_iters=g["meta"]["summary"]["iterations"], log_cap=100000)
    log = g["log"]
    assert out["accepted"] == len(log)
    np.testing.assert_array_equal(out["log"][:, 0], log[:, 0])
    np.testing.assert_allclose(out["log"][:, 2], log[:, 2], rtol=1e-5)


def test_whole_run_fixture():
    """The reference's whole config-0 run (tests/golden/make_full_run.py), the
    target of tests/test_gpu_full_run.py: made from the configuration file as
    it is now, with the noise the GPU runs use, ending at Rn."""
    import os
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cfg = os.path.join(root, "xflat_gb300", "configs", "config0_ma.txt")
    ref = np.load(os.path.join(root, "tests", "golden", "c0_full_ref.npz"))
    text = str(ref["config"])
    assert text == open(cfg).read()
    assert int(ref["seed"]) == key(text, "seed", int) and float(ref["noise_amp"]) == key(text, "noise_amp")
    assert float(ref["r_end"]) == key(text, "Rn")
    assert ref["pee"].shape == (key(text, "Abins", int), key(text, "Ebins", int))
    assert np.all((ref["pee"] >= 0.) & (ref["pee"] <= 1.))
    assert int(ref["accepted"]) <= int(ref["iterations"]) < key(text, "Ts", int)
