"""Double-float path (precision= df: every state, propagator, average and
moment as a pair of FP32 numbers, about 48 significant bits; MA, MAA and SA)
against the reference's own outputs and the FP64 path.

Bars: the reference's accepted-step sequence replayed, every beam's
polarization vector within 1e-10 relative of the reference's (the FP64
parity bar), and the same for the FP64 path's own accepted steps;
free-running windows take the FP64 path's accept/reject decisions; the step
error within 1e-5
relative of FP64's (it is the difference of two pair states, each exact to
about 3.6e-15 of the state)."""
import numpy as np
import pytest

import xflat_gb300 as xg
from helpers import derive, golden, golden_names, noise_state, pol_rel_err, replay_inputs

pytestmark = pytest.mark.gpu

POL_TOL = 1e-10


def _df(text):
    return text.replace("precision= fp64", "precision= df")


def _pair(text, seed=1, amp=1e-7):
    a = xg.Simulation(xg.Config.from_text(text))
    b = xg.Simulation(xg.Config.from_text(_df(text)))
    psi = noise_state(a.nbeams, a.ebins, seed, amp)
    a.set_state(psi)
    b.set_state(psi)
    return a, b


def pee(psi):
    """P_ee(E) = |a(E)|^2 of the nu_e beams (particle index 0)."""
    x = psi[0::4]
    return x[:, 0] ** 2 + x[:, 1] ** 2


@pytest.mark.parametrize("name", golden_names("replay"))
def test_replay_reference_step_sequence(name):
    g = golden(name)
    sim = xg.Simulation(xg.Config.from_text(_df(g["config"])))
    sim.set_state(noise_state(sim.nbeams, sim.ebins, g["meta"]["seed"], g["meta"]["noise_amp"]))
    rb, dr = replay_inputs(g["config"], g["log"])
    sim.replay(rb, dr)
    err = pol_rel_err(sim.get_state(0), g["final"].reshape(sim.state_shape))
    assert err <= POL_TOL, err


@pytest.mark.parametrize("r,dr,tol", [(10.0, 1.3e-8, 1e-13), (20.0, 1.2e-5, 1e-13), (50.0, 1.5e-4, 1e-13),
                                      (200.0, 5e-3, 1e-13), (40.0, 0.05, 1e-13), (10.0, 1e-3, 1e-11)])
def test_one_iteration_vs_fp64(r, dr, tol):
    """Includes a step with t = |h|^2 dl^2 above 1e-3 (the pair Horner series)
    and the first step of a run from 10 km (dl = 1e-3 km / cos, up to 0.06 km
    in the outermost angle bin, across the matter and neutrino potentials at
    the neutrinosphere: angles |h| dl far above 1 in most bins, the reduced
    branch, whose pairs keep the angle to about 1e-14 of itself, so the state
    bar grows with the largest angle; measured 2.6e-12 on a GB300).  The step
    error, which is all a rejected first step passes on, stays within 1e-5 of
    FP64's."""
    a, b = _pair(derive("config0_ma.txt", Abins=32, Ebins=64))
    me64 = a.step(r, dr)
    me2 = b.step(r, dr)
    assert abs(me2 - me64) <= 1e-5 * me64, (me2, me64)
    a.accept()
    b.accept()
    assert np.max(np.abs(b.get_state(0) - a.get_state(0))) <= tol


def _pair_rounded(x):
    """x as the double-float kernels see it: a hi FP32 part and an FP32 lo part."""
    h = x.astype(np.float32).astype(np.float64)
    return h + (x - h).astype(np.float32).astype(np.float64)


@pytest.mark.parametrize("half", [0, 1])
def test_propagator_coefficients_every_branch(half):
    """q (cos(|h| dl) - 1) and q sin(|h| dl) / |h| against numpy's FP64 sine
    on the pair-rounded inputs, in each series branch (warps of 32 inputs):
    the FP32 tail (t <= 1e-3), the pair Horner series (t <= 0.25) and the
    reduced branch, with angles up to 2000 and next to multiples of pi/2.
    The bar, 1e-14 + 4e-14 |h| dl, is the pairs' own precision of the angle
    (about 1e-14 of it) with a margin of four."""
    rng = np.random.default_rng(7 + half)
    theta = np.concatenate([10.0 ** rng.uniform(-4, np.log10(0.03), 128),
                            rng.uniform(0.04, 0.5, 128),
                            10.0 ** rng.uniform(np.log10(0.51), np.log10(2000.0), 256),
                            np.repeat(np.arange(1, 33) * np.pi / 2, 2) + np.tile([-1e-7, 1e-7], 32)])
    lam = 10.0 ** rng.uniform(-2, 4, theta.size)
    u = rng.normal(size=(theta.size, 3))
    h = _pair_rounded(u / np.linalg.norm(u, axis=1)[:, None] * lam[:, None])
    dl = _pair_rounded(theta / lam)
    lib = xg.load()
    cm, S = np.empty(theta.size), np.empty(theta.size)
    rc = lib.xf_probe_df_propagator(theta.size, xg._dp(np.ascontiguousarray(h.reshape(-1))), xg._dp(dl), half,
                                    xg._dp(cm), xg._dp(S))
    assert rc == 0
    q = 0.5 if half else 1.0
    lam_r = np.sqrt(np.sum(h * h, axis=1))
    th = lam_r * dl
    cm_ref = -2.0 * q * np.sin(0.5 * th) ** 2
    S_ref = q * np.sin(th) / lam_r
    tol = 1e-14 + 4e-14 * th
    assert np.all(np.abs(cm - cm_ref) <= q * tol), np.max(np.abs(cm - cm_ref) / tol)
    assert np.all(np.abs(S - S_ref) <= q * dl * tol), np.max(np.abs(S - S_ref) / (dl * tol))


@pytest.mark.parametrize("r0,iters", [(10.0, 400), (50.0, 300)])
def test_free_running_window_vs_fp64(r0, iters):
    text = derive("config0_ma.txt", Abins=64, Ebins=64, R0=r0, dr="1e-6")
    a, b = _pair(text)
    oa = a.evolutionLoop(max_iters=iters, log_cap=1000)
    ob = b.evolutionLoop(max_iters=iters, log_cap=1000)
    assert (oa["iterations"], oa["accepted"]) == (ob["iterations"], ob["accepted"])
    # the step error is the difference of two pair states (exact to about
    # 3.6e-15 of the state, against a difference near 1e-9): dr follows FP64's
    # to about 1e-6 relative per step, and the integrator's own truncation
    # error (eps0 = 1e-9 per step) follows the step sequence
    np.testing.assert_allclose(ob["log"][:, 2], oa["log"][:, 2], rtol=1e-4)
    d = np.max(np.abs(pee(a.get_state(0)) - pee(b.get_state(0))))
    assert d <= 1e-8, d


@pytest.mark.parametrize("r0,iters", [(10.0, 400), (50.0, 300)])
def test_fp64_step_sequence_replayed(r0, iters):
    """The FP64 path's accepted steps replayed in double-float: the arithmetic
    alone, every polarization vector within the FP64 parity bar."""
    text = derive("config0_ma.txt", Abins=64, Ebins=64, R0=r0, dr="1e-6")
    a, b = _pair(text)
    oa = a.evolutionLoop(max_iters=iters, log_cap=1000)
    rb, dr = replay_inputs(text, oa["log"][:oa["accepted"]])
    b.replay(rb, dr)
    assert pol_rel_err(b.get_state(0), a.get_state(0)) <= POL_TOL


def test_device_control_equals_host_loop():
    text = _df(derive("config0_ma.txt", Abins=32, Ebins=64))
    s1 = xg.Simulation(xg.Config.from_text(text))
    s2 = xg.Simulation(xg.Config.from_text(text))
    a = s1.evolutionLoop(max_iters=250, log_cap=1000)
    b = s2.evolutionLoop(max_iters=250, log_cap=1000, device_control=True, iters_per_launch=16)
    assert (a["iterations"], a["accepted"]) == (b["iterations"], b["accepted"])
    np.testing.assert_array_equal(a["log"], b["log"])
    assert np.array_equal(s1.get_state(0), s2.get_state(0))


def test_config1_shape_window_vs_fp64():
    """The 2048 x 4 x 512-bin workload: 20 device-controlled iterations from 50 km."""
    text = derive("config1_ma.txt", R0=50, dr="1.5e-4")
    a, b = _pair(text)
    oa = a.evolutionLoop(max_iters=20, device_control=True)
    ob = b.evolutionLoop(max_iters=20, device_control=True)
    assert (oa["iterations"], oa["accepted"]) == (ob["iterations"], ob["accepted"])
    assert abs(ob["last_max_err"] - oa["last_max_err"]) <= 1e-5 * oa["last_max_err"]
    d = np.max(np.abs(pee(a.get_state(0)) - pee(b.get_state(0))))
    assert d <= 1e-11, d
    # the candidate's per-beam survival sums from the pair state
    assert np.max(np.abs(a.survival() - b.survival())) <= 1e-11


def test_unitarity_without_renormalisation():
    """|a|^2 + |b|^2 = 1 holds without renormalisation: over 2000 steps of the
    stiff 10 km region it drifts by 1.65e-12 (GB300), a random walk of the
    pair state's rounding (2^-48 per component per step), far below anything
    that P_ee(E) at the 1e-5 level could see."""
    text = _df(derive("config0_ma.txt", Abins=32, Ebins=64))
    s = xg.Simulation(xg.Config.from_text(text))
    s.evolutionLoop(max_iters=2000, device_control=True)
    psi = s.get_state(0)
    n = psi[:, 0] ** 2 + psi[:, 1] ** 2 + psi[:, 2] ** 2 + psi[:, 3] ** 2
    assert np.max(np.abs(n - 1.0)) <= 3e-12


def test_unsupported_combinations():
    s = xg.Simulation(xg.Config.from_text(_df(derive("config0_ma.txt", Abins=8, Ebins=16))))
    assert s.lib.xf_set_option(s.h, b"renorm_every", 16.0) == xg._abi.XF_EUNSUPPORTED
    assert s.lib.xf_set_option(s.h, b"renorm_every", 0.0) == 0


# ------------------------------------------------------------------ MAA (16-scalar reduction)

MAA = dict(Abins=16, Pbins=8, Ebins=32)


@pytest.mark.parametrize("r,dr", [(12.0, 1.4e-6), (60.0, 2e-4), (40.0, 0.05)])
def test_maa_one_iteration_vs_fp64(r, dr):
    a, b = _pair(derive("config3_maa.txt", **MAA), 3, 1e-6)
    me64, me2 = a.step(r, dr), b.step(r, dr)
    assert abs(me2 - me64) <= 1e-5 * me64, (me2, me64)
    a.accept()
    b.accept()
    assert np.max(np.abs(b.get_state(0) - a.get_state(0))) <= 1e-13


@pytest.mark.parametrize("r0,iters", [(15.0, 300), (60.0, 200)])
def test_maa_fp64_step_sequence_replayed(r0, iters):
    text = derive("config3_maa.txt", R0=r0, dr="1e-6", **MAA)
    a, b = _pair(text, 3, 1e-6)
    oa = a.evolutionLoop(max_iters=iters, log_cap=iters)
    rb, dr = replay_inputs(text, oa["log"][:oa["accepted"]])
    b.replay(rb, dr)
    assert pol_rel_err(b.get_state(0), a.get_state(0)) <= POL_TOL


def test_maa_free_running_takes_fp64_decisions():
    text = derive("config3_maa.txt", R0=15, dr="1e-6", **MAA)
    a, b = _pair(text, 3, 1e-6)
    oa = a.evolutionLoop(max_iters=300, log_cap=300, device_control=True)
    ob = b.evolutionLoop(max_iters=300, log_cap=300, device_control=True)
    assert (oa["iterations"], oa["accepted"]) == (ob["iterations"], ob["accepted"])
    np.testing.assert_allclose(ob["log"][:, 2], oa["log"][:, 2], rtol=1e-4)
    assert np.max(np.abs(pee(a.get_state(0)) - pee(b.get_state(0)))) <= 1e-8


def test_maa_workload_shape_window_vs_fp64():
    """256 polar x 64 azimuthal x 4 x 128 energy bins (8.39 M): 6 iterations from 50 km."""
    text = derive("config3_maa.txt", R0=50, dr="1e-4")
    a, b = _pair(text, 3, 1e-6)
    oa = a.evolutionLoop(max_iters=6, device_control=True)
    ob = b.evolutionLoop(max_iters=6, device_control=True)
    assert (oa["iterations"], oa["accepted"]) == (ob["iterations"], ob["accepted"])
    assert abs(ob["last_max_err"] - oa["last_max_err"]) <= 1e-5 * oa["last_max_err"]
    assert np.max(np.abs(pee(a.get_state(0)) - pee(b.get_state(0)))) <= 1e-11


# ------------------------------------------------------------------ normal hierarchy

@pytest.mark.parametrize("base,over", [
    ("config0_ma.txt", dict(Abins=64, Ebins=64, R0=20, dr="1e-5")),
    ("config1_ma.txt", dict(Abins=128, Ebins=128, R0=50, dr="1.5e-4")),
    ("config3_maa.txt", dict(Abins=16, Pbins=8, Ebins=32, R0=15, dr="1e-6")),
])
def test_normal_hierarchy_vs_fp64(base, over):
    """dm2 = +3e-3 eV^2 (src/Parser.cpp:99-100: the hierarchy is the sign of
    dm2): free runs take FP64's decisions, and FP64's accepted steps replayed
    in double-float stay within the FP64 parity bar."""
    text = derive(base, dm2="3E-3", **over)
    a, b = _pair(text, 3, 1e-6)
    oa = a.evolutionLoop(max_iters=300, device_control=True, log_cap=300)
    ob = b.evolutionLoop(max_iters=300, device_control=True)
    assert (oa["iterations"], oa["accepted"]) == (ob["iterations"], ob["accepted"])
    assert np.max(np.abs(pee(a.get_state(0)) - pee(b.get_state(0)))) <= 1e-8
    c = xg.Simulation(xg.Config.from_text(_df(text)))
    c.set_state(noise_state(c.nbeams, c.ebins, 3, 1e-6))
    rb, dr = replay_inputs(text, oa["log"][:oa["accepted"]])
    c.replay(rb, dr)
    assert pol_rel_err(c.get_state(0), a.get_state(0)) <= POL_TOL
