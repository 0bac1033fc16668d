"""xf_calc_hvv_static: the allocation-free Hamiltonian evaluation.

It serves callers that cannot call cudaMalloc (device memory owned and
budgeted up front by another allocator, or per-step loops that must not pay
cudaMalloc's implicit synchronisation): the caller owns every input and
output buffer, and the entry point's scratch is a fixed device array inside
the library.  Its result is checked through the C ABI against the existing
entry point xf_calc_hvv, on two calls in a row and after the state changed.
This file is collected last so that a run stopping at the first failure has
already run every other test.  It is also pinned directly to the reference's
own Hamiltonians (the probe_hvv fixtures written by the reference built from
its sources), for MA and MAA."""
import ctypes

import numpy as np
import pytest

import xflat_gb300 as xg
from helpers import derive, golden, key

pytestmark = pytest.mark.gpu

SQRT2, PI = 1.41421356237, 3.14159265359
GF = 1.16637E-11 * 3.893793036626876e-32


def _coefficients(sim, cfg):
    """Hamiltonian coefficient and azimuth tables as the reference builds them
    (src/Phy_MA.cpp:271, src/Phy_MAA.cpp:176-185 and 297-298)."""
    P = sim.pbins
    if cfg.geometry == xg.XF_GEOM_MAA:
        dphi = (PI * 2.) / P
        phi, cp, sp = dphi * .5, [], []
        for _ in range(P):
            sp.append(np.sin(phi))
            cp.append(np.cos(phi))
            phi += dphi
        kappa = ((SQRT2 * GF) / (4. * PI * PI * cfg.Rv * cfg.Rv)) * dphi
        return kappa, np.array(cp), np.array(sp)
    return (SQRT2 * GF) / (2. * PI * cfg.Rv * cfg.Rv), np.ones(1), np.zeros(1)


def _static_hvv(sim, cfg, pt, r, dr, dev):
    import torch
    epad = (sim.ebins + 31) // 32 * 32
    psi = np.zeros((sim.nbeams, 4, epad))
    psi[:, :, :sim.ebins] = sim.get_state(0)
    t = sim.tables()
    fv = np.zeros((4, epad))
    fv[:, :sim.ebins] = t["fv"]
    c, s, d, _ = sim.calcAngleBins(r, dr)
    kappa, cp, sp = _coefficients(sim, cfg)
    bufs = [torch.tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)
            for x in (psi, fv, c[pt], s[pt], d[pt], cp, sp)]
    hvv = torch.zeros(4 * sim.abins * sim.pbins, dtype=torch.float64, device=dev)
    le = np.ascontiguousarray(t["LE"])
    stream = torch.cuda.current_stream(dev)
    rc = sim.lib.xf_calc_hvv_static(cfg.geometry, sim.abins, sim.pbins, sim.ebins, epad,
                                    *[ctypes.c_void_p(b.data_ptr()) for b in bufs],
                                    le.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), kappa,
                                    ctypes.c_void_p(hvv.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0
    torch.cuda.synchronize(dev)
    return hvv.cpu().numpy().reshape(-1, 4)


@pytest.mark.parametrize("base,over", [
    ("config0_ma.txt", dict(Abins=64, Ebins=48)),
    ("config3_maa.txt", dict(Abins=12, Pbins=10, Ebins=40)),
])
def test_static_entry_point_matches_xf_calc_hvv(base, over):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    cfg = xg.Config.from_text(derive(base, **over))
    sim = xg.Simulation(cfg)
    r, dr = 20.0, 1e-5
    for round_ in range(2):
        if round_ == 1:
            sim.evolutionLoop(max_iters=5, r0=r, dr0=dr)   # new state between the calls
        for pt in range(3):
            ref = sim.calc_Hvv(0, pt, r, dr)
            tol = 1e-12 * np.max(np.abs(ref))   # same bar as the moment-reduction parity tests
            first = _static_hvv(sim, cfg, pt, r, dr, dev)
            second = _static_hvv(sim, cfg, pt, r, dr, dev)
            assert np.max(np.abs(first - ref)) <= tol
            assert np.max(np.abs(second - ref)) <= tol


@pytest.mark.parametrize("name", ["ma_small_r10", "ma_c0shape", "maa_small_r10", "maa_ragged"])
def test_static_entry_point_matches_reference_probes(name):
    """phy::calc_Hvv of the reference at its three stage points, on the
    reference's initial state, against the allocation-free entry point fed the
    same state and this library's angle tables (which match the reference's to
    2e-13)."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    g = golden(name)
    cfg = xg.Config.from_text(g["config"])
    sim = xg.Simulation(cfg)
    sim.set_noise(g["meta"]["seed"], g["meta"]["noise_amp"])
    r, dr = key(g["config"], "R0"), key(g["config"], "dr")
    for pt in range(3):
        ref = g["probe_hvv%d" % pt].reshape(-1, 4)
        # the moment sums are reduced in a different order than the reference's serial loop
        tol = 1e-12 * np.max(np.abs(ref))
        for _ in range(2):
            h = _static_hvv(sim, cfg, pt, r, dr, dev)
            assert np.max(np.abs(h - ref)) <= tol, pt


def test_static_entry_point_rejects_sizes_beyond_its_scratch():
    lib = xg.load()
    one = ctypes.c_void_p(1)
    le = (ctypes.c_double * 4)(1., 1., 1., 1.)
    # 16385 angle bins * 4 particles = 65540 beams > 65536
    rc = lib.xf_calc_hvv_static(0, 16385, 1, 8, 32, one, one, one, one, one, one, one, le, 1.0, one, None)
    assert rc == xg._abi.XF_EINVAL
