"""Known-answer tests from the mathematics (no reference run needed).

With no neutrino luminosity and no matter, the neutrino-neutrino term and
the matter term vanish and every bin evolves under its constant vacuum
Hamiltonian.  In the single-angle geometry the stepper's two half steps
compose to the full step exactly (U(dr/2) U(dr/2) = U(dr)), so after any
accepted step sequence psi(r) = exp(-i h_vac (r - R0)) psi(R0): a closed form
for every bin, computed here independently of the CUDA path."""
import numpy as np
import pytest

import xflat_gb300 as xg
from helpers import derive

pytestmark = pytest.mark.gpu


def _vacuum_text(precision):
    kv = dict(Ebins=48, R0=10, Rn="30", dr="1e-3", max_dr=".05", hasMatter=0, Ts=100000)
    for k in ("Lve", "Lv_e", "Lvt", "Lv_t"):
        kv[k] = "0"
    return derive("sa_bulb.txt", **kv).replace("precision= fp64", "precision= " + precision)


def _closed_form(psi0, hvac, L):
    """U = cos(lam L) - i sin(lam L)/lam sigma(h), sigma(h) = [[h00, h01], [h01, -h00]] (real h01)."""
    h00, h01 = hvac[:, 0], hvac[:, 1]
    lam = np.sqrt(h00 * h00 + h01 * h01)
    c, s = np.cos(lam * L), np.sin(lam * L) / lam
    a = psi0[:, 0] + 1j * psi0[:, 1]
    b = psi0[:, 2] + 1j * psi0[:, 3]
    a2 = c * a - 1j * s * (h00 * a + h01 * b)
    b2 = c * b - 1j * s * (h01 * a - h00 * b)
    return np.stack([a2.real, a2.imag, b2.real, b2.imag], axis=1)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("mixed", 1e-5)])
def test_vacuum_oscillation_closed_form(precision, tol):
    sim = xg.Simulation(xg.Config.from_text(_vacuum_text(precision)))
    sim.set_noise(3, 1e-2)
    psi0 = sim.get_state(0)
    out = sim.evolutionLoop(device_control=True)
    assert out["r_end"] == pytest.approx(30.0, abs=1e-12)
    assert out["accepted"] == out["iterations"] > 100   # nothing to reject: the step error is rounding
    hvac = sim.tables()["hvac"].reshape(-1, 2)
    ref = _closed_form(psi0, hvac, out["r_end"] - 10.0)
    got = sim.get_state(0)
    # about 50 oscillation lengths at the lowest energies
    assert np.max(np.abs(got - ref)) <= tol


def test_fp64_evolution_is_unitary():
    """|a|^2 + |b|^2 of every bin stays 1 to rounding over a coupled run."""
    sim = xg.Simulation(xg.Config.from_text(derive("config0_ma.txt", Abins=48, Ebins=64, R0=10, dr="1e-6")))
    sim.set_noise(1, 1e-3)
    sim.evolutionLoop(max_iters=400, device_control=True)
    psi = sim.get_state(0)
    assert np.max(np.abs((psi ** 2).sum(axis=1) - 1.0)) < 1e-13
