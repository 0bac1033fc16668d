"""Host-side logic of the product (C++ through the C ABI, no GPU calls):
config parsing with the reference's units, tables, matter, initial state, and
the exported symbol set."""
import ctypes
import os
import re

import numpy as np
import pytest

import xflat_gb300 as xg
from xflat_gb300 import _abi
from helpers import CONFIGS, TempConfig, derive, golden, golden_names, noise_state
from oracle.port import Port


def test_library_exports_every_declared_symbol():
    lib = _abi.load()
    names = _abi.header_symbols()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_config_units_and_keys():
    c = xg.Parser(os.path.join(CONFIGS, "config0_ma.txt"))
    MEV, EV2, ERG = 5.067731161976211e+15, 2.568189913006477e+19, 1.053613095584080e+16
    assert c.abins == 256 and c.ebins == 64 and c.pbins == 1 and c.flvs == 2
    assert c.E0 == 1 * MEV and c.E1 == 60 * MEV
    assert c.dm2 == -3e-3 * EV2
    assert c.theta2 == 0.2
    assert list(c.Lv) == [1e51 * ERG] * 4
    assert c.Tv[0] == 2.76 * MEV and c.Tv[3] == 6.26 * MEV
    assert c.eps0 == 1e-9 and c.ksi == 0.94 and c.R0 == 10 and c.Rn == 300
    assert c.geometry == xg.XF_GEOM_MA and c.precision == xg.XF_PREC_FP64
    assert c.seed == 1 and c.noise_amp == 1e-7
    c3 = xg.Parser(os.path.join(CONFIGS, "config3_maa.txt"))
    assert c3.geometry == xg.XF_GEOM_MAA and c3.pbins == 64
    c2 = xg.Parser(os.path.join(CONFIGS, "config2_ma_mixed.txt"))
    assert c2.precision == xg.XF_PREC_MIXED
    text = open(os.path.join(CONFIGS, "config0_ma.txt")).read()
    for word, prec in (("df", xg.XF_PREC_DF), ("DF", xg.XF_PREC_DF), ("mixed", xg.XF_PREC_MIXED)):
        assert xg.Config.from_text(text.replace("precision= fp64", "precision= " + word)).precision == prec
    with pytest.raises(xg.XflatError):
        xg.Config.from_text(text.replace("precision= fp64", "precision= fp16"))
    sa = xg.Parser(os.path.join(CONFIGS, "sa_bulb.txt"))
    assert sa.geometry == xg.XF_GEOM_SA and sa.ebins == 512


def test_config_reference_syntax():
    # comments, unknown keys, trailing comments, nb0 scaling, int keys parsed like istream >> int
    text = "# c\n\nfoo= 3\nnb0= 1.63E+36 # cm^-3\nAbins= 12\nEbins= 7\nt_step1= 300000.\nfilePrefix= abc\n"
    c = xg.Config.from_text(text)
    assert c.nb0 == 1.63e36 * 1e15
    assert c.abins == 12 and c.ebins == 7 and c.tstep1 == 300000
    assert c.file_prefix == b"abc"
    with pytest.raises(xg.XflatError):
        xg.Config.from_text("geometry= XYZ\n")
    with pytest.raises(xg.XflatError):
        xg.Parser("/nonexistent/config.txt")


@pytest.mark.parametrize("name", golden_names("probe"))
def test_host_tables_match_reference(name):
    g = golden(name)
    c = xg.Config.from_text(g["config"])
    lib = _abi.load()
    ne = c.ebins
    fv, hv, le, ev = np.empty(4 * ne), np.empty(2 * ne), np.empty(4), np.empty(4)
    dp = _abi.c_double_p
    assert lib.xf_host_tables(ctypes.byref(c.raw), fv.ctypes.data_as(dp), hv.ctypes.data_as(dp),
                              le.ctypes.data_as(dp), ev.ctypes.data_as(dp)) == 0
    np.testing.assert_allclose(fv, g["probe_fv"], rtol=1e-14, atol=0)
    np.testing.assert_allclose(hv, g["probe_hvac"], rtol=1e-14, atol=0)
    np.testing.assert_allclose(le, g["probe_LE"], rtol=1e-14, atol=0)
    np.testing.assert_allclose(ev, g["probe_Ev"], rtol=1e-14, atol=0)
    r, dr = c.R0, c.dr
    hm = []
    for x in (r, r + .5 * dr, r + dr):
        o = ctypes.c_double()
        assert lib.xf_host_matter(ctypes.byref(c.raw), x, ctypes.byref(o)) == 0
        hm.append(o.value)
    np.testing.assert_allclose(hm, g["probe_hm"], rtol=1e-15, atol=0)


def test_matter_profile_is_the_baseline_lambda():
    """lambda(r) = 1e3 (10/r)^3 km^-1 with the workload's matter keys; hm = lambda/2."""
    c = xg.Parser(os.path.join(CONFIGS, "config0_ma.txt"))
    lib = _abi.load()
    for r in (10., 50., 300.):
        o = ctypes.c_double()
        lib.xf_host_matter(ctypes.byref(c.raw), r, ctypes.byref(o))
        assert abs(2 * o.value / (1e3 * (10. / r) ** 3) - 1) < 1e-5


@pytest.mark.parametrize("geom,a,p,e", [("config0_ma.txt", 13, 1, 21), ("config3_maa.txt", 5, 3, 9),
                                        ("sa_bulb.txt", 6, 1, 11)])
def test_host_initial_state_matches_numpy_and_oracle(geom, a, p, e):
    text = derive(geom, Abins=a, Pbins=p, Ebins=e)
    c = xg.Config.from_text(text)
    # SA: one trajectory whatever Abins says
    nb = (1 if c.geometry == xg.XF_GEOM_SA else a) * (p if c.geometry == xg.XF_GEOM_MAA else 1) * 4
    psi = np.empty(nb * 4 * e)
    assert _abi.load().xf_host_initial_state(ctypes.byref(c.raw), 7, 1e-6, psi.ctypes.data_as(_abi.c_double_p)) == 0
    ref = noise_state(nb, e, 7, 1e-6)
    assert np.array_equal(psi.reshape(nb, 4, e), ref)
    with TempConfig(text) as path:
        port = Port(path)
    port.noise(7, 1e-6)
    assert np.array_equal(port.get_state(0), ref)


def test_invalid_config_is_rejected_without_gpu_work():
    lib = _abi.load()
    c = xg.Config.from_text(derive("config0_ma.txt", Abins=0))
    h = ctypes.c_void_p()
    assert lib.xf_create(ctypes.byref(c.raw), ctypes.byref(h)) == _abi.XF_EINVAL
    c = xg.Config.from_text(derive("config0_ma.txt", Flvs=3))
    assert lib.xf_create(ctypes.byref(c.raw), ctypes.byref(h)) == _abi.XF_EUNSUPPORTED
    assert lib.xf_create(None, ctypes.byref(h)) == _abi.XF_EINVAL


def test_double_float_series_fast_path():
    """The double-float propagator's fast series (xflat_gb300/csrc/xf_df.cuh,
    dcoeffs, every lane t <= 1e-3): C - 1 = t c1 and S/dl - 1 = t s1 with
    c1 = -1/2 + t (1/24 - t/720) and s1 = -1/6 + t (1/120 - t/5040), the
    tails rounded as the FP32 FMA and product of the kernel, the leading
    constants exact.  Against cos(sqrt t) - 1 and sin(sqrt t)/sqrt t - 1 at
    40 digits: below 5e-15 absolute (3.1e-15 at t = 1e-3; the pair arithmetic
    itself carries about 2^-48 of C and S)."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    f32 = np.float32

    def fma32(a, b, c):  # one rounding, as fmaf: the float32 product is exact in float64
        return f32(np.float64(a) * np.float64(b) + np.float64(c))

    worst_c = worst_s = 0.
    for t in np.concatenate([np.geomspace(1e-12, 1e-3, 400), [1e-3]]):
        th = f32(t)
        tail_c = f32(th * fma32(th, f32(-1. / 720.), f32(1. / 24.)))
        tail_s = f32(th * fma32(th, f32(-1. / 5040.), f32(1. / 120.)))
        cm = t * (-0.5 + float(tail_c))
        sm = t * (float(mp.mpf(-1) / 6) + float(tail_s))
        x = mp.sqrt(mp.mpf(float(t)))
        worst_c = max(worst_c, abs(float(mp.cos(x) - 1 - cm)))
        worst_s = max(worst_s, abs(float(mp.sin(x) / x - 1 - sm)))
    assert worst_c <= 5e-15 and worst_s <= 5e-15, (worst_c, worst_s)


def test_double_float_large_angle_constants():
    """The double-float propagator's large-angle branch (xflat_gb300/csrc/
    xf_df.cuh, dcoeffs, t > 0.25): pi/2 as three FP32 numbers whose sum is
    pi/2 to 1.1e-23 (each product with an integer n < 2^24 is then an exact
    pair), 2/pi rounded to FP32, and the series of the remainder (|r| <=
    pi/4 + 1e-3) truncated below 4e-18: cos r - 1 after the u^8 term and
    sin r after the r u^8 term (u = r^2), the first omitted terms u^9/18!
    and r u^9/19!."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 50
    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "xflat_gb300", "csrc",
                            "xf_df.cuh")).read()
    hexf = r"(-?0x[0-9a-f.]+p[-+]?\d+)f"
    m = re.search(r"kPio2a = %s, kPio2b = %s, kPio2c = %s" % (hexf, hexf, hexf), src)
    assert m, "pi/2 split not found"
    parts = [float.fromhex(x) for x in m.groups()]
    for x in parts:
        assert float(np.float32(x)) == x
    assert abs(sum(mp.mpf(x) for x in parts) - mp.pi / 2) < mp.mpf("1.1e-23")
    m = re.search(r"kTwoOverPi = %s" % hexf, src)
    assert m and float.fromhex(m.group(1)) == float(np.float32(float(2 / mp.pi)))
    r = mp.pi / 4 + mp.mpf("1e-3")
    u = r * r
    assert u ** 9 / mp.factorial(18) < mp.mpf("4e-18")
    assert r * u ** 9 / mp.factorial(19) < mp.mpf("4e-18")
    # the kernel's coefficient tables run to 1/16! and 1/17! (index 7)
    assert "XF_DFC(1.0 / 20922789888000.0)" in src and "XF_DFC(1.0 / 355687428096000.0)" in src
    assert mp.factorial(16) == 20922789888000 and mp.factorial(17) == 355687428096000
