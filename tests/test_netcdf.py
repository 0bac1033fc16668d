"""Snapshot files (the reference's NetCDF IO surface, src/IO_f.cpp) written by
the project's own classic-format writer, read back by scipy's independent
NetCDF-3 reader and by the project's reader.  CPU only."""
import ctypes

import numpy as np
import pytest

import xflat_gb300 as xg
from xflat_gb300 import _abi
from helpers import derive

scipy_io = pytest.importorskip("scipy.io")
dp = _abi.c_double_p


def _write(path, cfg, psi, r, dr):
    lib = _abi.load()
    return lib.xf_snapshot_write(str(path).encode(), ctypes.byref(cfg.raw), len(r), r.ctypes.data_as(dp),
                                 dr.ctypes.data_as(dp), psi.ctypes.data_as(dp))


@pytest.mark.parametrize("base,over,shape", [
    ("config0_ma.txt", dict(Abins=5, Ebins=7), (5, 4, 4, 7)),
    ("config3_maa.txt", dict(Abins=3, Pbins=2, Ebins=6), (3, 2, 4, 4, 6)),
    # SA: no angle dimension (src/Phy_SA.cpp:67-96), Abins ignored
    ("sa_bulb.txt", dict(Abins=9, Ebins=5), (4, 4, 5)),
])
def test_snapshot_file_matches_reference_layout(tmp_path, base, over, shape):
    cfg = xg.Config.from_text(derive(base, **over))
    rng = np.random.default_rng(0)
    nrec = 3
    psi = rng.normal(size=(nrec,) + shape)
    r = np.array([10.0, 10.5, 11.25])
    dr = np.array([1e-3, 2e-3, 4e-3])
    path = tmp_path / "xSnapshot0_0_.nc"
    assert _write(path, cfg, np.ascontiguousarray(psi), r, dr) == 0
    with scipy_io.netcdf_file(str(path), "r", mmap=False) as f:
        dims = ["r"] + (["theta"] if len(shape) >= 4 else []) + (["phi"] if len(shape) == 5 else []) + \
            ["prtcl", "comp", "ebin"]
        assert list(f.variables["psi"].dimensions) == dims
        assert f.variables["psi"].shape == (nrec,) + shape
        np.testing.assert_array_equal(f.variables["psi"][:], psi)
        np.testing.assert_array_equal(f.variables["r"][:], r)
        np.testing.assert_array_equal(f.variables["dr"][:], dr)
        att = f.variables["psi"]._attributes
        assert att["E0"] == cfg.E0 and att["E1"] == cfg.E1
        # src/IO_f.cpp:139-142 names: the literal advanced by the flavour index
        assert att["Teprature for particle"] == cfg.Tv[0]
        assert att["eprature for particle"] == cfg.Tv[1]
        assert att["ta for anti-particle"] == cfg.eta[2]
    # project reader: last and a chosen record
    lib = _abi.load()
    out = np.empty(int(np.prod(shape)))
    rr, dd, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_long()
    assert lib.xf_snapshot_read(str(path).encode(), -1, ctypes.byref(rr), ctypes.byref(dd), out.ctypes.data_as(dp),
                                ctypes.byref(n)) == 0
    assert n.value == nrec and rr.value == r[-1] and dd.value == dr[-1]
    np.testing.assert_array_equal(out, psi[-1].reshape(-1))
    assert lib.xf_snapshot_read(str(path).encode(), 1, ctypes.byref(rr), None, out.ctypes.data_as(dp), None) == 0
    np.testing.assert_array_equal(out, psi[1].reshape(-1))


def test_snapshot_read_errors(tmp_path):
    lib = _abi.load()
    assert lib.xf_snapshot_read(str(tmp_path / "missing.nc").encode(), -1, None, None, None, None) == _abi.XF_EIO
    bad = tmp_path / "bad.nc"
    bad.write_bytes(b"NOTCDF" + b"\0" * 64)
    assert lib.xf_snapshot_read(str(bad).encode(), -1, None, None, None, None) == _abi.XF_EIO
    cfg = xg.Config.from_text(derive("config0_ma.txt", Abins=2, Ebins=3))
    empty = tmp_path / "empty.nc"
    assert _write(empty, cfg, np.zeros(1), np.zeros(0), np.zeros(0)) == 0
    n = ctypes.c_long()
    assert lib.xf_snapshot_read(str(empty).encode(), -1, None, None, None, ctypes.byref(n)) == 0 and n.value == 0
    with scipy_io.netcdf_file(str(empty), "r", mmap=False) as f:
        assert f.variables["psi"].shape[0] == 0


def test_truncated_snapshot_is_an_io_error(tmp_path):
    cfg = xg.Config.from_text(derive("config0_ma.txt", Abins=3, Ebins=5))
    psi = np.random.default_rng(1).normal(size=(2, 3, 4, 4, 5))
    path = tmp_path / "t.nc"
    assert _write(path, cfg, np.ascontiguousarray(psi), np.array([1.0, 2.0]), np.array([.1, .2])) == 0
    data = path.read_bytes()
    lib = _abi.load()
    out = np.empty(psi[0].size)
    for cut in (len(data) - 8, len(data) // 2, 40, 3):
        path.write_bytes(data[:cut])
        rc = lib.xf_snapshot_read(str(path).encode(), -1, None, None, out.ctypes.data_as(dp), None)
        assert rc == _abi.XF_EIO, cut
