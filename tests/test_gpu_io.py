"""Snapshot/Probability output during a run, resume from a snapshot, and the
xflat_gpu command-line driver (src/main.cpp argv contract)."""
import os
import subprocess

import numpy as np
import pytest

import xflat_gb300 as xg
from helpers import ROOT, derive, pol_rel_err

pytestmark = pytest.mark.gpu
scipy_io = pytest.importorskip("scipy.io")


def _cfg(tmp_path, dump_mode=3, base="config0_ma.txt", **over):
    kv = dict(Abins=8, Ebins=16, R0=20, dr="1e-5", dumpMode=dump_mode, r_step1="0.00005", r_step2="0.00005",
              filePrefix=str(tmp_path) + "/run")
    kv.update(over)
    return derive(base, **kv)


def test_dumps_during_run(tmp_path):
    # a radius trigger below any step size: every accepted step is written
    text = _cfg(tmp_path, r_step1="1e-12", r_step2="1e-12")
    sim = xg.Simulation(xg.Config.from_text(text))
    o = xg._abi.XfRunOpts()
    lib = sim.lib
    lib.xf_run_opts_default(o)
    o.max_iters = 60
    o.write_files = 1
    st = xg._abi.XfRunStats()
    assert lib.xf_run(sim.h, o, xg._abi.XF_STEP_CB(0), None, st) == 0
    assert lib.xf_io_close(sim.h) == 0
    snap = str(tmp_path / "runSnapshot0_0_.nc")
    prob = str(tmp_path / "runProbability0_0_.nc")
    with scipy_io.netcdf_file(snap, "r", mmap=False) as f:
        n = f.variables["r"].shape[0]
        assert n == st.accepted
        last = f.variables["psi"][n - 1].reshape(sim.nbeams, 4, sim.ebins)
        assert np.array_equal(last, sim.get_state(0))
        assert f.variables["r"][n - 1] == st.r_end
    with scipy_io.netcdf_file(prob, "r", mmap=False) as f:
        m = f.variables["r"].shape[0]
        sv = sim.survival()
        for p in range(4):
            np.testing.assert_allclose(f.variables["prtcl%d" % p][m - 1].reshape(-1), sv[:, p], rtol=1e-15)


def test_resume_continues_the_run(tmp_path):
    text = _cfg(tmp_path, dump_mode=1)
    a = xg.Simulation(xg.Config.from_text(text))
    o = xg._abi.XfRunOpts()
    a.lib.xf_run_opts_default(o)
    o.max_iters = 40
    o.write_files = 1
    st = xg._abi.XfRunStats()
    assert a.lib.xf_run(a.h, o, xg._abi.XF_STEP_CB(0), None, st) == 0
    a.lib.xf_io_close(a.h)
    snap = str(tmp_path / "runSnapshot0_0_.nc")
    with scipy_io.netcdf_file(snap, "r", mmap=False) as f:
        r_last = float(f.variables["r"][-1])
        dr_last = float(f.variables["dr"][-1])
        psi_last = f.variables["psi"][-1].reshape(a.nbeams, 4, a.ebins).copy()
    b = xg.Simulation(xg.Config.from_text(text.replace("dumpMode= 1", "dumpMode= 0")))
    r, dr = xg._abi.ctypes.c_double(), xg._abi.ctypes.c_double()
    assert b.lib.xf_resume(b.h, snap.encode(), r, dr) == 0
    assert r.value == r_last and dr.value == dr_last
    assert np.array_equal(b.get_state(0), psi_last)
    # the reference resumes with dr as stored (src/IO_f.cpp:214-217)
    c = xg.Simulation(xg.Config.from_text(text.replace("dumpMode= 1", "dumpMode= 0")))
    c.set_state(psi_last)
    ob = b.evolutionLoop(max_iters=20, r0=r.value, dr0=dr.value)
    oc = c.evolutionLoop(max_iters=20, r0=r_last, dr0=dr_last)
    assert ob["accepted"] == oc["accepted"]
    assert pol_rel_err(b.get_state(0), c.get_state(0)) <= 1e-14
    bad = xg.Simulation(xg.Config.from_text(derive("config0_ma.txt", Abins=9, Ebins=16)))
    assert bad.lib.xf_resume(bad.h, snap.encode(), r, dr) == xg._abi.XF_EINVAL


def test_command_line_driver(tmp_path):
    text = _cfg(tmp_path, dump_mode=1, Ts=30)
    cfg = tmp_path / "c.txt"
    cfg.write_text(text)
    exe = os.path.join(ROOT, "xflat_gb300", "_lib", "xflat_gpu")
    out = subprocess.run([exe, str(cfg)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert "Total iterations: 30" in out.stdout
    snap = tmp_path / "runSnapshot0_0_.nc"
    assert snap.exists()
    out2 = subprocess.run([exe, str(cfg), str(snap)], capture_output=True, text=True, timeout=120)
    assert out2.returncode == 0 and "Provided data file" in out2.stdout


@pytest.mark.parametrize("precision,iters", [("fp64", 40), ("mixed", 30), ("df", 30)])
def test_async_records_equal_states_of_each_accepted_step(tmp_path, precision, iters):
    """Every accepted step is dumped; the asynchronous copies and the writer
    thread must deliver, in order, exactly the state and survival of each
    step while the stepper runs ahead."""
    text = _cfg(tmp_path, r_step1="1e-12", r_step2="1e-12", Abins=16, Ebins=40).replace(
        "precision= fp64", "precision= " + precision)
    a = xg.Simulation(xg.Config.from_text(text))
    o = xg._abi.XfRunOpts()
    a.lib.xf_run_opts_default(o)
    o.max_iters = iters
    o.write_files = 1
    st = xg._abi.XfRunStats()
    assert a.lib.xf_run(a.h, o, xg._abi.XF_STEP_CB(0), None, st) == 0
    # the files are complete when xf_run returns (before xf_io_close)
    with scipy_io.netcdf_file(str(tmp_path / "runSnapshot0_0_.nc"), "r", mmap=False) as f:
        psi = f.variables["psi"][:].copy()
        r = f.variables["r"][:].copy()
    with scipy_io.netcdf_file(str(tmp_path / "runProbability0_0_.nc"), "r", mmap=False) as f:
        prob = np.stack([f.variables["prtcl%d" % p][:].reshape(len(r), -1) for p in range(4)], axis=-1)
    assert a.lib.xf_io_close(a.h) == 0
    # the same run stepped by hand, reading the state after every accepted step
    b = xg.Simulation(xg.Config.from_text(text))
    rr, dr = 20.0, 1e-5
    states, surv, radii = [], [], []
    eps0, ksi, maxdr = 1e-9, .94, .1
    for _ in range(iters):
        me = b.step(rr, dr)
        if me < eps0:
            rr += dr
            b.accept()
            states.append(b.get_state(0))
            surv.append(b.survival())
            radii.append(rr)
        dr = min(dr * (ksi * np.sqrt(eps0 / me)), maxdr)  # src/Nmr.cpp:247 operation order
    assert len(states) == st.accepted == len(r)
    np.testing.assert_array_equal(r, radii)
    for k in range(len(states)):
        assert np.array_equal(psi[k].reshape(states[k].shape), states[k]), k
        np.testing.assert_array_equal(prob[k].reshape(-1, 4), surv[k].reshape(-1, 4))


def _files(tmp_path, text, device, iters, k=5):
    sim = xg.Simulation(xg.Config.from_text(text))
    o = xg._abi.XfRunOpts()
    sim.lib.xf_run_opts_default(o)
    o.max_iters = iters
    o.write_files = 1
    o.device_control = 1 if device else 0
    o.iters_per_launch = k
    st = xg._abi.XfRunStats()
    assert sim.lib.xf_run(sim.h, o, xg._abi.XF_STEP_CB(0), None, st) == 0, sim.lib.xf_last_error(sim.h)
    assert sim.lib.xf_io_close(sim.h) == 0
    out = {}
    for name in sorted(os.listdir(tmp_path)):
        with scipy_io.netcdf_file(str(tmp_path / name), "r", mmap=False) as f:
            out[name] = {v: f.variables[v][:].copy() for v in f.variables}
    return out, st, sim.get_state(0)


@pytest.mark.parametrize("base,precision", [("config0_ma.txt", "fp64"), ("config0_ma.txt", "mixed"),
                                            ("config0_ma.txt", "df"), ("config3_maa.txt", "fp64"),
                                            ("config3_maa.txt", "mixed"), ("config3_maa.txt", "df")])
def test_device_control_writes_the_host_loops_files(tmp_path, base, precision):
    """Under device control the step controller evaluates the dump triggers
    and phase A stages the records: the files equal, record for record, those
    of the host-driven loop (radius and iteration triggers, both kinds,
    rotation every 4 Snapshot records, sync, a record decided at the last
    step, several graph launches)."""
    over = dict(dumpMode=3, r_step1="2.5e-5", r_step2="1e-5", itr_step1=7, newFile_step=4, sync_step=3,
                t_step1=300000, t_step2=300000, Abins=12, Ebins=24)
    a_dir, b_dir = tmp_path / "host", tmp_path / "dev"
    a_dir.mkdir()
    b_dir.mkdir()
    if base == "config3_maa.txt":
        over.update(Abins=6, Pbins=3, Ebins=20)
    ta = _cfg(a_dir, base=base, **over).replace("precision= fp64", "precision= " + precision)
    tb = _cfg(b_dir, base=base, **over).replace("precision= fp64", "precision= " + precision)
    fa, sa, pa = _files(a_dir, ta, False, 61)
    fb, sb, pb = _files(b_dir, tb, True, 61)
    assert (sa.iterations, sa.accepted) == (sb.iterations, sb.accepted)
    assert np.array_equal(pa, pb)
    assert list(fa) == list(fb) and len(fa) >= 4
    for name in fa:
        for v in fa[name]:
            assert np.array_equal(fa[name][v], fb[name][v]), (name, v)


@pytest.mark.parametrize("device", [False, True])
def test_unwritable_output_is_reported(tmp_path, device):
    """Files that cannot be created end the run with XF_EIO and a message
    naming the file (the reference exits on a NetCDF error, src/IO_f.cpp:88)."""
    text = _cfg(tmp_path / "missing" / "dir", r_step1="1e-12")
    sim = xg.Simulation(xg.Config.from_text(text))
    o = xg._abi.XfRunOpts()
    sim.lib.xf_run_opts_default(o)
    o.max_iters = 5
    o.write_files = 1
    o.device_control = 1 if device else 0
    st = xg._abi.XfRunStats()
    assert sim.lib.xf_run(sim.h, o, xg._abi.XF_STEP_CB(0), None, st) == xg._abi.XF_EIO
    assert b"cannot create" in sim.lib.xf_last_error(sim.h)
    assert sim.lib.xf_io_close(sim.h) in (0, xg._abi.XF_EIO)
    # the handle stays usable
    out = sim.evolutionLoop(max_iters=3)
    assert out["iterations"] == 3
