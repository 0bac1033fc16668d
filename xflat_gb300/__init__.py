"""GB300 implementation of XFLAT's per-radius-step hot path.

Python host mirror of the C ABI in include/xflat_gpu.h.  Names follow the
reference's module interface (src/Parser.cpp, include/Phy.h, include/Nmr.h,
include/Matt.h, include/Fio.h):

    cfg = Parser("config.txt")                 # Parser(configFile)
    sim = Simulation(cfg)                      # nbm::init + phy::init + nmr::init + matt::init
    sim.fillInitData(psi)                      # fio::fillInitData (psi: [beam][comp][ebin])
    hm = sim.getHm(r)                          # matt::getHm
    cos, sin, dcos, dl = sim.calcAngleBins(r, dr)  # phy::calcAngleBins + calcDeltaLs
    hvv = sim.calc_Hvv(0, pt, r, dr)           # phy::calc_Hvv
    max_err = sim.step(r, dr); sim.accept()    # one iteration of src/Nmr.cpp:153-249
    stats = sim.evolutionLoop()                # nmr::evolutionLoop

Errors raise XflatError carrying the native status code; there is no CPU
fallback.
"""
import ctypes
import math

import numpy as np

from . import _abi
from ._abi import (XF_EINVAL, XF_ENAN, XF_GEOM_MA, XF_GEOM_MAA, XF_GEOM_SA, XF_OK, XF_PREC_DF, XF_PREC_FP64, XF_PREC_MIXED, XfConfig,
                   XfRunOpts, XfRunStats)

__all__ = ["XflatError", "Parser", "Config", "Simulation", "Batch", "load", "XF_GEOM_MA", "XF_GEOM_MAA", "XF_GEOM_SA",
           "XF_PREC_DF", "XF_PREC_FP64", "XF_PREC_MIXED"]


class XflatError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (status %d)" % (msg, status))
        self.status = status


def load():
    return _abi.load()


def _dp(a):
    return a.ctypes.data_as(_abi.c_double_p)


def _check(rc, what, handle=None, lib=None):
    if rc != XF_OK:
        lib = lib or _abi.load()
        msg = lib.xf_strerror(rc).decode()
        if handle:
            detail = lib.xf_last_error(handle)
            if detail:
                msg += ": " + detail.decode()
        raise XflatError(rc, "%s failed: %s" % (what, msg))


class Config:
    """Run configuration (the reference's Util:: values after parse-time unit
    conversion, src/Parser.cpp:25-127)."""

    def __init__(self, raw=None):
        lib = _abi.load()
        if raw is None:
            raw = XfConfig()
            _check(lib.xf_config_default(ctypes.byref(raw)), "xf_config_default")
        self.raw = raw

    @classmethod
    def from_file(cls, path):
        c = cls()
        _check(_abi.load().xf_config_load(path.encode(), ctypes.byref(c.raw)), "xf_config_load(%s)" % path)
        return c

    @classmethod
    def from_text(cls, text):
        c = cls()
        _check(_abi.load().xf_config_parse(text.encode(), ctypes.byref(c.raw)), "xf_config_parse")
        return c

    def copy(self):
        raw = XfConfig()
        ctypes.memmove(ctypes.byref(raw), ctypes.byref(self.raw), ctypes.sizeof(XfConfig))
        return Config(raw)

    def __getattr__(self, k):
        if k == "raw":
            raise AttributeError(k)
        return getattr(self.raw, k)

    def __setattr__(self, k, v):
        if k == "raw":
            object.__setattr__(self, k, v)
        else:
            setattr(self.raw, k, v)


def Parser(path):
    """Parser(configFile) (src/Parser.cpp:13-23): returns a Config."""
    return Config.from_file(path)


class Simulation:
    """One simulation's device-resident state and the hot-path entry points."""

    def __init__(self, cfg):
        self.lib = _abi.load()
        self.cfg = cfg if isinstance(cfg, Config) else Config.from_file(cfg)
        h = ctypes.c_void_p()
        _check(self.lib.xf_create(ctypes.byref(self.cfg.raw), ctypes.byref(h)), "xf_create")
        self.h = h
        nb, ne, na, npb = (ctypes.c_int() for _ in range(4))
        self.lib.xf_dims(self.h, ctypes.byref(nb), ctypes.byref(ne), ctypes.byref(na), ctypes.byref(npb))
        self.nbeams, self.ebins, self.abins, self.pbins = nb.value, ne.value, na.value, npb.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.xf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def state_shape(self):
        return (self.nbeams, 4, self.ebins)

    def _c(self, rc, what):
        _check(rc, what, self.h, self.lib)

    # -- state (fio::fillInitData / phy::initBeam)
    def set_state(self, psi):
        psi = np.ascontiguousarray(psi, dtype=np.float64).reshape(-1)
        if psi.size != self.nbeams * 4 * self.ebins:
            raise XflatError(XF_EINVAL, "state has %d values, expected %d" % (psi.size, self.nbeams * 4 * self.ebins))
        self._c(self.lib.xf_set_state(self.h, _dp(psi)), "xf_set_state")

    fillInitData = set_state

    def get_state(self, which=0, out=None):
        """Reads buffer `which` (0 psi0, 1 psi1, 3 psi3, 4 psi4); `out` may be a
        caller-owned (e.g. pinned) float64 buffer of nbeams*4*ebins values."""
        n = self.nbeams * 4 * self.ebins
        if out is None:
            out = np.empty(n)
        elif out.dtype != np.float64 or out.size != n or not out.flags.c_contiguous:
            raise XflatError(XF_EINVAL, "out must be a contiguous float64 buffer of %d values" % n)
        self._c(self.lib.xf_get_state(self.h, int(which), _dp(out)), "xf_get_state")
        return out.reshape(self.state_shape)

    def set_noise(self, seed, amp):
        self._c(self.lib.xf_set_noise(self.h, int(seed), float(amp)), "xf_set_noise")

    # -- tables
    def tables(self):
        fv = np.empty(4 * self.ebins)
        hv = np.empty(2 * self.ebins)
        le = np.empty(4)
        ev = np.empty(4)
        self._c(self.lib.xf_tables(self.h, _dp(fv), _dp(hv), _dp(le), _dp(ev)), "xf_tables")
        return dict(fv=fv.reshape(4, self.ebins), hvac=hv, LE=le, Ev=ev)

    def getHm(self, r):
        out = ctypes.c_double()
        self._c(self.lib.xf_matter(self.h, float(r), ctypes.byref(out)), "xf_matter")
        return out.value

    def calcAngleBins(self, r, dr):
        n = 3 * self.abins
        c, s, d, l = (np.empty(n) for _ in range(4))
        self._c(self.lib.xf_angle_bins(self.h, float(r), float(dr), _dp(c), _dp(s), _dp(d), _dp(l)), "xf_angle_bins")
        return c.reshape(3, -1), s.reshape(3, -1), d.reshape(3, -1), l.reshape(3, -1)

    def calc_Hvv(self, which, pt, r, dr):
        out = np.empty(4 * self.abins * self.pbins)
        self._c(self.lib.xf_calc_hvv(self.h, int(which), int(pt), float(r), float(dr), _dp(out)), "xf_calc_hvv")
        return out.reshape(-1, 4)

    # -- stepping (src/Nmr.cpp:153-249)
    def step(self, r, dr):
        me = ctypes.c_double()
        rc = self.lib.xf_step(self.h, float(r), float(dr), ctypes.byref(me))
        if rc == XF_ENAN:
            return float("nan")
        self._c(rc, "xf_step")
        return me.value

    def accept(self):
        self._c(self.lib.xf_accept(self.h), "xf_accept")

    def replay(self, r_before, dr):
        rb = np.ascontiguousarray(r_before, dtype=np.float64)
        d = np.ascontiguousarray(dr, dtype=np.float64)
        self._c(self.lib.xf_replay(self.h, _dp(rb), _dp(d), len(rb)), "xf_replay")

    def evolutionLoop(self, max_iters=-1, device_control=False, iters_per_launch=16, r0=None, dr0=None,
                      log_cap=0, time_phases=False, callback=None):
        """nmr::evolutionLoop (src/Nmr.cpp:89-262).  Returns a dict of run stats
        (and 'log', an array of accepted (itr, r_after, dr_used), when log_cap > 0)."""
        o = XfRunOpts()
        self.lib.xf_run_opts_default(ctypes.byref(o))
        o.max_iters = int(max_iters)
        o.device_control = int(bool(device_control))
        o.iters_per_launch = int(iters_per_launch)
        o.time_phases = int(bool(time_phases))
        o.r0 = math.nan if r0 is None else float(r0)
        o.dr0 = math.nan if dr0 is None else float(dr0)
        log = None
        if log_cap > 0:
            log = np.zeros(3 * int(log_cap))
            o.log = _dp(log)
            o.log_cap = int(log_cap)
        st = XfRunStats()
        if callback is not None:
            cb = _abi.XF_STEP_CB(lambda u, itr, r, dr: int(bool(callback(itr, r, dr))))
        else:
            cb = ctypes.cast(None, _abi.XF_STEP_CB)
        rc = self.lib.xf_run(self.h, ctypes.byref(o), cb, None, ctypes.byref(st))
        out = {k: getattr(st, k) for k, _ in XfRunStats._fields_}
        out["status"] = rc
        if rc not in (XF_OK, XF_ENAN):
            self._c(rc, "xf_run")
        if log is not None:
            out["log"] = log[:3 * st.log_len].reshape(-1, 3)
        return out

    def phase_times(self):
        ms = np.zeros(3)
        n = (ctypes.c_long * 3)()
        self._c(self.lib.xf_phase_times(self.h, _dp(ms), n), "xf_phase_times")
        return ms, list(n)

    def survival(self):
        out = np.empty(self.abins * self.pbins * 4)
        self._c(self.lib.xf_survival(self.h, _dp(out)), "xf_survival")
        return out.reshape(-1, 4)


class Batch:
    """Many independent MA simulations advanced together (xf_batch_*)."""

    def __init__(self, cfgs):
        self.lib = _abi.load()
        self.cfgs = [c if isinstance(c, Config) else Config.from_file(c) for c in cfgs]
        arr = (XfConfig * len(self.cfgs))()
        for i, c in enumerate(self.cfgs):
            ctypes.memmove(ctypes.byref(arr[i]), ctypes.byref(c.raw), ctypes.sizeof(XfConfig))
        h = ctypes.c_void_p()
        rc = self.lib.xf_batch_create(arr, len(self.cfgs), ctypes.byref(h))
        _check(rc, "xf_batch_create", None, self.lib)
        self.h = h
        self.dims = []
        for i in range(len(self.cfgs)):
            nb, ne = ctypes.c_int(), ctypes.c_int()
            self.lib.xf_batch_dims(self.h, i, ctypes.byref(nb), ctypes.byref(ne))
            self.dims.append((nb.value, ne.value))

    def _c(self, rc, what):
        if rc != XF_OK:
            msg = self.lib.xf_strerror(rc).decode()
            d = self.lib.xf_batch_last_error(self.h)
            raise XflatError(rc, "%s failed: %s%s" % (what, msg, (": " + d.decode()) if d else ""))

    def close(self):
        if getattr(self, "h", None):
            self.lib.xf_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, i, psi):
        psi = np.ascontiguousarray(psi, dtype=np.float64).reshape(-1)
        self._c(self.lib.xf_batch_set_state(self.h, i, _dp(psi)), "xf_batch_set_state")

    def get_state(self, i):
        nb, ne = self.dims[i]
        out = np.empty(nb * 4 * ne)
        self._c(self.lib.xf_batch_get_state(self.h, i, _dp(out)), "xf_batch_get_state")
        return out.reshape(nb, 4, ne)

    def tile_shape(self):
        w = ctypes.c_int()
        ms = np.zeros(3)
        self._c(self.lib.xf_batch_tile_shape(self.h, ctypes.byref(w), _dp(ms)), "xf_batch_tile_shape")
        return w.value, ms

    def tuning(self):
        """The autotuner's choice and table: {'warps', 'beams_per_warp',
        'persistent', 'candidates': [(warps, beams_per_warp, persistent, ms), ...]}."""
        w, bpw, pers, nc = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        cw, cb, cp = (ctypes.c_int * 16)(), (ctypes.c_int * 16)(), (ctypes.c_int * 16)()
        ms = np.zeros(16)
        self._c(self.lib.xf_batch_tuning(self.h, ctypes.byref(w), ctypes.byref(bpw), ctypes.byref(pers),
                                         ctypes.byref(nc), cw, cb, cp, _dp(ms)), "xf_batch_tuning")
        return dict(warps=w.value, beams_per_warp=bpw.value, persistent=pers.value,
                    candidates=[(cw[i], cb[i], cp[i], float(ms[i])) for i in range(nc.value)])

    def run(self, max_iters=-1):
        n = len(self.cfgs)
        it = (ctypes.c_long * n)()
        acc = (ctypes.c_long * n)()
        rend = np.zeros(n)
        secs = ctypes.c_double()
        self._c(self.lib.xf_batch_run(self.h, int(max_iters), it, acc, _dp(rend), ctypes.byref(secs)), "xf_batch_run")
        return dict(iterations=list(it), accepted=list(acc), r_end=rend, seconds=secs.value)
