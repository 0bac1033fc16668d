"""Oracle (test infrastructure only; never imported by the product).

ctypes wrapper of the C restatement of the reference's hot path
(oracle/xf_port.c, built into oracle/_build/libxfport.so by oracle/Makefile).
Used by the tests as the checker, by smoke() and by bench.py's CPU-baseline
leg."""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libxfport.so")
EXE = os.path.join(HERE, "_build", "xfport")
P = ctypes.POINTER(ctypes.c_double)
_lib = None


def build():
    subprocess.run(["make", "-C", HERE, "port", "-j4"], check=True, capture_output=True)


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        build()
    lib = ctypes.CDLL(LIB)
    V = ctypes.c_void_p
    sig = {
        "xfp_create": (V, [ctypes.c_char_p]),
        "xfp_destroy": (None, [V]),
        "xfp_geometry": (ctypes.c_int, [V]),
        "xfp_nbeams": (ctypes.c_int, [V]),
        "xfp_ebins": (ctypes.c_int, [V]),
        "xfp_abins": (ctypes.c_int, [V]),
        "xfp_pbins": (ctypes.c_int, [V]),
        "xfp_params": (None, [V, P]),
        "xfp_tables": (None, [V, P, P, P, P]),
        "xfp_hm": (ctypes.c_double, [V, ctypes.c_double]),
        "xfp_set_state": (None, [V, P]),
        "xfp_get_state": (None, [V, ctypes.c_int, P]),
        "xfp_get_esum": (None, [V, ctypes.c_int, P]),
        "xfp_noise": (None, [V, ctypes.c_uint64, ctypes.c_double]),
        "xfp_probe": (None, [V, ctypes.c_double, ctypes.c_double, P, P, P, P]),
        "xfp_calc_hvv": (None, [V, ctypes.c_int, ctypes.c_int, P]),
        "xfp_iterate": (ctypes.c_double, [V, ctypes.c_double, ctypes.c_double]),
        "xfp_accept": (None, [V]),
        "xfp_run": (ctypes.c_long, [V, ctypes.c_double, ctypes.c_double, ctypes.c_long, P, ctypes.c_long,
                                    ctypes.POINTER(ctypes.c_long), P, P]),
        "xfp_replay": (None, [V, P, P, ctypes.c_long]),
    }
    for k, (r, a) in sig.items():
        f = getattr(lib, k)
        f.restype = r
        f.argtypes = a
    _lib = lib
    return lib


def _p(a):
    return a.ctypes.data_as(P)


class Port:
    """One simulation of the C restatement (config file path)."""

    def __init__(self, config_path):
        self.lib = load()
        self.s = self.lib.xfp_create(config_path.encode())
        if not self.s:
            raise RuntimeError("oracle port cannot load %s" % config_path)
        self.nbeams = self.lib.xfp_nbeams(self.s)
        self.ebins = self.lib.xfp_ebins(self.s)
        self.abins = self.lib.xfp_abins(self.s)
        self.pbins = self.lib.xfp_pbins(self.s)
        self.geometry = self.lib.xfp_geometry(self.s)
        prm = np.zeros(10)
        self.lib.xfp_params(self.s, _p(prm))
        self.R0, self.Rn, self.dr0, self.eps0, self.ksi, self.max_dr = prm[:6]
        self.Ts, self.Tn, self.seed, self.noise_amp = int(prm[6]), int(prm[7]), int(prm[8]), prm[9]

    def __del__(self):
        try:
            if self.s:
                self.lib.xfp_destroy(self.s)
                self.s = None
        except Exception:
            pass

    @property
    def shape(self):
        return (self.nbeams, 4, self.ebins)

    def noise(self, seed, amp):
        self.lib.xfp_noise(self.s, int(seed), float(amp))

    def set_state(self, psi):
        psi = np.ascontiguousarray(psi, dtype=np.float64)
        self.lib.xfp_set_state(self.s, _p(psi))

    def get_state(self, which=0):
        out = np.empty(self.nbeams * 4 * self.ebins)
        self.lib.xfp_get_state(self.s, int(which), _p(out))
        return out.reshape(self.shape)

    def get_esum(self, which=0):
        out = np.empty(self.nbeams * 4)
        self.lib.xfp_get_esum(self.s, int(which), _p(out))
        return out.reshape(self.nbeams, 4)

    def tables(self):
        fv, hv, le, ev = np.empty(4 * self.ebins), np.empty(2 * self.ebins), np.empty(4), np.empty(4)
        self.lib.xfp_tables(self.s, _p(fv), _p(hv), _p(le), _p(ev))
        return dict(fv=fv.reshape(4, -1), hvac=hv, LE=le, Ev=ev)

    def hm(self, r):
        return self.lib.xfp_hm(self.s, float(r))

    def probe(self, r, dr):
        n = 3 * self.abins
        c, s, d, l = (np.empty(n) for _ in range(4))
        self.lib.xfp_probe(self.s, float(r), float(dr), _p(c), _p(s), _p(d), _p(l))
        return c.reshape(3, -1), s.reshape(3, -1), d.reshape(3, -1), l.reshape(3, -1)

    def calc_hvv(self, which, pt):
        out = np.empty(4 * self.abins * self.pbins)
        self.lib.xfp_calc_hvv(self.s, int(which), int(pt), _p(out))
        return out.reshape(-1, 4)

    def iterate(self, r, dr):
        return self.lib.xfp_iterate(self.s, float(r), float(dr))

    def accept(self):
        self.lib.xfp_accept(self.s)

    def run(self, r0=None, dr0=None, max_iters=-1, log_cap=0):
        log = np.zeros(3 * max(1, log_cap))
        n_acc = ctypes.c_long()
        r_end, dr_end = ctypes.c_double(), ctypes.c_double()
        it = self.lib.xfp_run(self.s, float(self.R0 if r0 is None else r0), float(self.dr0 if dr0 is None else dr0),
                              int(max_iters), _p(log), int(log_cap), ctypes.byref(n_acc), ctypes.byref(r_end),
                              ctypes.byref(dr_end))
        return dict(iterations=it, accepted=n_acc.value, r_end=r_end.value, dr_end=dr_end.value,
                    log=log[:3 * min(n_acc.value, log_cap)].reshape(-1, 3))

    def replay(self, r_before, dr):
        rb = np.ascontiguousarray(r_before, dtype=np.float64)
        d = np.ascontiguousarray(dr, dtype=np.float64)
        self.lib.xfp_replay(self.s, _p(rb), _p(d), len(rb))
