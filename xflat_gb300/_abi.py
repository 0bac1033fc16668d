"""ctypes mirror of include/xflat_gpu.h.

Loads the in-tree native library built by ``xflat_gb300.build``.  There is no
fallback: if the library or a GPU is missing, calls fail loudly."""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libxflat_gb300.so")

XF_OK, XF_EINVAL, XF_ECUDA, XF_ETIMEOUT, XF_ENAN, XF_EIO, XF_ENOMEM, XF_EUNSUPPORTED = range(8)
XF_GEOM_MA, XF_GEOM_MAA, XF_GEOM_SA = 0, 1, 2
XF_PREC_FP64, XF_PREC_MIXED, XF_PREC_DF = 0, 1, 2

c_double_p = ctypes.POINTER(ctypes.c_double)
c_long_p = ctypes.POINTER(ctypes.c_long)
c_int_p = ctypes.POINTER(ctypes.c_int)


class XfConfig(ctypes.Structure):
    _fields_ = [
        ("geometry", ctypes.c_int), ("precision", ctypes.c_int),
        ("abins", ctypes.c_int), ("pbins", ctypes.c_int), ("ebins", ctypes.c_int), ("flvs", ctypes.c_int),
        ("has_matter", ctypes.c_int), ("dump_mode", ctypes.c_int), ("Ts", ctypes.c_int), ("Tn", ctypes.c_int),
        ("new_file_step", ctypes.c_int), ("sync_step", ctypes.c_int),
        ("tstep1", ctypes.c_int), ("itrstep1", ctypes.c_int), ("tstep2", ctypes.c_int), ("itrstep2", ctypes.c_int),
        ("start_beam", ctypes.c_int), ("end_beam", ctypes.c_int),
        ("rstep1", ctypes.c_double), ("rstep2", ctypes.c_double),
        ("eps0", ctypes.c_double), ("ksi", ctypes.c_double), ("mu", ctypes.c_double),
        ("R0", ctypes.c_double), ("Rn", ctypes.c_double), ("dr", ctypes.c_double), ("max_dr", ctypes.c_double),
        ("E0", ctypes.c_double), ("E1", ctypes.c_double),
        ("Ye", ctypes.c_double), ("Rv", ctypes.c_double), ("Mns", ctypes.c_double), ("gs", ctypes.c_double),
        ("S", ctypes.c_double), ("hNS", ctypes.c_double), ("nb0", ctypes.c_double),
        ("theta", ctypes.c_double), ("theta2", ctypes.c_double), ("dm2", ctypes.c_double),
        ("Lv", ctypes.c_double * 4), ("Tv", ctypes.c_double * 4), ("eta", ctypes.c_double * 4),
        ("seed", ctypes.c_uint64), ("noise_amp", ctypes.c_double),
        ("file_prefix", ctypes.c_char * 256),
    ]


class XfRunOpts(ctypes.Structure):
    _fields_ = [
        ("max_iters", ctypes.c_long), ("device_control", ctypes.c_int), ("iters_per_launch", ctypes.c_int),
        ("write_files", ctypes.c_int), ("time_phases", ctypes.c_int),
        ("r0", ctypes.c_double), ("dr0", ctypes.c_double),
        ("log", c_double_p), ("log_cap", ctypes.c_long),
    ]


class XfRunStats(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_long), ("accepted", ctypes.c_long),
        ("r_end", ctypes.c_double), ("dr_end", ctypes.c_double),
        ("seconds", ctypes.c_double), ("last_max_err", ctypes.c_double), ("device_ms", ctypes.c_double),
        ("kernel_launches", ctypes.c_long), ("log_len", ctypes.c_long),
        ("h2d_bytes", ctypes.c_long), ("d2h_bytes", ctypes.c_long),
    ]


XF_STEP_CB = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_long, ctypes.c_double, ctypes.c_double)

# name -> (restype, argtypes)
PROTOTYPES = {
    "xf_config_default": (ctypes.c_int, [ctypes.POINTER(XfConfig)]),
    "xf_config_load": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(XfConfig)]),
    "xf_config_parse": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(XfConfig)]),
    "xf_strerror": (ctypes.c_char_p, [ctypes.c_int]),
    "xf_host_tables": (ctypes.c_int, [ctypes.POINTER(XfConfig), c_double_p, c_double_p, c_double_p, c_double_p]),
    "xf_host_matter": (ctypes.c_int, [ctypes.POINTER(XfConfig), ctypes.c_double, c_double_p]),
    "xf_host_initial_state": (ctypes.c_int, [ctypes.POINTER(XfConfig), ctypes.c_uint64, ctypes.c_double, c_double_p]),
    "xf_set_option": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_double]),
    "xf_create": (ctypes.c_int, [ctypes.POINTER(XfConfig), ctypes.POINTER(ctypes.c_void_p)]),
    "xf_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "xf_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "xf_dims": (ctypes.c_int, [ctypes.c_void_p, c_int_p, c_int_p, c_int_p, c_int_p]),
    "xf_set_state": (ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    "xf_get_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_double_p]),
    "xf_set_noise": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double]),
    "xf_tables": (ctypes.c_int, [ctypes.c_void_p, c_double_p, c_double_p, c_double_p, c_double_p]),
    "xf_matter": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, c_double_p]),
    "xf_angle_bins": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, c_double_p, c_double_p,
                                     c_double_p, c_double_p]),
    "xf_calc_hvv": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                   c_double_p]),
    "xf_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, c_double_p]),
    "xf_accept": (ctypes.c_int, [ctypes.c_void_p]),
    "xf_run_opts_default": (ctypes.c_int, [ctypes.POINTER(XfRunOpts)]),
    "xf_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(XfRunOpts), XF_STEP_CB, ctypes.c_void_p,
                              ctypes.POINTER(XfRunStats)]),
    "xf_replay": (ctypes.c_int, [ctypes.c_void_p, c_double_p, c_double_p, ctypes.c_long]),
    "xf_phase_times": (ctypes.c_int, [ctypes.c_void_p, c_double_p, c_long_p]),
    "xf_survival": (ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    "xf_probe_fp64_peak": (ctypes.c_int, [ctypes.c_double, c_double_p]),
    "xf_probe_df_propagator": (ctypes.c_int, [ctypes.c_int, c_double_p, c_double_p, ctypes.c_int, c_double_p,
                                              c_double_p]),
    "xf_calc_hvv_static": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, c_double_p,
                                          ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]),
    "xf_dump": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_long, ctypes.c_double, ctypes.c_double]),
    "xf_resume": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, c_double_p, c_double_p]),
    "xf_io_close": (ctypes.c_int, [ctypes.c_void_p]),
    "xf_io_verbose": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "xf_snapshot_write": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(XfConfig), ctypes.c_long, c_double_p,
                                         c_double_p, c_double_p]),
    "xf_snapshot_read": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_long, c_double_p, c_double_p, c_double_p,
                                        c_long_p]),
    "xf_batch_create": (ctypes.c_int, [ctypes.POINTER(XfConfig), ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "xf_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "xf_batch_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "xf_batch_dims": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_int_p, c_int_p]),
    "xf_batch_set_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_double_p]),
    "xf_batch_get_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_double_p]),
    "xf_batch_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_long, c_long_p, c_long_p, c_double_p, c_double_p]),
    "xf_batch_tile_shape": (ctypes.c_int, [ctypes.c_void_p, c_int_p, c_double_p]),
    "xf_batch_tuning": (ctypes.c_int, [ctypes.c_void_p, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p,
                                       c_double_p]),
    "xf_batch_set_shape": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "xf_batch_set_persistent": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
}

_lib = None


def load():
    """Loads and returns the native library (cached)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("xflat_gb300 native library not built: %s (run xflat_gb300.build.build())" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def header_symbols(include_dir=None):
    """Function names declared in include/*.h (for the export check)."""
    import re
    include_dir = include_dir or os.path.join(os.path.dirname(HERE), "include")
    names = set()
    for f in os.listdir(include_dir):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(include_dir, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(xf_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)
