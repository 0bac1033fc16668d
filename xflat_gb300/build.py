"""Builds the in-tree native library ``xflat_gb300/_lib/libxflat_gb300.so`` (and
the ``xflat_gpu`` command-line driver) with nvcc for sm_103a, compiling the
translation units in parallel.  No CMake, no torch extension machinery."""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "_lib")
INCLUDE = os.path.join(ROOT, "include")

CU_SOURCES = ["xf_kernels.cu", "xf_engine.cu", "xf_mixed.cu", "xf_df.cu", "xf_persist.cu", "xf_batch.cu", "xf_probe.cu",
              "xf_noalloc.cu"]
CXX_SOURCES = ["xf_config.cpp", "xf_physics.cpp", "xf_netcdf.cpp", "xf_io.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build xflat_gb300")
    return exe


def _newer(src_list, target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in src_list)


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))] + [
        os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]


def _compile(src):
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    if not _newer([path] + _headers(), obj):
        return obj
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC]
    if src.endswith(".cu"):
        cmd = [nvcc()] + ARCH + ["-lineinfo"] + common + ["-c", path, "-o", obj]
    else:
        cmd = [nvcc(), "-x", "c++"] + common + ["-c", path, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), res.stdout, res.stderr))
    return obj


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    sources = [s for s in CU_SOURCES + CXX_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, sources))
    so = os.path.join(LIB, "libxflat_gb300.so")
    if _newer(objs, so):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", so] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (res.stdout, res.stderr))
    main_src = os.path.join(CSRC, "xf_main.cpp")
    exe = os.path.join(LIB, "xflat_gpu")
    if os.path.exists(main_src) and _newer([main_src, so], exe):
        cmd = [nvcc(), "-x", "c++", "-O2", "-std=c++17", "-I" + INCLUDE, main_src, "-o", exe, "-L" + LIB,
               "-lxflat_gb300", "-Xlinker", "-rpath=$ORIGIN"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("driver link failed: %s\n%s" % (res.stdout, res.stderr))
    if verbose:
        print("built", so)
    return so


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
