"""The module a maintainer adds to XFLAT (xflat_gb300/integration/Nmr_gpu.cpp,
as src/Nmr_gpu.cpp, in both of its evolutionLoop forms) compiles against
XFLAT's own headers and this repository's C ABI header, and links with
XFLAT's other modules and libxflat_gb300.so.  CPU only.  The reference
checkout is found through the XFLAT_REFERENCE environment variable, else a
`reference` directory beside the repository; the tests skip without one (the
GPU machines have none)."""
import os
import shutil
import subprocess

import pytest

from helpers import ROOT

REFERENCE = os.environ.get("XFLAT_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")
REF_INCLUDE = os.path.join(REFERENCE, "include")
MODULE = os.path.join(ROOT, "xflat_gb300", "integration", "Nmr_gpu.cpp")
VARIANTS = {"callback": [], "library_files": ["-DXFLAT_GPU_LIBRARY_FILES"]}

needs_reference = pytest.mark.skipif(not os.path.isdir(REF_INCLUDE) or shutil.which("g++") is None,
                                     reason="reference headers or g++ not available")


@needs_reference
@pytest.mark.parametrize("variant", sorted(VARIANTS))
@pytest.mark.parametrize("geom", ["MA", "MAA", "SA"])
def test_nmr_gpu_module_compiles(variant, geom):
    res = subprocess.run(["g++", "-std=c++11", "-fsyntax-only", "-D" + geom, "-I" + REF_INCLUDE,
                          "-I" + os.path.join(ROOT, "include")] + VARIANTS[variant] + [MODULE],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr


REF_OBJS = ["Fenergy", "Matt", "NBGroup", "NBeam", "Parser", "Util", "Phy_MA", "h_ref_io"]


@needs_reference
def test_xflat_links_with_the_library(tmp_path):
    """XFLAT's own modules (objects built from its sources by oracle/Makefile),
    its src/main.cpp, the Nmr_gpu module and libxflat_gb300.so link into one
    executable: every entry point the module calls resolves."""
    objdir = os.path.join(ROOT, "oracle", "_ref", "ma")
    lib = os.path.join(ROOT, "xflat_gb300", "_lib", "libxflat_gb300.so")
    if not all(os.path.exists(os.path.join(objdir, o + ".o")) for o in REF_OBJS) or not os.path.exists(lib):
        pytest.skip("oracle/_ref objects or the library not built")
    flags = ["-std=c++11", "-fopenmp", "-DMA", "-DOMP", "-w", "-I" + REF_INCLUDE, "-I" + os.path.join(ROOT, "include")]
    for name, path, extra in [("Nmr_gpu.o", MODULE, VARIANTS["library_files"]),
                              ("main.o", os.path.join(REFERENCE, "src", "main.cpp"), [])]:
        res = subprocess.run(["g++"] + flags + extra + ["-c", path, "-o", str(tmp_path / name)], capture_output=True,
                             text=True)
        assert res.returncode == 0, res.stderr
    objs = [os.path.join(objdir, o + ".o") for o in REF_OBJS] + [str(tmp_path / "Nmr_gpu.o"), str(tmp_path / "main.o")]
    res = subprocess.run(["g++", "-fopenmp"] + objs + ["-L" + os.path.dirname(lib), "-lxflat_gb300",
                          "-Wl,-rpath," + os.path.dirname(lib), "-o", str(tmp_path / "xflat_gpu_module")],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
