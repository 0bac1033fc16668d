"""The module INTEGRATION.md shows a maintainer adding to XFLAT (src/Nmr_gpu.cpp,
in both its variants) compiles against XFLAT's own headers and this
repository's C ABI header.  CPU only; skipped where the reference sources are
not checked out (the GPU machines have none)."""
import os
import re
import shutil
import subprocess

import pytest

from helpers import ROOT

REFERENCE = os.environ.get("XFLAT_REFERENCE", "/root/reference")
REF_INCLUDE = os.path.join(REFERENCE, "include")


def _blocks():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    return re.findall(r"```cpp\n(.*?)```", text, re.S)


@pytest.mark.skipif(not os.path.isdir(REF_INCLUDE) or shutil.which("g++") is None,
                    reason="reference headers or g++ not available")
@pytest.mark.parametrize("variant", ["callback", "library_files"])
@pytest.mark.parametrize("geom", ["MA", "MAA", "SA"])
def test_nmr_gpu_module_compiles(tmp_path, variant, geom):
    blocks = _blocks()
    assert len(blocks) == 2
    src = blocks[0]
    if variant == "library_files":
        i = src.index("int evolutionLoop() throw()")
        j = src.index("void freemem()")
        src = src[:i] + blocks[1] + "\n" + src[j:]
    path = tmp_path / "Nmr_gpu.cpp"
    path.write_text(src)
    res = subprocess.run(["g++", "-std=c++11", "-fsyntax-only", "-D" + geom, "-I" + REF_INCLUDE,
                          "-I" + os.path.join(ROOT, "include"), str(path)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr


REF_OBJS = ["Fenergy", "Matt", "NBGroup", "NBeam", "Parser", "Util", "Phy_MA", "h_ref_io"]


@pytest.mark.skipif(not os.path.isdir(REF_INCLUDE) or shutil.which("g++") is None,
                    reason="reference sources or g++ not available")
def test_xflat_links_with_the_library(tmp_path):
    """XFLAT's own modules (objects built from its sources by oracle/Makefile),
    its src/main.cpp, the Nmr_gpu module and libxflat_gb300.so link into one
    executable: every entry point the module calls resolves."""
    objdir = os.path.join(ROOT, "oracle", "_ref", "ma")
    lib = os.path.join(ROOT, "xflat_gb300", "_lib", "libxflat_gb300.so")
    if not all(os.path.exists(os.path.join(objdir, o + ".o")) for o in REF_OBJS) or not os.path.exists(lib):
        pytest.skip("oracle/_ref objects or the library not built")
    blocks = _blocks()
    src = blocks[0]
    i, j = src.index("int evolutionLoop() throw()"), src.index("void freemem()")
    (tmp_path / "Nmr_gpu.cpp").write_text(src[:i] + blocks[1] + "\n" + src[j:])
    flags = ["-std=c++11", "-fopenmp", "-DMA", "-DOMP", "-w", "-I" + REF_INCLUDE, "-I" + os.path.join(ROOT, "include")]
    for name, path in [("Nmr_gpu.o", str(tmp_path / "Nmr_gpu.cpp")), ("main.o", os.path.join(REFERENCE, "src", "main.cpp"))]:
        res = subprocess.run(["g++"] + flags + ["-c", path, "-o", str(tmp_path / name)], capture_output=True, text=True)
        assert res.returncode == 0, res.stderr
    objs = [os.path.join(objdir, o + ".o") for o in REF_OBJS] + [str(tmp_path / "Nmr_gpu.o"), str(tmp_path / "main.o")]
    res = subprocess.run(["g++", "-fopenmp"] + objs + ["-L" + os.path.dirname(lib), "-lxflat_gb300",
                          "-Wl,-rpath," + os.path.dirname(lib), "-o", str(tmp_path / "xflat_gpu_module")],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
