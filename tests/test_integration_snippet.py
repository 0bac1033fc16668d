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
