"""The C++ drop-in: include/ugsdr_cuda_policies.hpp compiled against the
reference's own headers (FastSearchEngineBase<ParametricCudaFseConfig<...>>
instantiates) and linked against libugsdr_cuda.so.  Needs the reference tree
(skipped where it is absent); the binary runs only under -m gpu."""
import os
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT

REF = Path(os.environ.get("UGSDR_REF_DIR", str(ROOT.parent / "reference")))
BIN = ROOT / "tests" / "native" / "_bin" / "fse_dropin"


def build():
    if not (REF / "src" / "acquisition" / "fse.hpp").exists():
        pytest.skip("reference sources not present")
    BIN.parent.mkdir(exist_ok=True)
    lib = ROOT / "ugsdr_gb300" / "_lib"
    cmd = ["g++", "-std=gnu++20", "-O1", "-include", "algorithm", "-DIppDft=SequentialDft",
           f"-DUGSDR_REF_SRC={REF / 'src'}", "-I", str(ROOT / "include"), "-I", str(ROOT / "oracle" / "shims"),
           "-I", str(ROOT / "oracle" / "shims" / "anchor" / "dir"), str(ROOT / "tests" / "native" / "fse_dropin.cpp"),
           str(REF / "src" / "prn_codes" / "GalileoMemoryCodes.cpp"), str(ROOT / "oracle" / "fftw_shim.cpp"),
           "-I", str(ROOT / "oracle"), "-L", str(lib), "-lugsdr_cuda",
           f"-Wl,-rpath,{lib}", "-o", str(BIN)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_dropin_compiles_and_links(lib):
    build()
    assert BIN.exists()


@pytest.mark.gpu
def test_dropin_runs(lib):
    build()
    r = subprocess.run([str(BIN)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
