"""Register DFTs of the FFT kernels on the CPU (ugsdr_gb300/csrc/fft_core.cuh
is __host__ __device__): the pruned DFTs that pass 0 of the inverse row
stage runs when the upper half of its input is zero (one-sided code
spectra) equal the full DFTs on the zero-filled input for every radix of
the plans and every count of live inputs (tests/native/dft_pruned_check.cpp)."""
import subprocess
from pathlib import Path

from conftest import ROOT
from ugsdr_gb300 import build as B


def test_pruned_dfts_equal_full_dfts(tmp_path):
    cuda_include = Path(B.nvcc()).resolve().parent.parent / "include"
    exe = tmp_path / "dft_pruned_check"
    cmd = ["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-D__host__=", "-D__device__=", "-D__forceinline__=inline",
           "-I", str(cuda_include), "-I", str(ROOT / "ugsdr_gb300" / "csrc"),
           str(ROOT / "tests" / "native" / "dft_pruned_check.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout[-3000:]
