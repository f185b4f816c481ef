"""The double-float arithmetic of the FP32x2 form (csrc/scft_dfloat.cuh),
compiled for the host and checked against long double: sums, products, the
two-product difference of the complex twiddle product, division and the
compensated 48-term dot of the dense z pass, each within a double-word error
bound (a few 2^-48 of the operands' magnitudes), and every result a
normalised pair. The device build uses the same code with the _rn intrinsics,
which round like the host's IEEE single-precision operations."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "stimuli-responsive-nanodroplets_gb300" / "csrc"


def _cuda_include():
    for base in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if base and (Path(base) / "include" / "cuda_runtime.h").exists():
            return Path(base) / "include"
    return None


def test_double_float_arithmetic_bounds(tmp_path):
    gxx = shutil.which("g++")
    inc = _cuda_include()
    if gxx is None or inc is None:
        pytest.skip("needs g++ and the CUDA runtime headers")
    exe = tmp_path / "dfloat_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", f"-I{inc}", f"-I{CSRC}",
                    str(ROOT / "tests" / "dfloat_check.cpp"), "-o", str(exe), "-lm"], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
