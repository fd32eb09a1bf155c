"""The integer-pipe binary64 routines the FP32-state kernels use for the time
and step-size updates (diffrax_gb300/csrc/gbdx_f64i.cuh) return the IEEE-754
round-to-nearest-even result bit for bit: compiled for the host and compared
with the host's FP64 arithmetic on random, cancelling, tie-producing and
edge-of-range operands."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "diffrax_gb300", "csrc")


@pytest.mark.parametrize("seed", [1, 2])
def test_f64i_bit_exact(tmp_path, seed):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "f64i_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC,
                    os.path.join(HERE, "f64i_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe, "4000000", str(seed)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.count(" 0 mismatches") == 3, out.stdout
