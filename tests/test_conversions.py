"""The chosen form's FP64 <-> FP32 conversions (csrc/mhd_conv.cuh, integer
instructions instead of GB300's narrow FP64-pipe conversions) against an
independent statement of their semantics, in both the branching and the
selecting form; host compile of the same header, no GPU needed."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "code_tohoku_gb300", "csrc")


@pytest.mark.parametrize("branch", [0, 1])
def test_conversions_match_reference_semantics(tmp_path, branch):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    exe = str(tmp_path / "conv_check")
    subprocess.run([gxx, "-O2", "-std=c++17", f"-DMHD_CONV_BRANCH={branch}", "-I", CSRC, "-I", cuda_inc,
                    os.path.join(HERE, "native", "conv_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert " 0 mismatches" in out.stdout
