"""The back-projection quotient computed in 64-bit integers
(csrc/uds_backproject.cuh) against the double formula of transformation.cuh
it replaces, bit for bit, on random and edge-case inputs (host build of the
same header the kernels use); and the rule that one double operation on
float operands, rounded to float, equals the float operation."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "unbiased_differentiable_splatting_gb300", "csrc")


def test_backproject_quotient_matches_double(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "backproject_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC,
                    os.path.join(HERE, "backproject_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe, "2000000"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    cases, fast, ops, bad = (int(v) for v in out.stdout.split()[-4:])
    assert bad == 0
    assert cases > 4_000_000 and ops > 4_000_000
    assert fast > 0.8 * cases  # the double fallback stays rare


def test_blend_remainder_matches_double(tmp_path):
    """The blend's remaining transmittance computed on the exact integer
    product (csrc/uds_blendrem.cuh) against (float)((double)rem * (1.0 -
    (double)w)), bit for bit, on random and edge-case inputs."""
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "blendrem_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC,
                    os.path.join(HERE, "blendrem_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe, "2000000"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    cases, fast, bad = (int(v) for v in out.stdout.split()[-3:])
    assert bad == 0
    assert cases > 8_000_000
    assert fast > 0.9 * cases  # the double fallback stays rare
