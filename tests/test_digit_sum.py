"""The integer digit-to-float running sum used by the fused generalized-net
kernel (qmctoolscl_gb300/csrc/digit_sum.cuh), compiled for the host with g++
and checked against the host's IEEE double arithmetic: single steps
v + r*s over random operands, and whole gdn_integer_to_float chains
(recip_0 = 1/b, recip_{t+1} = recip_t/b) over random bases and digits."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("dsum") / "digit_sum_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe,
                    os.path.join(HERE, "digit_sum_check.cpp")], check=True)
    return exe


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_digit_sum_matches_ieee(checker, seed):
    out = subprocess.run([checker, "3000000", "300000", str(seed)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok")
