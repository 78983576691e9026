"""Integer replacements for FP64 operations used by the kernels, compiled for
the host with g++ and checked against the host's IEEE arithmetic:

* digit_sum.cuh -- the running sum of gdn_integer_to_float (fused
  generalized-net kernel): single adds over random operands and whole chains
  (recip_0 = 1/b, recip_{t+1} = recip_t/b, terms RN(recip_t * digit)) over
  random bases and digits;
* fpconv.cuh -- FP64 <-> FP32 conversions with round to nearest even
  (tensor-core transforms);
* qrng_step.cuh -- one Horner step of halton_qrng, RN(RN(v + c) / b), over
  random operands, ties and whole 32-step chains.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _compile(tmp_path_factory, src):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("hostmath") / os.path.splitext(src)[0])
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe, os.path.join(HERE, src)], check=True)
    return exe


@pytest.fixture(scope="module")
def digit_sum_checker(tmp_path_factory):
    return _compile(tmp_path_factory, "digit_sum_check.cpp")


@pytest.fixture(scope="module")
def fpconv_checker(tmp_path_factory):
    return _compile(tmp_path_factory, "fpconv_check.cpp")


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_digit_sum_matches_ieee(digit_sum_checker, seed):
    out = subprocess.run([digit_sum_checker, "3000000", "300000", str(seed)], capture_output=True, text=True,
                         timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok")


@pytest.mark.parametrize("seed", [1, 2])
def test_fp64_fp32_conversions_match_hardware(fpconv_checker, seed):
    out = subprocess.run([fpconv_checker, "5000000", str(seed)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok")


@pytest.fixture(scope="module")
def qrng_step_checker(tmp_path_factory):
    return _compile(tmp_path_factory, "qrng_step_check.cpp")


@pytest.mark.parametrize("seed", [1, 2])
def test_qrng_step_matches_ieee(qrng_step_checker, seed):
    out = subprocess.run([qrng_step_checker, "3000000", str(seed)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok")
