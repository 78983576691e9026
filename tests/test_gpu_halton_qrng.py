"""The generalized Halton sequence of halton_qrng (qmctoolscl/c_funcs/halton_qrng.c:3-162)
on the GPU, bit for bit: the golden vectors of the reference's own compiled C
and seeded cases against the oracle, through the drop-in binding
qmctoolscl_gb300.c_funcs.halton_qrng_c (numpy arrays and CUDA tensors)."""
import numpy as np
import pytest

import oracle
from qmctoolscl_gb300.c_funcs import halton_qrng_c

from .test_oracle_halton_qrng import _cases

pytestmark = pytest.mark.gpu


def _same(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


@pytest.mark.parametrize("case", list(_cases()), ids=lambda cs: "case%d" % cs[0])
def test_golden(case):
    _c, (n, d, n0, gen), dvec, randu, want = case
    res = np.full(d * n, np.nan)
    halton_qrng_c(n, d, n0, gen, res, np.ascontiguousarray(randu), np.ascontiguousarray(dvec, dtype=np.int32))
    assert _same(res, want)


@pytest.mark.parametrize("n,d,n0,gen", [(1, 1, 0, 1), (1000, 360, 0, 1), (4096, 17, 1, 0), (300, 9, -77, 1),
                                        (2 ** 18, 4, 0, 1), (999, 5, 2 ** 31 - 1000, 1), (50, 3, 2 ** 30, 0)])
def test_against_oracle(n, d, n0, gen):
    rng = np.random.Generator(np.random.SFC64(n + d))
    dvec = (np.arange(d) if d == 360 else rng.integers(0, 360, d)).astype(np.int32)
    randu = rng.random(d * 32)
    want, res = np.full(d * n, np.nan), np.full(d * n, np.nan)
    oracle.halton_qrng(n, d, n0, gen, want, randu, dvec)
    halton_qrng_c(n, d, n0, gen, res, randu, dvec)
    assert _same(res, want)


def test_tensors_in_place_and_bad_dimension_index():
    import torch
    rng = np.random.Generator(np.random.SFC64(11))
    n, d = 777, 6
    dvec = rng.integers(0, 360, d).astype(np.int32)
    randu = rng.random(d * 32)
    want = np.full(d * n, np.nan)
    oracle.halton_qrng(n, d, 5, 1, want, randu, dvec)
    res_t = torch.full((d * n,), float("nan"), dtype=torch.float64, device="cuda")
    halton_qrng_c(n, d, 5, 1, res_t, torch.from_numpy(randu).cuda(), torch.from_numpy(dvec).cuda())
    assert _same(res_t.cpu().numpy(), want)
    bad = dvec.copy()
    bad[2] = 360  # outside the reference's tables: reported, never read
    with pytest.raises(Exception, match="device error"):
        halton_qrng_c(n, d, 5, 1, np.full(d * n, np.nan), randu, bad)
    import qmctoolscl_gb300._ffi as ffi
    ffi.check(ffi.lib().qmc_device_error_reset(torch.cuda.current_stream().cuda_stream), "reset")
