"""Fused pipelines (qmctoolscl_gb300.batch) equal the chain of reference
calls they replace, bit for bit, including when the output is written
straight into pinned host memory."""
import numpy as np
import pytest

import oracle
import qmctoolscl_gb300 as q
from qmctoolscl_gb300 import batch

pytestmark = pytest.mark.gpu
U = np.uint64


def oracle_lattice(r, n, d, n_start, g, shifts, order):
    x = np.empty((r, n, d))
    oracle.call("lat_gen_gray" if order == "gray" else "lat_gen_natural", U(r), U(n), U(d), U(n_start), g, x)
    xr = np.empty((r, n, d))
    oracle.call("lat_shift_mod_1", U(r), U(n), U(d), U(r), x, shifts, xr)
    return xr


@pytest.mark.parametrize("order,n_start,n,d", [("gray", 0, 4096, 64), ("gray", 37, 1000, 5), ("natural", 0, 2048, 6),
                                               ("natural", 1024, 1024, 3), ("gray", 0, 512, 100)])
@pytest.mark.parametrize("pinned", [False, True])
def test_lattice_gen_shift_matches_chain(order, n_start, n, d, pinned):
    rng = np.random.Generator(np.random.SFC64(n + d))
    r = 3
    g = (rng.integers(0, 1 << 19, (r, d)) * 2 + 1).astype(U)
    g[0, 0] = U((1 << 45) + 1)  # a column on the FP64 path
    shifts = q.lat_get_shifts(rng, r, d)
    shifts[1, 0] = 0.3 + 2.0 ** -60  # a shift off the 2^-53 grid
    xr = batch.pinned_empty((r, n, d)) if pinned else np.empty((r, n, d))
    A = batch.lattice_gen_shift(r, n, d, n_start, g, shifts, xr, order=order)
    assert A.direct == pinned
    want = oracle_lattice(r, n, d, n_start, g, shifts, order)
    assert np.array_equal(xr.view(U), want.view(U))


@pytest.mark.parametrize("order", ["natural", "gray"])
@pytest.mark.parametrize("stages", ["gen", "shift", "float", "shift+float", "float_only"])
def test_dnb2_gen_fused_matches_chain(order, stages):
    rng = np.random.Generator(np.random.SFC64(len(stages)))
    r, r_C, n, d, mmax, n_start = 4, 2, 1 << 12, 16, 14, 0
    C = q.random_tbit_uint64s(rng, 63, (r_C, d, mmax))
    lsh = np.array([0, 1, 3, 0], U)
    sb = q.dnb2_get_digital_shifts(rng, r, d, 64)
    tm = np.array([63, 64, 70, 1], U)
    # the reference chain: generation per matrix set, shift with r_x = r_C, float
    xb = np.empty((r_C, n, d), U)
    oracle.call("dnb2_gen_gray" if order == "gray" else "dnb2_gen_natural", U(r_C), U(n), U(d), U(n_start),
                U(mmax), C, xb)
    want_int = xb
    if "shift" in stages:
        want_int = np.empty((r, n, d), U)
        oracle.call("dnb2_digital_shift", U(r), U(n), U(d), U(r_C), lsh[:r_C], xb, sb, want_int)
    else:
        want_int = np.stack([xb[l % r_C] for l in range(r)])
    want_f = np.empty((r, n, d))
    oracle.call("dnb2_integer_to_float", U(r), U(n), U(d), tm, want_int, want_f)
    xrb = np.empty((r, n, d), U) if stages != "float_only" else None
    x = np.empty((r, n, d)) if "float" in stages else None
    kw = {}
    if "shift" in stages:
        kw = dict(lshifts=lsh[:r_C], r_x=r_C, shiftsb=sb)
    batch.dnb2_gen_fused(r, n, d, n_start, mmax, C, r_C=r_C, order=order, tmaxes=tm if x is not None else None,
                         xrb=xrb, x=x, **kw)
    if xrb is not None:
        assert np.array_equal(xrb, want_int)
    if x is not None:
        assert np.array_equal(x.view(U), want_f.view(U))
