"""The oracle's halton_qrng (qmctoolscl/c_funcs/halton_qrng.c:3-162) pinned
bit for bit: against the golden vectors made by the reference's own
compiled C (tests/golden/make_halton_qrng.py) and, where the reference is
built here (oracle/_ref), against it on seeded random cases."""
import os

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))


def _cases():
    z = np.load(os.path.join(HERE, "golden", "halton_qrng.npz"))
    c = 0
    while "case%d_args" % c in z:
        yield c, [int(v) for v in z["case%d_args" % c]], z["case%d_dvec" % c], z["case%d_randu" % c], \
            z["case%d_res" % c]
        c += 1


@pytest.mark.parametrize("case", list(_cases()), ids=lambda cs: "case%d" % cs[0])
def test_oracle_matches_golden(case):
    _c, (n, d, n0, gen), dvec, randu, want = case
    res = np.full(d * n, np.nan)
    oracle.halton_qrng(n, d, n0, gen, res, np.ascontiguousarray(randu), np.ascontiguousarray(dvec, dtype=np.int32))
    assert np.array_equal(res.view(np.uint64), want.view(np.uint64))


@pytest.mark.skipif(not oracle.ref_available(), reason="reference C backend not built here")
@pytest.mark.parametrize("seed", range(6))
def test_oracle_matches_compiled_reference(seed):
    rng = np.random.Generator(np.random.SFC64(seed))
    n, d = int(rng.integers(1, 300)), int(rng.integers(1, 40))
    n0 = int(rng.choice([0, 1, int(rng.integers(2, 10 ** 6)), -int(rng.integers(1, 500))]))
    gen = int(seed % 2)
    dvec = rng.integers(0, 360, d).astype(np.int32)
    randu = rng.random(d * 32)
    a, b = np.full(d * n, np.nan), np.full(d * n, np.nan)
    oracle.halton_qrng(n, d, n0, gen, a, randu, dvec)
    oracle.halton_qrng_ref(n, d, n0, gen, b, randu, dvec)
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_binding_checks_arguments_like_ctypes():
    """halton_qrng_c checks its arrays as np.ctypeslib.ndpointer does, before any device use."""
    import ctypes
    from qmctoolscl_gb300.c_funcs import halton_qrng_c
    res, randu, dvec = np.empty(6), np.random.rand(64), np.arange(2, dtype=np.int32)
    with pytest.raises(ctypes.ArgumentError):
        halton_qrng_c(3, 2, 0, 1, res.astype(np.float32), randu, dvec)
    with pytest.raises(ctypes.ArgumentError):
        halton_qrng_c(3, 2, 0, 1, res, randu, dvec.astype(np.int64))
    with pytest.raises(ctypes.ArgumentError):
        halton_qrng_c(3, 2, 0, 1, np.empty((2, 6))[:, :3], randu, dvec)
    with pytest.raises(ctypes.ArgumentError):
        halton_qrng_c(3.0, 2, 0, 1, res, randu, dvec)
    assert halton_qrng_c(0, 2, 0, 1, res, randu, dvec) is None  # nothing to do: the reference's loops do not run
