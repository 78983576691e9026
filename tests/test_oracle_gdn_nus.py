"""The oracle's nested uniform scramble of generalized (base-b) nets
(oracle.GdnNusForest) against the reference's own Python code: golden
vectors of tests/golden/make_gdn_nus.py (qmctoolscl/rand_funcs.py:255-356),
the documented example first, with several calls on the same root nodes and
the generator states after each call.  The GPU form of this routine is not
built; the oracle is ready for it."""
import os

import numpy as np
import pytest

import oracle

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "gdn_nus.npz"))
NCASES = len([k for k in GOLD.files if k.endswith("_args")])


@pytest.mark.parametrize("c", range(NCASES))
def test_oracle_matches_reference(c):
    r, n, d, r_x, r_b, tmax, tmax_new, calls = (int(v) for v in GOLD["case%d_args" % c])
    states = GOLD["case%d_state0" % c].reshape(-1).copy()
    bases = GOLD["case%d_bases" % c]
    forest = oracle.GdnNusForest(r * d)
    for k in range(calls):
        xr = np.zeros((r, n, d, tmax_new), dtype=np.uint64)
        rc = forest.scramble(r, n, d, r_x, r_b, tmax, tmax_new, states, bases, GOLD["case%d_xdig%d" % (c, k)], xr)
        assert rc == 0
        assert np.array_equal(xr, GOLD["case%d_xrdig%d" % (c, k)]), (c, k)
        assert np.array_equal(states, GOLD["case%d_state%d" % (c, k + 1)].reshape(-1)), (c, k)
    forest.close()


def test_documented_example_is_case_0():
    assert [int(v) for v in GOLD["case0_args"][:3]] == [2, 9, 3]
    assert GOLD["case0_xrdig0"][0, 0, 0].tolist() == [0, 0, 1, 0, 0, 1, 0, 0]  # docs/index.md, first row


def test_where_the_reference_raises():
    """a digit at or above its base, and tmax_new = tmax with a repeated point
    (the reference's walk indexes an empty digit array): reported, not run on"""
    st = np.zeros(6, np.uint64)
    st[:4] = [1, 2, 3, 4]
    f = oracle.GdnNusForest(1)
    xr = np.zeros((1, 1, 1, 3), np.uint64)
    assert f.scramble(1, 1, 1, 1, 1, 3, 3, st.copy(), np.array([[3]], np.uint64),
                      np.array([[[[0, 3, 1]]]], np.uint64), xr) == 1
    f.close()
    f = oracle.GdnNusForest(1)
    xr = np.zeros((1, 3, 1, 2), np.uint64)
    dig = np.array([[[[1, 0]], [[1, 1]], [[1, 0]]]], np.uint64)
    assert f.scramble(1, 3, 1, 1, 1, 2, 2, st.copy(), np.array([[2]], np.uint64), dig, xr) == 1
    f.close()
