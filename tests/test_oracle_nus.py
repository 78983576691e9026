"""The oracle's nested uniform scramble of base-2 nets against the
reference's own Python code (golden vectors of tests/golden/make_nus.py,
qmctoolscl/rand_funcs.py:155-253), including the reference's documented
example, continuation calls on the same root nodes and the generator states
after each call; and the SFC64 state helpers against numpy."""
import os

import numpy as np
import pytest

import oracle
from qmctoolscl_gb300.nus import set_sfc64_state, sfc64_state_words

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "nus.npz"))
NCASES = len([k for k in GOLD.files if k.endswith("_args")])


@pytest.mark.parametrize("c", range(NCASES))
def test_oracle_matches_reference(c):
    r, n, d, r_x, tmax, tmax_new, calls = (int(v) for v in GOLD["case%d_args" % c])
    states = GOLD["case%d_state0" % c].reshape(-1).copy()
    forest = oracle.NusForest(r * d)
    for k in range(calls):
        xrb = np.zeros((r, n, d), dtype=np.uint64)
        forest.scramble(r, n, d, r_x, tmax, tmax_new, states, GOLD["case%d_xb%d" % (c, k)], xrb)
        assert np.array_equal(xrb, GOLD["case%d_xrb%d" % (c, k)]), (c, k)
        assert np.array_equal(states, GOLD["case%d_state%d" % (c, k + 1)].reshape(-1)), (c, k)


def test_documented_example_is_case_0():
    r, n, d = (int(v) for v in GOLD["case0_args"][:3])
    assert (r, n, d) == (2, 8, 4)
    assert GOLD["case0_xrb0"][0, 0].tolist() == [94, 54, 235, 30]  # docs/index.md, first row


def test_state_words_round_trip():
    g = np.random.Generator(np.random.SFC64(3))
    g.integers(0, 2 ** 7)  # leaves a buffered 32-bit half
    w = sfc64_state_words(g)
    assert w[4] == 1
    h = np.random.Generator(np.random.SFC64(99))
    set_sfc64_state(h, w)
    assert [int(h.integers(0, 2 ** 40)) for _ in range(5)] == [int(g.integers(0, 2 ** 40)) for _ in range(5)]


def test_other_bit_generators_are_refused():
    with pytest.raises(TypeError):
        sfc64_state_words(np.random.Generator(np.random.PCG64(1)))
