"""The decomposition the GPU scrambles rest on, checked on the CPU: the model
of tests/nus_model.py (stable sort, Apetrei's bottom-up pass with its
threads interleaved at random, draws in point order, the walk up each point's
ancestors) against the oracle's restatement of the reference's tree walks and
against the reference's golden vectors (first calls, fresh trees)."""
import os

import numpy as np
import pytest

import oracle

from . import nus_model

HERE = os.path.dirname(__file__)
GOLD2 = np.load(os.path.join(HERE, "golden", "nus.npz"))
GOLDB = np.load(os.path.join(HERE, "golden", "gdn_nus.npz"))


def _states(rng, count):
    return np.stack([np.array([int(x) for x in rng.integers(0, 2 ** 63, 4)] + [int(rng.integers(0, 2)),
                                                                               int(rng.integers(0, 2 ** 32))],
                              dtype=np.uint64) for _ in range(count)])


@pytest.mark.parametrize("c", range(len([k for k in GOLD2.files if k.endswith("_args")])))
def test_base2_model_matches_golden(c):
    r, n, d, r_x, tmax, tmax_new, _calls = (int(v) for v in GOLD2["case%d_args" % c])
    states = [list(w) for w in GOLD2["case%d_state0" % c]]
    got = nus_model.dnb2_scramble(r, n, d, r_x, tmax, tmax_new, states, GOLD2["case%d_xb0" % c].tolist(), seed=c)
    assert np.array_equal(np.array(got, dtype=np.uint64).reshape(r, n, d), GOLD2["case%d_xrb0" % c])
    assert np.array_equal(np.array(states, dtype=np.uint64), GOLD2["case%d_state1" % c])


@pytest.mark.parametrize("seed", range(30))
def test_base2_model_matches_oracle(seed):
    rng = np.random.Generator(np.random.SFC64(900 + seed))
    r_x = int(rng.integers(1, 3))
    r, d, n = r_x * int(rng.integers(1, 3)), int(rng.integers(1, 3)), int(rng.integers(0, 50))
    tmax, tmax_new = int(rng.integers(0, 65)), int(rng.integers(0, 65))
    kind = seed % 3
    if kind == 0:
        xb = rng.integers(0, 2 ** 63, (r_x, n, d), dtype=np.uint64) * np.uint64(2)
    elif kind == 1:
        xb = rng.integers(0, 4, (r_x, n, d), dtype=np.uint64) << np.uint64(max(tmax - 2, 0))
    else:
        xb = rng.integers(0, 8, (r_x, n, d), dtype=np.uint64)
    st = _states(rng, r * d)
    words = st.reshape(-1).copy()
    want = np.zeros((r, n, d), dtype=np.uint64)
    f = oracle.NusForest(r * d)
    f.scramble(r, n, d, r_x, tmax, tmax_new, words, xb, want)
    f.close()
    states = [list(w) for w in st]
    got = nus_model.dnb2_scramble(r, n, d, r_x, tmax, tmax_new, states, xb.tolist(), seed=seed)
    assert np.array_equal(np.array(got, dtype=np.uint64).reshape(r, n, d), want)
    assert np.array_equal(np.array(states, dtype=np.uint64).reshape(-1), words)


@pytest.mark.parametrize("c", range(len([k for k in GOLDB.files if k.endswith("_args")])))
def test_baseb_model_matches_golden(c):
    r, n, d, r_x, r_b, tmax, tmax_new, _calls = (int(v) for v in GOLDB["case%d_args" % c])
    states = [list(w) for w in GOLDB["case%d_state0" % c]]
    got = nus_model.gdn_scramble(r, n, d, r_x, r_b, tmax, tmax_new, GOLDB["case%d_bases" % c].tolist(), states,
                                 GOLDB["case%d_xdig0" % c].tolist(), seed=c)
    assert np.array_equal(np.array(got, dtype=np.uint64).reshape(r, n, d, tmax_new), GOLDB["case%d_xrdig0" % c])
    assert np.array_equal(np.array(states, dtype=np.uint64), GOLDB["case%d_state1" % c])


@pytest.mark.parametrize("seed", range(20))
def test_baseb_model_matches_oracle(seed):
    rng = np.random.Generator(np.random.SFC64(950 + seed))
    r_x = int(rng.integers(1, 3))
    r, d, n = r_x * int(rng.integers(1, 3)), int(rng.integers(1, 3)), int(rng.integers(0, 30))
    r_b = 1 if r % 2 else int(rng.integers(1, 3))
    bases = rng.choice(np.array([2, 3, 5, 7, 11, 541], dtype=np.uint64), (r_b, d))
    w = max(max(1, int(b - 1).bit_length()) for b in bases.reshape(-1))
    tmax = int(rng.integers(1, min(10, 128 // w) + 1))
    tmax_new = tmax + int(rng.integers(1, 4))
    x = rng.integers(0, 1 << 30, (r_x, n, d, tmax), dtype=np.uint64)
    if seed % 3 == 1:
        x = x % np.uint64(2)
    x = np.ascontiguousarray(x % bases.min(axis=0)[None, None, :, None])
    st = _states(rng, r * d)
    words = st.reshape(-1).copy()
    want = np.zeros((r, n, d, tmax_new), dtype=np.uint64)
    f = oracle.GdnNusForest(r * d)
    assert f.scramble(r, n, d, r_x, r_b, tmax, tmax_new, words, bases, x, want) == 0
    f.close()
    states = [list(v) for v in st]
    got = nus_model.gdn_scramble(r, n, d, r_x, r_b, tmax, tmax_new, bases.tolist(), states, x.tolist(), seed=seed)
    assert np.array_equal(np.array(got, dtype=np.uint64).reshape(r, n, d, tmax_new), want)
    assert np.array_equal(np.array(states, dtype=np.uint64).reshape(-1), words)


def _net_bits(rng, n_log2, d, tmax):
    """natural-order points of random nonsingular upper-triangular matrices, MSB first in tmax bits"""
    n = 1 << n_log2
    xb = np.zeros((1, n, d), dtype=np.uint64)
    for j in range(d):
        M = np.triu(rng.integers(0, 2, (n_log2, n_log2)), 1) + np.eye(n_log2, dtype=np.int64)
        cols = [sum(int(M[t, k]) << (tmax - 1 - t) for t in range(n_log2)) for k in range(n_log2)]
        for i in range(n):
            v = 0
            for k in range(n_log2):
                if (i >> k) & 1:
                    v ^= cols[k]
            xb[0, i, j] = v
    return xb


def test_scramble_keeps_the_net_property():
    """Owen scrambling maps a (0, m, 1)-net to a (0, m, 1)-net: the top m bits of
    the 2^m scrambled points stay a permutation of 0 .. 2^m - 1 in every
    dimension (oracle and model alike)"""
    rng = np.random.Generator(np.random.SFC64(5))
    m, d, r, T = 7, 3, 2, 32
    xb = _net_bits(rng, m, d, T)
    st = _states(rng, r * d)
    words = st.reshape(-1).copy()
    got = np.zeros((r, 1 << m, d), dtype=np.uint64)
    f = oracle.NusForest(r * d)
    f.scramble(r, 1 << m, d, 1, T, T, words, xb, got)
    f.close()
    model = np.array(nus_model.dnb2_scramble(r, 1 << m, d, 1, T, T, [list(w) for w in st], xb.tolist()),
                     dtype=np.uint64)
    assert np.array_equal(model, got)
    for l in range(r):
        for j in range(d):
            top = np.sort(got[l, :, j] >> np.uint64(T - m))
            assert np.array_equal(top, np.arange(1 << m, dtype=np.uint64))
    assert not np.array_equal(got[0], xb[0])  # and it did scramble


def test_base_b_scramble_keeps_the_digit_net_property():
    """the same for base b: the first m digits of the b^m scrambled points take
    every value once"""
    rng = np.random.Generator(np.random.SFC64(6))
    b, m, tmax, tmax_new, r = 3, 4, 4, 6, 2
    n = b ** m
    bases = np.array([[b]], dtype=np.uint64)
    C = np.tile(np.eye(tmax, dtype=np.uint64)[None, None], (1, 1, 1, 1))
    xdig = np.zeros((1, n, 1, tmax), dtype=np.uint64)
    oracle.call("gdn_gen_natural", 1, n, 1, 1, tmax, tmax, 0, bases, C, xdig)
    st = _states(rng, r)
    got = np.zeros((r, n, 1, tmax_new), dtype=np.uint64)
    f = oracle.GdnNusForest(r)
    assert f.scramble(r, n, 1, 1, 1, tmax, tmax_new, st.reshape(-1).copy(), bases, xdig, got) == 0
    f.close()
    for l in range(r):
        prefix = sorted(tuple(int(v) for v in got[l, i, 0, :m]) for i in range(n))
        assert len(set(prefix)) == n
