"""Nested uniform scrambling of generalized (base-b) nets on the GPU
(qmctoolscl_gb300.gdn_nested_uniform_scramble, C entry point
qmc_gdn_nested_uniform_scramble) against the reference's own results (golden
vectors from qmctoolscl/rand_funcs.py:262-356, the documented example
included, every call of the multi-call cases on the same root nodes) and
against the oracle on seeded inputs: digits bit for bit and the numpy
generator states after each call, over bases 2..541, replicated bases and
points, repeated points, chunked workspaces, device tensors, and trees
continued after their generators were drawn from between calls."""
import os

import numpy as np
import pytest

import oracle
import qmctoolscl_gb300 as q
from qmctoolscl_gb300.nus import NUSNode_gdn, set_sfc64_state, sfc64_state_words

pytestmark = pytest.mark.gpu
GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "gdn_nus.npz"))
NCASES = len([k for k in GOLD.files if k.endswith("_args")])


def _gens(words):
    out = []
    for w in words:
        g = np.random.Generator(np.random.SFC64(0))
        set_sfc64_state(g, w)
        out.append(g)
    return out


def _states(gens):
    return np.stack([sfc64_state_words(g) for g in gens])


@pytest.mark.parametrize("c", range(NCASES))
def test_golden_first_call(c):
    r, n, d, r_x, r_b, tmax, tmax_new, _calls = (int(v) for v in GOLD["case%d_args" % c])
    gens = _gens(GOLD["case%d_state0" % c])
    xr = np.full((r, n, d, tmax_new), 9, dtype=np.uint64)
    q.gdn_nested_uniform_scramble(r, n, d, r_x, r_b, tmax, tmax_new, np.array(gens, dtype=object).reshape(r, d),
                                  np.array([NUSNode_gdn() for _ in range(r * d)]).reshape(r, d),
                                  GOLD["case%d_bases" % c], GOLD["case%d_xdig0" % c], xr)
    assert np.array_equal(xr, GOLD["case%d_xrdig0" % c])
    assert np.array_equal(_states(gens), GOLD["case%d_state1" % c])


@pytest.mark.parametrize("c", range(NCASES))
@pytest.mark.parametrize("tensors", [False, True])
def test_golden_every_call(c, tensors):
    """later calls on the same root nodes continue the trees from the kept
    keys and permutations, as the reference's nodes do; with numpy arrays or
    CUDA tensors for xdig and xrdig"""
    import torch
    r, n, d, r_x, r_b, tmax, tmax_new, calls = (int(v) for v in GOLD["case%d_args" % c])
    if calls < 2 and tensors:
        pytest.skip("single-call case")
    gens = _gens(GOLD["case%d_state0" % c])
    rngs = np.array(gens, dtype=object).reshape(r, d)
    roots = np.array([NUSNode_gdn() for _ in range(r * d)]).reshape(r, d)
    for k in range(calls):
        xd = GOLD["case%d_xdig%d" % (c, k)]
        if tensors:
            xd = torch.from_numpy(np.ascontiguousarray(xd).reshape(-1).view(np.int64)).cuda()
            xr = torch.full((r * n * d * tmax_new,), 9, dtype=torch.int64, device="cuda")
        else:
            xr = np.full((r, n, d, tmax_new), 9, dtype=np.uint64)
        q.gdn_nested_uniform_scramble(r, n, d, r_x, r_b, tmax, tmax_new, rngs, roots, GOLD["case%d_bases" % c], xd,
                                      xr)
        got = xr.cpu().numpy().view(np.uint64).reshape(r, n, d, tmax_new) if tensors else xr
        assert np.array_equal(got, GOLD["case%d_xrdig%d" % (c, k)]), (c, k)
        assert np.array_equal(_states(gens), GOLD["case%d_state%d" % (c, k + 1)]), (c, k)


def test_generators_drawn_from_between_calls_continue_their_streams():
    """the reference's nodes keep their trees and the generators simply go on:
    draws taken from a generator between calls shift the next call's draws"""
    rng = np.random.Generator(np.random.SFC64(83))
    r, n, d, tmax, tmax_new = 2, 400, 2, 6, 8
    bases = np.array([[3, 7]], dtype=np.uint64)
    gens = [np.random.Generator(np.random.SFC64(s)) for s in range(r * d)]
    roots = np.array([NUSNode_gdn() for _ in range(r * d)]).reshape(r, d)
    f = oracle.GdnNusForest(r * d)
    for call in range(3):
        xdig = _digits(rng, 1, n, d, tmax, bases)
        words = _states(gens).reshape(-1).copy()
        want = np.zeros((r, n, d, tmax_new), dtype=np.uint64)
        assert f.scramble(r, n, d, 1, 1, tmax, tmax_new, words, bases, xdig, want) == 0
        got = np.zeros((r, n, d, tmax_new), dtype=np.uint64)
        q.gdn_nested_uniform_scramble(r, n, d, 1, 1, tmax, tmax_new, np.array(gens, dtype=object).reshape(r, d),
                                      roots, bases, xdig, got)
        assert np.array_equal(got, want), call
        assert np.array_equal(_states(gens).reshape(-1), words), call
        for g in gens[::2]:
            g.integers(0, 1000, 3)  # between calls
    f.close()


def _check(rng, r, n, d, r_x, r_b, tmax, tmax_new, bases, xdig, **kw):
    seeds = np.random.SeedSequence(int(rng.integers(0, 2 ** 31))).spawn(r * d)
    gens = [np.random.Generator(np.random.SFC64(s)) for s in seeds]
    for k, g in enumerate(gens):
        if k % 3 == 1:
            g.integers(0, 2 ** 9)
    words = _states(gens).reshape(-1).copy()
    want = np.zeros((r, n, d, tmax_new), dtype=np.uint64)
    f = oracle.GdnNusForest(r * d)
    assert f.scramble(r, n, d, r_x, r_b, tmax, tmax_new, words, bases, xdig, want) == 0
    f.close()
    got = np.zeros((r, n, d, tmax_new), dtype=np.uint64)
    q.gdn_nested_uniform_scramble(r, n, d, r_x, r_b, tmax, tmax_new, np.array(gens, dtype=object).reshape(r, d),
                                  np.array([NUSNode_gdn() for _ in range(r * d)]).reshape(r, d), bases, xdig, got,
                                  **kw)
    assert np.array_equal(got, want)
    assert np.array_equal(_states(gens).reshape(-1), words)


def _digits(rng, r_x, n, d, tmax, bases, low=False):
    bmin = bases.min(axis=0)
    x = rng.integers(0, 1 << 30, (r_x, n, d, tmax), dtype=np.uint64)
    if low:
        x = x % np.uint64(2)
    return np.ascontiguousarray(x % bmin[None, None, :, None])


@pytest.mark.parametrize("seed", range(10))
def test_random_against_oracle(seed):
    rng = np.random.Generator(np.random.SFC64(700 + seed))
    r_x = int(rng.integers(1, 3))
    r = r_x * int(rng.integers(1, 3))
    d = int(rng.integers(1, 4))
    r_b = 1 if r % 2 else int(rng.integers(1, 3))
    bases = rng.choice(np.array([2, 3, 5, 7, 11, 13, 541], dtype=np.uint64), (r_b, d))
    w = max(max(1, int(b - 1).bit_length()) for b in bases.reshape(-1))
    tmax = int(rng.integers(1, min(12, 128 // w) + 1))
    tmax_new = tmax + int(rng.integers(1, 5))
    n = int(rng.integers(1, 1500)) if bases.max() < 100 else int(rng.integers(1, 60))
    _check(rng, r, n, d, r_x, r_b, tmax, tmax_new, bases, _digits(rng, r_x, n, d, tmax, bases, low=seed % 3 == 1))


@pytest.mark.parametrize("b,tmax,tmax_new,n", [(2, 64, 70, 4096), (3, 41, 44, 3000), (5, 28, 30, 2000),
                                               (541, 8, 9, 300)])
def test_halton_depths_against_oracle(b, tmax, tmax_new, n):
    """tmax = ceil(64 / log2 b) digits as for 64-bit Halton points: keys of 64 to 82 bits"""
    rng = np.random.Generator(np.random.SFC64(b))
    bases = np.array([[b, b]], dtype=np.uint64)
    C = np.tile(np.eye(tmax, dtype=np.uint64)[None, None], (1, 2, 1, 1))
    xdig = np.zeros((1, n, 2, tmax), dtype=np.uint64)
    oracle.call("gdn_gen_natural", 1, n, 2, 1, tmax, tmax, 0, bases, C, xdig)
    _check(rng, 2, n, 2, 1, 1, tmax, tmax_new, bases, xdig)


def test_chunked_workspace_matches():
    rng = np.random.Generator(np.random.SFC64(81))
    bases = np.array([[3, 2, 7]], dtype=np.uint64)
    n = 700
    xdig = _digits(rng, 1, n, 3, 6, bases)
    per = q.nus.gdn_workspace_bytes(n, 0, 1)
    _check(rng, 2, n, 3, 1, 1, 6, 9, bases, xdig, workspace_bytes=per + 1000)


def test_device_tensors():
    import torch
    rng = np.random.Generator(np.random.SFC64(82))
    bases = np.array([[3, 5]], dtype=np.uint64)
    r, n, d, tmax, tmax_new = 2, 500, 2, 5, 7
    xdig = _digits(rng, 1, n, d, tmax, bases)
    gens_a = [np.random.Generator(np.random.SFC64(s)) for s in range(r * d)]
    gens_b = [np.random.Generator(np.random.SFC64(s)) for s in range(r * d)]
    want = np.zeros((r, n, d, tmax_new), np.uint64)
    q.gdn_nested_uniform_scramble(r, n, d, 1, 1, tmax, tmax_new, np.array(gens_a, dtype=object).reshape(r, d),
                                  np.array([NUSNode_gdn() for _ in range(r * d)]).reshape(r, d), bases, xdig, want)
    dx = torch.from_numpy(xdig.reshape(-1).view(np.int64)).cuda()
    dout = torch.zeros(r * n * d * tmax_new, dtype=torch.int64, device="cuda")
    q.gdn_nested_uniform_scramble(r, n, d, 1, 1, tmax, tmax_new, np.array(gens_b, dtype=object).reshape(r, d),
                                  np.array([NUSNode_gdn() for _ in range(r * d)]).reshape(r, d), bases, dx, dout)
    assert np.array_equal(dout.cpu().numpy().view(np.uint64).reshape(r, n, d, tmax_new), want)
    assert np.array_equal(_states(gens_a), _states(gens_b))


def test_digit_at_its_base_raises_index_error():
    gens = [np.random.Generator(np.random.SFC64(1))]
    xdig = np.array([[[[0, 1, 2]], [[1, 3, 0]]]], dtype=np.uint64)  # 3 is not a base-3 digit
    with pytest.raises(IndexError):
        q.gdn_nested_uniform_scramble(1, 2, 1, 1, 1, 3, 5, gens, [NUSNode_gdn()], np.array([[3]], np.uint64), xdig,
                                      np.zeros((1, 2, 1, 5), np.uint64))
