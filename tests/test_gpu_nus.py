"""Nested uniform scrambling of base-2 nets on the GPU
(qmctoolscl_gb300.nus, C entry point qmc_dnb2_nested_uniform_scramble)
against the reference's own results (golden vectors from
qmctoolscl/rand_funcs.py:162-253, the documented example included) and
against the oracle on seeded inputs: outputs bit for bit and the numpy
generator states after every call, over fresh trees, continuation calls on
the same root nodes, duplicates, keys of 1 to 64 bits, tmax above
tmax_new, chunked workspaces and device-tensor arguments."""
import os

import numpy as np
import pytest

import oracle
import qmctoolscl_gb300 as q
from qmctoolscl_gb300.nus import NUSNode_dnb2, set_sfc64_state, sfc64_state_words

pytestmark = pytest.mark.gpu
GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "nus.npz"))
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
def test_golden(c):
    r, n, d, r_x, tmax, tmax_new, calls = (int(v) for v in GOLD["case%d_args" % c])
    gens = _gens(GOLD["case%d_state0" % c])
    rngs = np.array(gens, dtype=object).reshape(r, d)
    roots = np.array([NUSNode_dnb2() for _ in range(r * d)]).reshape(r, d)
    for k in range(calls):
        xrb = np.full((r, n, d), 7, dtype=np.uint64)
        q.dnb2_nested_uniform_scramble(r, n, d, r_x, tmax, tmax_new, rngs, roots, GOLD["case%d_xb%d" % (c, k)], xrb)
        assert np.array_equal(xrb, GOLD["case%d_xrb%d" % (c, k)]), (c, k)
        assert np.array_equal(_states(gens), GOLD["case%d_state%d" % (c, k + 1)]), (c, k)


def _net(rng, r_x, n, d, m, tmax):
    """natural-order net points with random upper-unit-triangular matrices, MSB-first in tmax bits"""
    C = np.zeros((d, m), dtype=np.uint64)
    for j in range(d):
        M = np.triu(rng.integers(0, 2, (m, m)), 1) + np.eye(m, dtype=np.int64)
        for k in range(m):
            C[j, k] = sum(int(M[t, k]) << (tmax - 1 - t) for t in range(m))
    i = np.arange(n, dtype=np.uint64)
    xb = np.zeros((n, d), dtype=np.uint64)
    for k in range(m):
        bit = ((i >> np.uint64(k)) & np.uint64(1)).astype(bool)
        xb[bit] ^= C[:, k]
    return np.ascontiguousarray(np.broadcast_to(xb, (r_x, n, d)))


def _check_against_oracle(rng, r, n, d, r_x, tmax, tmax_new, xbs, workspace=None):
    seeds = np.random.SeedSequence(int(rng.integers(0, 2 ** 31))).spawn(r * d)
    gens = [np.random.Generator(np.random.SFC64(s)) for s in seeds]
    for k, g in enumerate(gens):
        if k % 3 == 1:
            g.integers(0, 2 ** 9)  # a buffered 32-bit half
    words = _states(gens).reshape(-1).copy()
    forest = oracle.NusForest(r * d)
    rngs = np.array(gens, dtype=object).reshape(r, d)
    roots = np.array([NUSNode_dnb2() for _ in range(r * d)]).reshape(r, d)
    kw = {} if workspace is None else {"workspace_bytes": workspace}
    for xb in xbs:
        want = np.zeros((r, n, d), dtype=np.uint64)
        forest.scramble(r, n, d, r_x, tmax, tmax_new, words, xb, want)
        got = np.zeros((r, n, d), dtype=np.uint64)
        q.dnb2_nested_uniform_scramble(r, n, d, r_x, tmax, tmax_new, rngs, roots, xb, got, **kw)
        assert np.array_equal(got, want)
        assert np.array_equal(_states(gens).reshape(-1), words)
    forest.close()


@pytest.mark.parametrize("seed", range(12))
def test_random_words_against_oracle(seed):
    rng = np.random.Generator(np.random.SFC64(500 + seed))
    r_x = int(rng.integers(1, 3))
    r, d, n = r_x * int(rng.integers(1, 3)), int(rng.integers(1, 6)), int(rng.integers(1, 3000))
    tmax = int(rng.integers(0, 65))
    tmax_new = int(rng.integers(0, 65)) if seed % 4 == 3 else int(rng.integers(tmax, 65))
    kind = seed % 3
    if kind == 0:
        mk = lambda: rng.integers(0, 2 ** 63, (r_x, n, d), dtype=np.uint64) * np.uint64(2)  # noqa: E731
    elif kind == 1:
        mk = lambda: rng.integers(0, 4, (r_x, n, d), dtype=np.uint64) << np.uint64(max(tmax - 2, 0))  # noqa: E731
    else:
        mk = lambda: rng.integers(0, 1 << max(min(tmax, 62), 1), (r_x, n, d), dtype=np.uint64)  # noqa: E731
    _check_against_oracle(rng, r, n, d, r_x, tmax, tmax_new, [mk(), mk()])


@pytest.mark.parametrize("m,tmax,tmax_new,r,d", [(10, 32, 64, 2, 5), (14, 64, 64, 3, 4), (12, 12, 40, 1, 3),
                                                 (16, 63, 64, 1, 2)])
def test_net_points_against_oracle(m, tmax, tmax_new, r, d):
    rng = np.random.Generator(np.random.SFC64(m))
    n = 1 << m
    xb = _net(rng, 1, n, d, m, tmax)
    nxt = _net(rng, 1, n, d, m, tmax)
    _check_against_oracle(rng, r, n, d, 1, tmax, tmax_new, [xb, nxt])


def test_chunked_workspace_matches():
    rng = np.random.Generator(np.random.SFC64(77))
    r, n, d = 3, 5000, 7
    xb = _net(rng, 1, 8192, d, 13, 64)[:, :n].copy()
    per = q.nus.workspace_bytes(n, 0, 1)
    for ws in (per, 3 * per + 100):  # one generator per chunk, then three
        _check_against_oracle(np.random.Generator(np.random.SFC64(78)), r, n, d, 1, 64, 64, [xb], workspace=ws)


def test_zero_points_draws_root_bits_only():
    rng = np.random.Generator(np.random.SFC64(79))
    _check_against_oracle(rng, 2, 0, 3, 1, 8, 40, [np.zeros((1, 0, 3), np.uint64), np.zeros((1, 0, 3), np.uint64)])


def test_device_tensors_in_place():
    import torch
    rng = np.random.Generator(np.random.SFC64(80))
    r, n, d = 2, 4096, 3
    xb = _net(rng, 1, n, d, 12, 64)
    gens_a = [np.random.Generator(np.random.SFC64(s)) for s in range(r * d)]
    gens_b = [np.random.Generator(np.random.SFC64(s)) for s in range(r * d)]
    want = np.zeros((r, n, d), np.uint64)
    q.dnb2_nested_uniform_scramble(r, n, d, 1, 64, 64, np.array(gens_a, dtype=object).reshape(r, d),
                                   np.array([NUSNode_dnb2() for _ in range(r * d)]).reshape(r, d), xb, want)
    dx = torch.from_numpy(xb.reshape(-1).view(np.int64).copy()).cuda()
    dout = torch.zeros(r * n * d, dtype=torch.int64, device="cuda")
    q.dnb2_nested_uniform_scramble(r, n, d, 1, 64, 64, np.array(gens_b, dtype=object).reshape(r, d),
                                   np.array([NUSNode_dnb2() for _ in range(r * d)]).reshape(r, d), dx, dout)
    assert np.array_equal(dout.cpu().numpy().view(np.uint64).reshape(r, n, d), want)
    assert np.array_equal(_states(gens_a), _states(gens_b))


def test_argument_errors():
    g = [np.random.Generator(np.random.SFC64(1))]
    xb = np.zeros((1, 4, 1), np.uint64)
    with pytest.raises(AssertionError):
        q.dnb2_nested_uniform_scramble(1, 4, 1, 1, 8, 65, g, [NUSNode_dnb2()], xb, np.zeros_like(xb))
    with pytest.raises(TypeError):
        q.dnb2_nested_uniform_scramble(1, 4, 1, 1, 8, 16, [np.random.Generator(np.random.PCG64(1))],
                                       [NUSNode_dnb2()], xb, np.zeros_like(xb))
    used = NUSNode_dnb2()
    q.dnb2_nested_uniform_scramble(1, 4, 1, 1, 8, 16, g, [used], xb, np.zeros_like(xb))
    gens2 = [np.random.Generator(np.random.SFC64(2)) for _ in range(2)]
    with pytest.raises(ValueError):  # one used tree next to a fresh one
        q.dnb2_nested_uniform_scramble(2, 4, 1, 1, 8, 16, gens2, [used, NUSNode_dnb2()],
                                       xb, np.zeros((2, 4, 1), np.uint64))
    with pytest.raises(ValueError):  # a tree built for another tmax_new
        q.dnb2_nested_uniform_scramble(1, 4, 1, 1, 8, 20, g, [used], xb, np.zeros_like(xb))
