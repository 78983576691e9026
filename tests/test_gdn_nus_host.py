"""Host-side checks of gdn_nested_uniform_scramble (qmctoolscl_gb300.nus)
that run before any GPU work: the GPU form's domain (fresh trees, bases
2..65536, tmax < tmax_new, keys of at most 128 bits), root nodes of another
class, generators other than SFC64 or shared between pairs; and the
workspace query of the C ABI (no GPU call)."""
import numpy as np
import pytest

import qmctoolscl_gb300 as q
from qmctoolscl_gb300 import nus


def _call(r=1, n=2, d=1, tmax=3, tmax_new=5, bases=None, gens=None, roots=None):
    gens = gens if gens is not None else [np.random.Generator(np.random.SFC64(k)) for k in range(r * d)]
    roots = roots if roots is not None else [q.NUSNode_gdn() for _ in range(r * d)]
    bases = bases if bases is not None else np.full((1, d), 3, np.uint64)
    xdig = np.zeros((1, n, d, tmax), np.uint64)
    return q.gdn_nested_uniform_scramble(r, n, d, 1, 1, tmax, tmax_new, np.array(gens, dtype=object),
                                         np.array(roots, dtype=object), bases, xdig,
                                         np.zeros((r, n, d, tmax_new), np.uint64))


def test_foreign_used_roots_are_refused():
    node = q.NUSNode_gdn()
    node.perm = np.zeros(0, np.uint64)  # used, but not by this package: no history to continue
    with pytest.raises(ValueError):
        _call(roots=[node])


def _oracle_fresh(r, n, d, r_x, r_b, tmax, tmax_new, states, bases_np, xdig, xrdig, kwargs):
    """the oracle in place of the GPU call (numpy arrays only)"""
    import oracle
    words = np.ascontiguousarray(states, dtype=np.uint64).reshape(-1).copy()
    out = np.zeros((r, n, d, tmax_new), dtype=np.uint64)
    f = oracle.GdnNusForest(r * d)
    assert f.scramble(r, n, d, r_x, r_b, tmax, tmax_new, words, bases_np.reshape(r_b, d),
                      np.ascontiguousarray(xdig).reshape(r_x, n, d, tmax), out) == 0
    f.close()
    xrdig.reshape(-1)[:out.size] = out.reshape(-1)
    return words.reshape(r * d, 6)


def test_continued_trees_match_the_reference(monkeypatch):
    """Later calls on the same root nodes replay the earlier points from the
    first call's generator states; with the oracle in place of the GPU call,
    every call of the reference's multi-call golden cases matches, states too"""
    import os
    from qmctoolscl_gb300.nus import set_sfc64_state, sfc64_state_words
    monkeypatch.setattr(nus, "_gdn_fresh", _oracle_fresh)
    gold = np.load(os.path.join(os.path.dirname(__file__), "golden", "gdn_nus.npz"))
    ran = 0
    for c in range(len([k for k in gold.files if k.endswith("_args")])):
        r, n, d, r_x, r_b, tmax, tmax_new, calls = (int(v) for v in gold["case%d_args" % c])
        if calls < 2:
            continue
        gens = []
        for w in gold["case%d_state0" % c]:
            g = np.random.Generator(np.random.SFC64(0))
            set_sfc64_state(g, w)
            gens.append(g)
        rngs = np.array(gens, dtype=object).reshape(r, d)
        roots = np.array([q.NUSNode_gdn() for _ in range(r * d)]).reshape(r, d)
        for k in range(calls):
            xr = np.zeros((r, n, d, tmax_new), np.uint64)
            q.gdn_nested_uniform_scramble(r, n, d, r_x, r_b, tmax, tmax_new, rngs, roots, gold["case%d_bases" % c],
                                          gold["case%d_xdig%d" % (c, k)], xr)
            assert np.array_equal(xr, gold["case%d_xrdig%d" % (c, k)]), (c, k)
            assert np.array_equal(np.stack([sfc64_state_words(g) for g in gens]), gold["case%d_state%d" % (c, k + 1)])
        ran += 1
    assert ran >= 3


def test_a_generator_drawn_from_between_calls_is_refused(monkeypatch):
    monkeypatch.setattr(nus, "_gdn_fresh", _oracle_fresh)
    g = np.random.Generator(np.random.SFC64(4))
    roots = [q.NUSNode_gdn()]
    _call(gens=[g], roots=roots)
    _call(gens=[g], roots=roots)  # a continuation
    g.integers(0, 10)
    with pytest.raises(ValueError):
        _call(gens=[g], roots=roots)


def test_domain_of_the_gpu_form():
    with pytest.raises(ValueError):
        _call(tmax=3, tmax_new=3)
    with pytest.raises(ValueError):
        _call(bases=np.array([[70000]], np.uint64))
    with pytest.raises(ValueError):
        _call(bases=np.array([[1]], np.uint64))
    with pytest.raises(ValueError):  # 65 base-3 digits: 130 bits
        _call(tmax=65, tmax_new=66)


def test_generators_and_nodes():
    with pytest.raises(TypeError):
        _call(gens=[np.random.Generator(np.random.PCG64(1))])
    g = np.random.Generator(np.random.SFC64(2))
    with pytest.raises(ValueError):
        _call(r=2, gens=[g, g], bases=np.full((1, 1), 3, np.uint64))
    with pytest.raises(AssertionError):
        _call(roots=[q.NUSNode_dnb2()])


def test_workspace_query():
    one = nus.gdn_workspace_bytes(1 << 12, 1)
    assert nus.gdn_workspace_bytes(1 << 12, 8) > 7 * one


def test_history_digits_from_tensors_and_arrays():
    """the digits a tree keeps for replay, read from a numpy array or a tensor
    (here on the CPU; the drop-in passes CUDA tensors) and written back"""
    import torch
    x = np.arange(2 * 3 * 2 * 4, dtype=np.uint64).reshape(2, 3, 2, 4)
    assert np.array_equal(nus._host_digits(x, 2, 3, 2, 4), x)
    t = torch.from_numpy(x.reshape(-1).view(np.int64).copy())
    assert np.array_equal(nus._host_digits(t, 2, 3, 2, 4), x)
    out_t = torch.zeros(x.size, dtype=torch.int64)
    nus._store_digits(out_t, x)
    assert np.array_equal(out_t.numpy().view(np.uint64).reshape(x.shape), x)
    out_a = np.zeros_like(x)
    nus._store_digits(out_a, x)
    assert np.array_equal(out_a, x)
