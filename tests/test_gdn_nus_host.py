"""Host-side checks of gdn_nested_uniform_scramble (qmctoolscl_gb300.nus)
that run before any GPU work: the GPU form's domain (bases 2..65536,
tmax < tmax_new, keys of at most 128 bits), root nodes of another class or
used by another implementation, generators other than SFC64 or shared
between pairs; and the workspace query of the C ABI (no GPU call)."""
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
    one = nus.gdn_workspace_bytes(1 << 12, 0, 1)
    assert nus.gdn_workspace_bytes(1 << 12, 0, 8) > 7 * one
    assert nus.gdn_workspace_bytes(1 << 12, 1 << 12, 1) > one  # trees with earlier entries hold more
