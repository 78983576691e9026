"""Host-side checks of dnb2_nested_uniform_scramble (qmctoolscl_gb300.nus)
that run before any GPU work: the reference's AssertionError for tmax_new
above 64 on fresh trees (rand_funcs.py:13), root nodes of another class,
generators other than SFC64, argument types; and the workspace query of the
C ABI (no GPU call)."""
import ctypes

import numpy as np
import pytest

import qmctoolscl_gb300 as q
from qmctoolscl_gb300 import nus


def _args(r=1, n=4, d=1):
    gens = np.array([np.random.Generator(np.random.SFC64(k)) for k in range(r * d)], dtype=object).reshape(r, d)
    roots = np.array([q.NUSNode_dnb2() for _ in range(r * d)]).reshape(r, d)
    return gens, roots, np.zeros((1, n, d), np.uint64), np.zeros((r, n, d), np.uint64)


def test_tmax_new_above_64_asserts_like_the_reference():
    gens, roots, xb, xrb = _args()
    with pytest.raises(AssertionError):
        q.dnb2_nested_uniform_scramble(1, 4, 1, 1, 8, 65, gens, roots, xb, xrb)


def test_foreign_root_nodes_assert():
    gens, _roots, xb, xrb = _args()

    class Other:
        shift_bits = None

    with pytest.raises(AssertionError):
        q.dnb2_nested_uniform_scramble(1, 4, 1, 1, 8, 16, gens, [Other()], xb, xrb)


def test_non_sfc64_generators_are_refused():
    _gens, roots, xb, xrb = _args()
    with pytest.raises(TypeError):
        q.dnb2_nested_uniform_scramble(1, 4, 1, 1, 8, 16, [np.random.Generator(np.random.PCG64(1))], roots, xb, xrb)


def test_array_types_checked():
    gens, roots, xb, xrb = _args()
    with pytest.raises(ctypes.ArgumentError):
        q.dnb2_nested_uniform_scramble(1, 4, 1, 1, 8, 16, gens, roots, xb.astype(np.int64), xrb)
    with pytest.raises(ValueError):
        q.dnb2_nested_uniform_scramble(1, 4, 1, 1, 8, 16, gens, roots, xb[:, :2].copy(), xrb)
    with pytest.raises(ValueError):  # r*d generators needed
        q.dnb2_nested_uniform_scramble(2, 4, 1, 1, 8, 16, gens, roots, xb, np.zeros((2, 4, 1), np.uint64))


def test_workspace_query():
    one = nus.workspace_bytes(1 << 16, 0, 1)
    many = nus.workspace_bytes(1 << 16, 0, 64)
    assert one > 50 * (1 << 16) and 60 * one <= many <= 64 * one + 4096
    with pytest.raises(ValueError):  # more than 2^30 - 1 entries per generator
        nus.workspace_bytes(1 << 30, 0, 1)


def test_shared_generator_is_refused():
    g = np.random.Generator(np.random.SFC64(3))
    _gens, roots, xb, xrb = _args(r=2)
    with pytest.raises(ValueError):
        q.dnb2_nested_uniform_scramble(2, 4, 1, 1, 8, 16, np.array([g, g], dtype=object).reshape(2, 1), roots, xb,
                                       xrb)
    h = np.random.Generator(g.bit_generator)  # a second Generator on the same bit generator
    with pytest.raises(ValueError):
        q.dnb2_nested_uniform_scramble(2, 4, 1, 1, 8, 16, np.array([g, h], dtype=object).reshape(2, 1), roots, xb,
                                       xrb)
