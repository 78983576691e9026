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


def test_c_entry_points_check_arguments_before_any_launch():
    """the C ABI rejects out-of-domain calls with a status and a message, on
    the host, before touching any pointer (addresses here are never used)"""
    from qmctoolscl_gb300 import _ffi
    lib = _ffi.lib()
    fake = 0x100000  # 256-byte aligned, never dereferenced by a rejected call
    rc = lib.qmc_dnb2_nested_uniform_scramble(1, 4, 1, 1, 8, 65, fake, 0, None, None, fake, fake, None, None, fake,
                                              1 << 30, None)
    assert rc == _ffi.QMC_ERR_DOMAIN and b"between 0 and 64" in lib.qmc_last_error()
    rc = lib.qmc_dnb2_nested_uniform_scramble(1, 4, 1, 1, 8, 16, fake, 0, None, None, fake, fake, None, None, fake,
                                              64, None)  # workspace far too small
    assert rc == _ffi.QMC_ERR_ARG and b"workspace" in lib.qmc_last_error()
    needed = ctypes.c_uint64(7)
    off = (ctypes.c_uint64 * 2)()

    def gdn(r, tmax_new, states=fake, h0=0, hist=None, off_=off):
        # (r, n, d, r_x, r_b, tmax, tmax_new, states, bases, h0, hist_keys, hist_perms, hist_perm_off, xdig,
        #  xrdig, keys_out, perms, perm_capacity, perm_off, perm_needed, work, work_bytes, stream)
        return lib.qmc_gdn_nested_uniform_scramble(r, 4, 1, 1, 1, 3, tmax_new, states, fake, h0, hist, hist, hist,
                                                   fake, fake, None, fake, 1 << 20, off_, ctypes.byref(needed), fake,
                                                   1 << 30, None)

    rc = gdn(1, 3)
    assert rc == _ffi.QMC_ERR_ARG and b"tmax < tmax_new" in lib.qmc_last_error() and needed.value == 0
    assert gdn(1, 5, states=None) == _ffi.QMC_ERR_ARG
    assert gdn(1, 5, off_=None) == _ffi.QMC_ERR_ARG  # no permutation offsets
    rc = gdn(1, 5, h0=3)  # earlier entries without their keys and permutations
    assert rc == _ffi.QMC_ERR_ARG and b"h0" in lib.qmc_last_error()
    assert gdn(0, 5, states=None) == _ffi.QMC_OK  # r = 0: nothing to do


def test_host_write_decision(monkeypatch):
    """where the kernels may write a numpy result directly: the device alias of
    pinned memory; the array's own address when the GPU reaches pageable memory
    through the host page tables; otherwise nowhere (a device buffer and a copy)"""
    from qmctoolscl_gb300 import _ffi
    arr = np.zeros(8, np.uint64)
    ptr = arr.ctypes.data
    monkeypatch.setattr(nus, "_ATTRS", {})
    monkeypatch.setattr(_ffi, "device_pointer_of_host", lambda p: p + 4096)
    assert nus._host_writable(arr, True) == ptr + 4096
    assert nus._host_writable(arr, False) is None
    monkeypatch.setattr(_ffi, "device_pointer_of_host", lambda p: None)
    monkeypatch.setattr(_ffi, "device_attributes",
                        lambda: {"pageable_access": 1, "uses_host_page_tables": 1, "sms": 152})
    assert nus._host_writable(arr, True) == ptr
    monkeypatch.setattr(nus, "_ATTRS", {})
    monkeypatch.setattr(_ffi, "device_attributes",
                        lambda: {"pageable_access": 1, "uses_host_page_tables": 0, "sms": 132})
    assert nus._host_writable(arr, True) is None
