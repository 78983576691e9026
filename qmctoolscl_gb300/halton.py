"""Fused generalized digital nets with a base per dimension (randomised Halton).

For each dimension j the reference's chain

    gdn_linear_matrix_scramble -> gdn_gen_natural -> gdn_digital_permutation
    -> gdn_digital_shift -> gdn_integer_to_float

called with d = 1, r_b = 1, r_C = 1 and tmax_new = tmax_j
(qmctoolscl/c_funcs/gdn_*.c), its floats written to column j of one
r x n x d array.  The reference takes a single tmax per call, so a Halton
point set with per-base digit counts is one such chain per dimension; here it
is one kernel over all dimensions that never stores a digit.

A step is left out when its array is None (S: no linear matrix scramble,
perms: no permutation, shifts: no digital shift), for all dimensions alike.

    dims = [dict(b=2, tmax=64, mmax=18, C=C0, S=S0, perms=P0, shifts=H0), ...]
    plan = HaltonPlan(r, n, n_start, dims, x)   # x: r*n*d float64 CUDA tensor
    plan.prepare()                              # packs S*C mod b, perms, shifts
    plan.run()                                  # writes x

C is mmax x tmax, S r x tmax x tmax, perms r x tmax x b and shifts r x tmax
per dimension (the reference's shapes at d = 1), uint64 values in int64 or
uint64 CUDA tensors.  ``generalized_net_fused`` does the same from numpy
arrays, copying them in and the points out (or writing the points straight
into pinned host memory).
"""
import ctypes as _ct

import numpy as np

from . import _ffi

_U64, _P = _ct.c_uint64, _ct.c_void_p


class GdnDim(_ct.Structure):
    """qmc_gdn_dim (include/qmcgb.h)."""
    _fields_ = [("b", _U64), ("tmax", _U64), ("mmax", _U64), ("S", _P), ("C", _P), ("perms", _P), ("shifts", _P)]


def _lib():
    L = _ffi.lib()
    if not getattr(L, "_halton_bound", False):
        L.qmc_halton_plan_create.argtypes = [_U64, _U64, _U64, _U64, _ct.POINTER(GdnDim), _P, _ct.POINTER(_P)]
        L.qmc_halton_plan_prepare.argtypes = [_P, _P]
        L.qmc_halton_plan_run.argtypes = [_P, _P]
        L.qmc_halton_plan_destroy.argtypes = [_P]
        L.qmc_halton_plan_set_fp64_share.argtypes = [_P, _ct.c_double]
        for fn in ("qmc_halton_plan_create", "qmc_halton_plan_prepare", "qmc_halton_plan_run",
                   "qmc_halton_plan_destroy", "qmc_halton_plan_set_fp64_share"):
            getattr(L, fn).restype = _ct.c_int
        L._halton_bound = True
    return L


def _torch():
    import torch
    return torch


def _check_tensor(t, name, count, dtypes):
    torch = _torch()
    if not isinstance(t, torch.Tensor) or not t.is_cuda or not t.is_contiguous():
        raise TypeError("%s must be a contiguous CUDA tensor" % name)
    if t.dtype not in dtypes:
        raise TypeError("%s has dtype %s" % (name, t.dtype))
    if t.numel() < count:
        raise ValueError("%s has %d elements, needs %d" % (name, t.numel(), count))


def _create(r, n, n_start, structs, x_ptr):
    arr = (GdnDim * len(structs))(*structs)
    h = _P()
    _ffi.check(_lib().qmc_halton_plan_create(int(r), int(n), int(n_start), len(structs), arr, x_ptr, _ct.byref(h)),
               "halton_plan_create")
    return h


class HaltonPlan:
    """One fused generalized-net generation over device tensors.  The plan
    keeps the tensors alive; prepare() reads S, C, perms and shifts (call it
    again after changing them), run() writes x.  x may also be a pinned
    float64 numpy array (batch.pinned_empty): the kernel then writes the
    points straight into host memory."""

    def __init__(self, r, n, n_start, dims, x):
        torch = _torch()
        r, n, n_start = int(r), int(n), int(n_start)
        ints = (torch.int64, torch.uint64)
        if not dims:
            raise ValueError("need at least one dimension")
        d = len(dims)
        if isinstance(x, np.ndarray):
            if x.dtype != np.float64 or not x.flags["C_CONTIGUOUS"] or x.size < r * n * d:
                raise ValueError("x must be a C-contiguous float64 array of at least r*n*d elements")
            x_ptr = _ffi.device_pointer_of_host(x.ctypes.data)
            if x_ptr is None:
                raise ValueError("a numpy x must be pinned host memory (batch.pinned_empty)")
        else:
            _check_tensor(x, "x", r * n * d, (torch.float64,))
            x_ptr = x.data_ptr()
        structs, keep = [], [x]
        for j, q in enumerate(dims):
            b, tmax, mmax = int(q["b"]), int(q["tmax"]), int(q["mmax"])
            _check_tensor(q["C"], "dims[%d].C" % j, mmax * tmax, ints)
            ptrs = {"C": q["C"].data_ptr()}
            for key, count in (("S", r * tmax * tmax), ("perms", r * tmax * b), ("shifts", r * tmax)):
                t = q.get(key)
                if t is None:
                    ptrs[key] = None
                else:
                    _check_tensor(t, "dims[%d].%s" % (j, key), count, ints)
                    ptrs[key] = t.data_ptr()
                    keep.append(t)
            keep.append(q["C"])
            structs.append(GdnDim(b=b, tmax=tmax, mmax=mmax, **ptrs))
        self._h = _create(r, n, n_start, structs, x_ptr)
        self._keep = keep
        self.r, self.n, self.d = r, n, d

    def prepare(self, stream=None):
        s = stream if stream is not None else _torch().cuda.current_stream()
        _ffi.check(_lib().qmc_halton_plan_prepare(self._h, s.cuda_stream), "halton_plan_prepare")

    def run(self, stream=None):
        s = stream if stream is not None else _torch().cuda.current_stream()
        _ffi.check(_lib().qmc_halton_plan_run(self._h, s.cuda_stream), "halton_plan_run")

    def set_fp64_share(self, share):
        """Share of the digit adds run on the FP64 unit (the rest in integer
        arithmetic); the results are the same bits either way."""
        _ffi.check(_lib().qmc_halton_plan_set_fp64_share(self._h, float(share)), "halton_plan_set_fp64_share")

    def close(self):
        if getattr(self, "_h", None):
            _lib().qmc_halton_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def generalized_net_fused(r, n, n_start, dims, x, check=True, stream=None):
    """The fused chain from numpy inputs (or CUDA tensors): copies each
    dimension's arrays to the GPU, prepares, runs, and delivers the r x n x d
    floats into x -- written directly when x is pinned (batch.pinned_empty),
    else staged on the device and copied back.  With check, the device error
    word is read afterwards.  Returns the batch._Args of the call (its
    h2d_bytes / d2h_bytes count the copies)."""
    from .batch import _Args
    torch = _torch()
    r, n, n_start = int(r), int(n), int(n_start)
    A = _Args(stream)
    with torch.cuda.stream(A.stream):
        structs = []
        for j, q in enumerate(dims):
            b, tmax, mmax = int(q["b"]), int(q["tmax"]), int(q["mmax"])
            structs.append(GdnDim(
                b=b, tmax=tmax, mmax=mmax,
                C=A.ptr(q["C"], np.uint64, mmax * tmax, name="dims[%d].C" % j),
                S=A.ptr(q.get("S"), np.uint64, r * tmax * tmax, name="dims[%d].S" % j),
                perms=A.ptr(q.get("perms"), np.uint64, r * tmax * b, name="dims[%d].perms" % j),
                shifts=A.ptr(q.get("shifts"), np.uint64, r * tmax, name="dims[%d].shifts" % j)))
        px = A.ptr(x, np.float64, r * n * len(dims), out=True, name="x")
        h = _create(r, n, n_start, structs, px)
        try:
            L = _lib()
            if check:
                _ffi.check(_ffi.lib().qmc_device_error_reset(A.stream.cuda_stream), "device_error_reset")
            _ffi.check(L.qmc_halton_plan_prepare(h, A.stream.cuda_stream), "halton_plan_prepare")
            _ffi.check(L.qmc_halton_plan_run(h, A.stream.cuda_stream), "halton_plan_run")
            if check:
                _ffi.check(_ffi.lib().qmc_device_error_check(A.stream.cuda_stream), "generalized_net_fused")
            A.finish()
        finally:
            A.stream.synchronize()  # the plan's tables are freed below
            _lib().qmc_halton_plan_destroy(h)
    return A
