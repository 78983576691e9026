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


class HaltonRequest(_ct.Structure):
    """qmc_halton_request (include/qmcgb.h)."""
    _fields_ = [("r", _U64), ("n", _U64), ("n_start", _U64), ("d", _U64), ("dims", _ct.POINTER(GdnDim)), ("x", _P)]


def _lib():
    L = _ffi.lib()
    if not getattr(L, "_halton_bound", False):
        L.qmc_halton_plan_create.argtypes = [_U64, _U64, _U64, _U64, _ct.POINTER(GdnDim), _P, _ct.POINTER(_P)]
        L.qmc_halton_batch_create.argtypes = [_ct.POINTER(HaltonRequest), _ct.c_int, _ct.POINTER(_P)]
        L.qmc_halton_plan_prepare.argtypes = [_P, _P]
        L.qmc_halton_plan_run.argtypes = [_P, _P]
        L.qmc_halton_plan_graph_launch.argtypes = [_P, _P]
        L.qmc_halton_plan_destroy.argtypes = [_P]
        L.qmc_halton_plan_set_fp64_share.argtypes = [_P, _ct.c_double]
        for fn in ("qmc_halton_plan_create", "qmc_halton_batch_create", "qmc_halton_plan_prepare",
                   "qmc_halton_plan_run", "qmc_halton_plan_graph_launch", "qmc_halton_plan_destroy",
                   "qmc_halton_plan_set_fp64_share"):
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


def _x_pointer(x, count):
    torch = _torch()
    if isinstance(x, np.ndarray):
        if x.dtype != np.float64 or not x.flags["C_CONTIGUOUS"] or x.size < count:
            raise ValueError("x must be a C-contiguous float64 array of at least r*n*d elements")
        ptr = _ffi.device_pointer_of_host(x.ctypes.data)
        if ptr is None:
            raise ValueError("a numpy x must be pinned host memory (batch.pinned_empty)")
        return ptr
    _check_tensor(x, "x", count, (torch.float64,))
    return x.data_ptr()


def _dim_structs(r, dims, keep, tag):
    torch = _torch()
    ints = (torch.int64, torch.uint64)
    if not dims:
        raise ValueError("%s: need at least one dimension" % tag)
    structs = []
    for j, q in enumerate(dims):
        b, tmax, mmax = int(q["b"]), int(q["tmax"]), int(q["mmax"])
        _check_tensor(q["C"], "%sdims[%d].C" % (tag, j), mmax * tmax, ints)
        ptrs = {"C": q["C"].data_ptr()}
        for key, count in (("S", r * tmax * tmax), ("perms", r * tmax * b), ("shifts", r * tmax)):
            t = q.get(key)
            if t is None:
                ptrs[key] = None
            else:
                _check_tensor(t, "%sdims[%d].%s" % (tag, j, key), count, ints)
                ptrs[key] = t.data_ptr()
                keep.append(t)
        keep.append(q["C"])
        structs.append(GdnDim(b=b, tmax=tmax, mmax=mmax, **ptrs))
    return (GdnDim * len(structs))(*structs)


class HaltonBatch:
    """Many generalized-net requests of uneven (r, n, n_start, d, bases, digit
    counts) in one plan: preparation and generation each one launch over all
    requests.  Each request is a dict(r, n, n_start=0, dims=[...], x=...) with
    the arrays of HaltonPlan.  The plan keeps the tensors alive; prepare()
    reads S, C, perms and shifts (call it again after changing them), run()
    writes every request's x; graph_launch(stream) does both from a CUDA graph
    captured at the first call."""

    def __init__(self, requests):
        if not requests:
            raise ValueError("need at least one request")
        keep, structs, dim_arrays = [], [], []
        for k, q in enumerate(requests):
            r, n = int(q["r"]), int(q["n"])
            d = len(q["dims"])
            arr = _dim_structs(r, q["dims"], keep, "requests[%d]." % k)
            dim_arrays.append(arr)
            x = q["x"]
            keep.append(x)
            structs.append(HaltonRequest(r=r, n=n, n_start=int(q.get("n_start", 0)), d=d, dims=arr,
                                         x=_x_pointer(x, r * n * d)))
        reqs = (HaltonRequest * len(structs))(*structs)
        h = _P()
        _ffi.check(_lib().qmc_halton_batch_create(reqs, len(structs), _ct.byref(h)), "halton_batch_create")
        self._h = h
        self._keep = keep
        self.nreq = len(structs)
        self.coords = sum(int(q["r"]) * int(q["n"]) * len(q["dims"]) for q in requests)
        self.share = 1.0

    def prepare(self, stream=None):
        s = stream if stream is not None else _torch().cuda.current_stream()
        _ffi.check(_lib().qmc_halton_plan_prepare(self._h, s.cuda_stream), "halton_plan_prepare")

    def run(self, stream=None):
        s = stream if stream is not None else _torch().cuda.current_stream()
        _ffi.check(_lib().qmc_halton_plan_run(self._h, s.cuda_stream), "halton_plan_run")

    def graph_launch(self, stream):
        _ffi.check(_lib().qmc_halton_plan_graph_launch(self._h, stream.cuda_stream), "halton_plan_graph_launch")

    def set_fp64_share(self, share):
        """Share of the digit adds run on the FP64 unit (the rest in integer
        arithmetic); the results are the same bits either way."""
        _ffi.check(_lib().qmc_halton_plan_set_fp64_share(self._h, float(share)), "halton_plan_set_fp64_share")
        self.share = float(share)

    def tune(self, stream=None, shares=(0.0, 0.5, 0.75, 1.0), reps=3, use_cache=True):
        """Time run() at each FP64 share, keep the fastest, remember it for plans of the same
        shape class (the autotuner cache of qmctoolscl_gb300.batch).  Returns (share, ms)."""
        from . import batch
        torch = _torch()
        stream = stream if stream is not None else torch.cuda.current_stream()
        key = "halton|coords2^%d|req2^%d|%s" % (int(np.log2(max(self.coords, 1))), int(np.log2(max(self.nreq, 1))),
                                               batch._device_name())
        if use_cache:
            hit = batch._load_cache().get(key)
            if hit:
                self.set_fp64_share(hit[0])
                return tuple(hit)
        self.prepare(stream)
        best = None
        for sh in shares:
            self.set_fp64_share(sh)
            ms = batch.time_plan(self, stream, reps)
            if best is None or ms < best[1]:
                best = (sh, ms)
        self.set_fp64_share(best[0])
        batch._store_cache(key, list(best))
        return best

    def close(self):
        if getattr(self, "_h", None):
            _lib().qmc_halton_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class HaltonPlan(HaltonBatch):
    """One fused generalized-net generation over device tensors (a batch of
    one request).  x may also be a pinned float64 numpy array
    (batch.pinned_empty): the kernel then writes the points straight into host
    memory."""

    def __init__(self, r, n, n_start, dims, x):
        super().__init__([dict(r=r, n=n, n_start=n_start, dims=dims, x=x)])
        self.r, self.n, self.d = int(r), int(n), len(dims)


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
