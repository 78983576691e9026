"""qmc_net_gen_noalloc: one digital-net request without any device
allocation, for callers whose device memory belongs to another allocator
(a framework's caching pool, a serving process's fixed arena) or who must not
take cudaMalloc's implicit synchronisation in a latency-bound loop.

Called through the C ABI and checked, bit for bit (the tolerance every
integer test here uses), against the existing entry point that runs the same
chain -- a one-request plan -- on two calls in a row with different inputs;
the second call reuses the library's fixed matrix scratch the first one
filled.  Collected last so a run that stops at the first failure has run
everything else; it also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest

import qmctoolscl_gb300 as q
from qmctoolscl_gb300 import _ffi, batch

pytestmark = pytest.mark.gpu
U = np.uint64


def _lib():
    L = _ffi.lib()
    L.qmc_net_gen_noalloc.argtypes = [ctypes.POINTER(batch.NetRequest), ctypes.c_void_p]
    L.qmc_net_gen_noalloc.restype = ctypes.c_int
    return L


def _dev(a):
    import torch
    if a is None:
        return None
    a = np.ascontiguousarray(a)
    return torch.from_numpy(a.view(np.int64) if a.dtype == np.uint64 else a).cuda()


def _request(seed, r, m, d, alpha, order, with_float):
    rng = np.random.Generator(np.random.SFC64(seed))
    n = 1 << m
    d_pre = d * alpha
    C = q.random_tbit_uint64s(rng, 63, (1, d_pre, m + 1))
    S = q.dnb2_get_linear_scramble_matrix(rng, r, d_pre, 63, 64, False)
    shifts = q.dnb2_get_digital_shifts(rng, r, d, 64)
    req = dict(r=r, n=n, d=d, alpha=alpha, d_pre=d_pre, mmax=m + 1, tmax=63, tmax_new=64,
               tmax_alpha=min(alpha * 64, 64), r_C=1, order=order, C=_dev(C), S=_dev(S),
               lshifts=_dev(np.arange(r, dtype=U)), shifts=_dev(shifts),
               tmaxes=_dev(np.full(r, 64, U)) if with_float else None)
    return req


def _struct(req, xb, x):
    p = lambda t: None if t is None else t.data_ptr()  # noqa: E731
    return batch.NetRequest(r=req["r"], n=req["n"], d=req["d"], n_start=0, mmax=req["mmax"], d_pre=req["d_pre"],
                            alpha=req["alpha"], tmax=req["tmax"], tmax_new=req["tmax_new"],
                            tmax_alpha=req["tmax_alpha"], r_C=req["r_C"], gray=1 if req["order"] == "gray" else 0,
                            C=p(req["C"]), S=p(req["S"]), lshifts=p(req["lshifts"]), shifts=p(req["shifts"]),
                            tmaxes=p(req.get("tmaxes")), xb=p(xb), x=p(x))


def test_no_alloc_entry_point_matches_plan_on_two_calls():
    import torch
    L = _lib()
    stream = torch.cuda.current_stream()
    reqs = [_request(1, r=3, m=12, d=16, alpha=2, order="natural", with_float=False),
            _request(2, r=2, m=13, d=70, alpha=3, order="gray", with_float=True)]
    outs = []
    # two calls in a row on one stream; the second overwrites the scratch
    for req in reqs:
        size = req["r"] * req["n"] * req["d"]
        xb = torch.full((size,), -1, dtype=torch.int64, device="cuda")
        x = torch.full((size,), -1.0, dtype=torch.float64, device="cuda") if req["tmaxes"] is not None else None
        st = _struct(req, xb, x)
        rc = L.qmc_net_gen_noalloc(ctypes.byref(st), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, _ffi.last_error()
        outs.append((xb, x))
    torch.cuda.synchronize()
    for req, (xb, x) in zip(reqs, outs):
        want_xb = torch.full_like(xb, -1)
        want_x = torch.full_like(x, -1.0) if x is not None else None
        plan = batch.NetPlan([dict(req, xb=want_xb, x=want_x)])
        plan.run(stream)
        torch.cuda.synchronize()
        assert torch.equal(xb, want_xb)
        if x is not None:
            assert torch.equal(x.view(torch.int64), want_x.view(torch.int64))


def test_no_alloc_rejects_requests_beyond_its_scratch():
    import torch
    L = _lib()
    # r*d*mmax = 64*128*17 words of prepared matrices: more than the fixed scratch
    req = _request(3, r=64, m=16, d=128, alpha=1, order="natural", with_float=False)
    xb = torch.empty(1, dtype=torch.int64, device="cuda")  # rejected before any launch
    st = _struct(req, xb, None)
    rc = L.qmc_net_gen_noalloc(ctypes.byref(st), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == _ffi.QMC_ERR_ARG
    assert "131072" in _ffi.last_error()
