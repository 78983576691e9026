"""Concurrent use of the C ABI: the reference's functions are pure over their
arguments (qmctoolscl/c_funcs/*.c; `util.py:111` releases the GIL around
each call), and the library keeps that contract with per-call streams.
Several host threads, each on its own CUDA stream, call the kernels
(through ctypes, GIL released) and create and run generalized-net plans
of different shared-memory sizes at the same time; every result must equal
the one computed alone."""
import threading

import numpy as np
import pytest

import qmctoolscl_gb300 as q
from qmctoolscl_gb300 import _ffi, halton

from .test_gpu_halton import PRIMES, _dev_dims, make_dims, same_bits

pytestmark = pytest.mark.gpu
U = np.uint64
THREADS = 4
ROUNDS = 6


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).reshape(-1).view(np.int64)).cuda()


def _run_threads(work):
    """work(k) for k < THREADS on THREADS host threads; re-raises the first failure."""
    errors = []

    def body(k):
        try:
            work(k)
        except BaseException as e:  # noqa: BLE001 - reported below
            errors.append(e)

    ts = [threading.Thread(target=body, args=(k,)) for k in range(THREADS)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    if errors:
        raise errors[0]


def test_plain_kernels_from_threads_on_own_streams():
    import torch
    lib = _ffi.lib()
    rng = np.random.Generator(np.random.SFC64(90))
    r, n, d = 3, 1 << 14, 12
    g = (rng.integers(0, 1 << 19, (r, d), dtype=U) * U(2) + U(1))
    shifts = rng.random((r, d))
    mmax = 14
    C = rng.integers(0, 1 << 62, (r, d, mmax), dtype=U)
    b, tmax = 3, 41
    xdig = rng.integers(0, b, (r, n, 1, tmax), dtype=U)
    bb = np.array([[b]], U)
    nf, nv = 1 << 13, 8
    fr, fi = rng.standard_normal((nv, nf)), rng.standard_normal((nv, nf))
    gd, sd, Cd, xd, bd = _dev(g), torch.from_numpy(shifts).cuda(), _dev(C), _dev(xdig), _dev(bb)

    def compute(st):
        """Every kernel family once on stream st; returns the outputs."""
        h = st.cuda_stream
        with torch.cuda.stream(st):
            xl = torch.empty(r * n * d, dtype=torch.float64, device="cuda")
            xs = torch.empty_like(xl)
            xb = torch.empty(r * n * d, dtype=torch.int64, device="cuda")
            xf = torch.empty(r * n, dtype=torch.float64, device="cuda")
            zr, zi = torch.from_numpy(fr).cuda(), torch.from_numpy(fi).cuda()
        _ffi.check(lib.qmc_lat_gen_gray(r, n, d, 0, gd.data_ptr(), xl.data_ptr(), h), "lat_gen_gray")
        _ffi.check(lib.qmc_lat_shift_mod_1(r, n, d, r, xl.data_ptr(), sd.data_ptr(), xs.data_ptr(), h), "shift")
        _ffi.check(lib.qmc_dnb2_gen_natural(r, n, d, 0, mmax, Cd.data_ptr(), xb.data_ptr(), h), "dnb2_gen")
        _ffi.check(lib.qmc_gdn_integer_to_float(r, n, 1, 1, tmax, bd.data_ptr(), xd.data_ptr(), xf.data_ptr(), h),
                   "gdn_integer_to_float")
        _ffi.check(lib.qmc_tc_fft_bro_1d(nv, 1, nf // 2, zr.data_ptr(), zi.data_ptr(), h), "tc_fft")
        st.synchronize()
        return [t.cpu().numpy() for t in (xs, xb, xf, zr, zi)]

    want = compute(torch.cuda.current_stream())
    got = {}

    def work(k):
        st = torch.cuda.Stream()
        for i in range(ROUNDS):
            got[(k, i)] = compute(st)

    _run_threads(work)
    _ffi.check(lib.qmc_device_error_check(torch.cuda.current_stream().cuda_stream), "device error word")
    for outs in got.values():
        for a, w in zip(outs, want):
            assert same_bits(a, w)


def test_halton_plans_created_and_run_from_threads():
    """Plans of different dimension counts (output tiles of different shared-memory
    sizes, some above the 48 KB default) created and run concurrently."""
    import torch
    rng = np.random.Generator(np.random.SFC64(91))
    specs = []
    for k in range(THREADS):
        d = (100, 40, 97, 12)[k]
        r, n, n_start = 2, 700 + 37 * k, 5 * k
        dims = make_dims(rng, r, PRIMES[:d], n_start + n - 1)
        specs.append((r, n, n_start, dims))
    # each spec alone first
    wants = []
    for r, n, n_start, dims in specs:
        x = torch.empty(r * n * len(dims), dtype=torch.float64, device="cuda")
        plan = halton.HaltonPlan(r, n, n_start, _dev_dims(dims), x)
        plan.prepare()
        plan.run()
        torch.cuda.synchronize()
        wants.append(x.cpu().numpy())
        plan.close()
    got = {}

    def work(k):
        r, n, n_start, dims = specs[k]
        st = torch.cuda.Stream()
        for i in range(ROUNDS):
            with torch.cuda.stream(st):
                x = torch.full((r * n * len(dims),), float("nan"), dtype=torch.float64, device="cuda")
            plan = halton.HaltonPlan(r, n, n_start, _dev_dims(dims), x)
            plan.prepare(st)
            plan.run(st)
            st.synchronize()
            got[(k, i)] = x.cpu().numpy()
            plan.close()

    _run_threads(work)
    for (k, _i), x in got.items():
        assert same_bits(x, wants[k])
