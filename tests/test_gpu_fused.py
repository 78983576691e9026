"""The fused fast-transform forms against numpy: y <- IFFT(FFT(y) * lam) * s
and y <- FWHT(FWHT(y) * lam) * s (and the quotients), in FP64
(qmc_fft_mul_ifft, qmc_fwht_mul_fwht: to 1e-10 like the reference's
documented matrix-vector product and solve, docs/index.md:1825-1884 and
1929-1978) and with the tensor cores (qmc_tc_fwht_mul_fwht: 1e-6); one, two
and three passes, lam shared by the vectors or one per element, numpy
arrays and CUDA tensors.  The Walsh-Hadamard checker is a numpy restatement
of the orthonormal transform (Sylvester order, the reference's sympy.fwht(x)
/ sqrt(n))."""
import numpy as np
import pytest

import qmctoolscl_gb300 as q
from qmctoolscl_gb300 import tc_fft

pytestmark = pytest.mark.gpu


def _bitrev(m):
    i = np.arange(1 << m)
    out = np.zeros_like(i)
    for b in range(m):
        out |= ((i >> b) & 1) << (m - 1 - b)
    return out


def _fwht_np(x):
    """orthonormal Walsh-Hadamard transform along the last axis (Sylvester order)"""
    y = np.array(x, dtype=np.float64, copy=True)
    n = y.shape[-1]
    h = 1
    while h < n:
        y = y.reshape(y.shape[:-1] + (n // (2 * h), 2, h))
        a, b = y[..., 0, :].copy(), y[..., 1, :].copy()
        y[..., 0, :], y[..., 1, :] = a + b, a - b
        y = y.reshape(y.shape[:-3] + (n,))
        h *= 2
    return y / np.sqrt(n)


CASES = [(1, 1, 1, False, False), (5, 2, 1, False, True), (10, 1, 3, True, False), (12, 2, 2, False, True),
         (13, 1, 2, True, False), (16, 1, 1, False, False), (20, 1, 1, True, True), (21, 1, 1, False, False)]


@pytest.mark.parametrize("m,d1,d2,per_element,divide", CASES)
def test_fft_mul_ifft_fp64(m, d1, d2, per_element, divide):
    rng = np.random.Generator(np.random.SFC64(900 + m))
    n = 1 << m
    br = _bitrev(m)
    y = rng.standard_normal((d1, d2, n)) + 1j * rng.standard_normal((d1, d2, n))
    shape = (d1, d2, n) if per_element else (n,)
    lam = (0.5 + rng.random(shape)) * np.exp(2j * np.pi * rng.random(shape))
    scale = float(np.sqrt(2 * n))
    Y = np.fft.fft(y[..., br], norm="ortho")
    want = np.fft.ifft(Y / lam if divide else Y * lam, norm="ortho")[..., br] * scale
    xr, xi = np.ascontiguousarray(y.real), np.ascontiguousarray(y.imag)
    tc_fft.fft_mul_ifft(d1, d2, n // 2, np.ascontiguousarray(lam.real), np.ascontiguousarray(lam.imag), xr, xi,
                        divide=divide, scale=scale)
    err = np.linalg.norm((xr + 1j * xi) - want) / np.linalg.norm(want)
    assert err < 1e-12, err


@pytest.mark.parametrize("m,d1,d2,per_element,divide", CASES)
@pytest.mark.parametrize("tensor_cores", [False, True])
def test_fwht_mul_fwht(m, d1, d2, per_element, divide, tensor_cores):
    rng = np.random.Generator(np.random.SFC64(950 + m))
    n = 1 << m
    y = rng.standard_normal((d1, d2, n))
    shape = (d1, d2, n) if per_element else (n,)
    lam = (0.5 + rng.random(shape)) * np.where(rng.random(shape) < 0.5, -1.0, 1.0)
    scale = float(np.sqrt(2 * n))
    Y = _fwht_np(y)
    want = _fwht_np(Y / lam if divide else Y * lam) * scale
    x = np.ascontiguousarray(y)
    fn = tc_fft.fwht_mul_fwht_tc if tensor_cores else tc_fft.fwht_mul_fwht
    fn(d1, d2, n // 2, np.ascontiguousarray(lam), x, divide=divide, scale=scale)
    err = np.linalg.norm(x - want) / np.linalg.norm(want)
    assert err < (1e-6 if tensor_cores else 1e-12), err


def test_reference_matvec_and_solve_fp64():
    """docs/index.md:1825-1884 in one call each: u = ifft(yt*kt)*sqrt(2n) and
    v = ifft(yt/kt)/sqrt(2n), kt = fft(k) from the drop-in fft_bro_1d_radix2,
    against numpy at the documentation's tolerance (1e-10)"""
    rng = np.random.Generator(np.random.SFC64(7))
    m = 10
    n = 1 << m
    ir = _bitrev(m + 1)
    y = rng.random(2 * n) + 1j * rng.random(2 * n)
    k = rng.random(2 * n) + 0j
    kr, ki = np.ascontiguousarray(k.real), np.ascontiguousarray(k.imag)
    q.fft_bro_1d_radix2(np.uint64(1), np.uint64(1), np.uint64(n), np.empty(2 * n), np.empty(2 * n), kr, ki)
    u_np = np.fft.ifft(np.fft.fft(y[ir], norm="ortho") * np.fft.fft(k[ir], norm="ortho"), norm="ortho")[ir] \
        * np.sqrt(2 * n)
    v_np = np.fft.ifft(np.fft.fft(y[ir], norm="ortho") / np.fft.fft(k[ir], norm="ortho"), norm="ortho")[ir] \
        / np.sqrt(2 * n)
    ur, ui = np.ascontiguousarray(y.real), np.ascontiguousarray(y.imag)
    tc_fft.fft_mul_ifft(1, 1, n, kr, ki, ur, ui, scale=np.sqrt(2 * n))
    assert np.allclose(ur + 1j * ui, u_np, atol=1e-10)
    vr, vi = np.ascontiguousarray(y.real), np.ascontiguousarray(y.imag)
    tc_fft.fft_mul_ifft(1, 1, n, kr, ki, vr, vi, divide=True, scale=1.0 / np.sqrt(2 * n))
    assert np.allclose(vr + 1j * vi, v_np, atol=1e-10)


def test_reference_walsh_matvec_and_solve():
    """docs/index.md:1929-1978 in one call each (u = fwht(yt*kt)*sqrt(2n), v =
    fwht(yt/kt)/sqrt(2n), kt = fwht(k) from the drop-in fwht_1d_radix2), FP64
    at the documentation's 1e-8 against the numpy transform, the tensor-core
    form at 1e-6 relative"""
    rng = np.random.Generator(np.random.SFC64(8))
    m = 10
    n = 1 << m
    y = rng.random(2 * n)
    kt = rng.random(2 * n)
    q.fwht_1d_radix2(np.uint64(1), np.uint64(1), np.uint64(n), kt)
    u_np = _fwht_np(_fwht_np(y) * kt) * np.sqrt(2 * n)
    v_np = _fwht_np(_fwht_np(y) / kt) / np.sqrt(2 * n)
    for fn, tol in ((tc_fft.fwht_mul_fwht, None), (tc_fft.fwht_mul_fwht_tc, 1e-6)):
        u = y.copy()
        fn(1, 1, n, kt, u, scale=np.sqrt(2 * n))
        v = y.copy()
        fn(1, 1, n, kt, v, divide=True, scale=1.0 / np.sqrt(2 * n))
        if tol is None:
            assert np.allclose(u, u_np, atol=1e-8) and np.allclose(v, v_np, atol=1e-8)
        else:
            # the solve divides by kt: its error is the transforms' times kt's condition
            cond = np.abs(kt).max() / np.abs(kt).min()
            assert np.linalg.norm(u - u_np) / np.linalg.norm(u_np) < tol
            assert np.linalg.norm(v - v_np) / np.linalg.norm(v_np) < tol * cond


def test_device_tensors_in_place():
    import torch
    rng = np.random.Generator(np.random.SFC64(9))
    n = 1 << 14
    y = rng.standard_normal((3, n))
    lam = 0.5 + rng.random(n)
    want = _fwht_np(_fwht_np(y) * lam)
    t = torch.from_numpy(y.copy()).cuda()
    tc_fft.fwht_mul_fwht(3, 1, n // 2, torch.from_numpy(lam).cuda(), t)
    assert np.linalg.norm(t.cpu().numpy() - want) / np.linalg.norm(want) < 1e-12
