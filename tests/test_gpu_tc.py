"""The tcgen05 (fifth-generation tensor core) building blocks: a one-CTA
BF16 x BF16 -> FP32 MMA through tensor memory, with the shared-memory and
instruction descriptors the tensor-core transforms use, against an exact
host product (small integers are exact in BF16 and in the FP32 sums); then
the tensor-core transforms against numpy."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from qmctoolscl_gb300 import _build, _ffi

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    """tests/cuda/tc_probe.cu built as a test-only library (it is not part of libqmcgb.so)."""
    so = str(tmp_path_factory.mktemp("tcprobe") / "libtcprobe.so")
    subprocess.run([_build.nvcc()] + _build.ARCH + ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-o", so,
                                                    os.path.join(HERE, "cuda", "tc_probe.cu")], check=True)
    L = ctypes.CDLL(so)
    L.tc_mma_probe.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_uint32] * 2 + [ctypes.c_void_p] * 2
    L.tc_mma_probe.restype = ctypes.c_int
    return L


@pytest.mark.parametrize("N,K", [(16, 16), (32, 16), (32, 64), (64, 32), (128, 128), (256, 16), (32, 192)])
def test_tcgen05_mma_probe_exact(probe, N, K):
    import torch
    g = torch.Generator().manual_seed(N * 1000 + K)
    A = torch.randint(-8, 9, (128, K), generator=g).to(torch.bfloat16).cuda()
    B = torch.randint(-8, 9, (N, K), generator=g).to(torch.bfloat16).cuda()
    D = torch.full((128, N), float("nan"), dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    assert probe.tc_mma_probe(A.data_ptr(), B.data_ptr(), D.data_ptr(), N, K, err.data_ptr(), s) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0, "the probe's completion wait ran out"
    want = A.double() @ B.double().T
    assert torch.equal(D.double(), want)


def _bitrev(m):
    i = np.arange(1 << m)
    out = np.zeros_like(i)
    for b in range(m):
        out |= ((i >> b) & 1) << (m - 1 - b)
    return out


# (11, 7, 143): 501 tiles of 4096 values, more than the grid's CTAs and the last one half full, so a
# CTA prefetches a partial tile while it works on a full one
@pytest.mark.parametrize("m,d1,d2", [(1, 1, 1), (4, 2, 3), (5, 1, 1), (8, 3, 5), (10, 2, 2), (11, 1, 3), (12, 2, 1),
                                     (13, 1, 2), (16, 1, 1), (17, 2, 1), (20, 1, 1), (22, 1, 1), (24, 1, 1),
                                     (11, 7, 143)])
def test_tc_fft_and_inverse_against_numpy(m, d1, d2):
    from qmctoolscl_gb300 import tc_fft
    rng = np.random.Generator(np.random.SFC64(m))
    n = 1 << m
    z = rng.standard_normal((d1, d2, n)) + 1j * rng.standard_normal((d1, d2, n))
    xr, xi = np.ascontiguousarray(z.real), np.ascontiguousarray(z.imag)
    tc_fft.fft_bro_1d_tc(d1, d2, n // 2, xr, xi)
    want = np.fft.fft(z[:, :, _bitrev(m)], norm="ortho")
    err = np.linalg.norm((xr + 1j * xi) - want) / np.linalg.norm(want)
    assert err < 1e-6, err
    tc_fft.ifft_bro_1d_tc(d1, d2, n // 2, xr, xi)
    err2 = np.linalg.norm((xr + 1j * xi) - z) / np.linalg.norm(z)
    assert err2 < 1e-6, err2


@pytest.mark.parametrize("m", [1, 4, 7, 12, 14, 19, 22])
def test_tc_fwht_against_fp64(m):
    from qmctoolscl_gb300 import tc_fft
    import qmctoolscl_gb300 as q
    rng = np.random.Generator(np.random.SFC64(100 + m))
    n = 1 << m
    x = rng.standard_normal((2, 1, n))
    want = x.copy()
    q.fwht_1d_radix2(np.uint64(2), np.uint64(1), np.uint64(n // 2), want)
    tc_fft.fwht_1d_tc(2, 1, n // 2, x)
    err = np.linalg.norm(x - want) / np.linalg.norm(want)
    assert err < 1e-6, err


def _fft_bro_np(x, br):
    """fft_bro_1d_radix2 of docs/index.md:1815: np.fft.fft of the bit-reversed input, orthonormal."""
    return np.fft.fft(x[..., br], norm="ortho")


def _ifft_bro_np(X, br):
    """ifft_bro_1d_radix2: the inverse of _fft_bro_np (natural input, bit-reversed output)."""
    return np.fft.ifft(X, norm="ortho")[..., br]


@pytest.mark.parametrize("m,d1,d2,per_element,divide", [(1, 1, 1, False, False), (5, 2, 1, False, False),
                                                        (10, 1, 3, True, False), (12, 2, 2, False, True),
                                                        (13, 1, 2, False, False), (16, 1, 1, True, True),
                                                        (20, 1, 1, False, False), (22, 1, 1, False, True),
                                                        (11, 7, 143, False, False)])
def test_tc_fft_mul_ifft_against_numpy(m, d1, d2, per_element, divide):
    """y <- IFFT(FFT(y) * lam) * s (or / lam) in one call against numpy: one, two and three
    passes, lam shared or per element, product and quotient."""
    from qmctoolscl_gb300 import tc_fft
    rng = np.random.Generator(np.random.SFC64(300 + m))
    n = 1 << m
    br = _bitrev(m)
    y = rng.standard_normal((d1, d2, n)) + 1j * rng.standard_normal((d1, d2, n))
    shape = (d1, d2, n) if per_element else (n,)
    lam = (0.5 + rng.random(shape)) * np.exp(2j * np.pi * rng.random(shape))  # |lam| in [0.5, 1.5)
    scale = float(np.sqrt(2 * n))
    Y = _fft_bro_np(y, br)
    want = _ifft_bro_np(Y / lam if divide else Y * lam, br) * scale
    xr, xi = np.ascontiguousarray(y.real), np.ascontiguousarray(y.imag)
    tc_fft.fft_mul_ifft_tc(d1, d2, n // 2, np.ascontiguousarray(lam.real), np.ascontiguousarray(lam.imag), xr, xi,
                           divide=divide, scale=scale)
    err = np.linalg.norm((xr + 1j * xi) - want) / np.linalg.norm(want)
    assert err < 1e-6, err


def test_tc_fft_mul_ifft_reference_matvec_and_solve():
    """The fast kernel matrix-vector product and solve of docs/index.md:1825-1884 (u =
    ifft(yt*kt)*sqrt(2n), v = ifft(yt/kt)/sqrt(2n), kt = fft(k)) with the kernel's
    transform kt from the FP64 drop-in fft_bro_1d_radix2, against numpy (TC tolerance)."""
    import qmctoolscl_gb300 as q
    from qmctoolscl_gb300 import tc_fft
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
    # the solve divides by kt: its error is the transforms' (about 1e-7) times kt's condition
    cond = np.abs(kr + 1j * ki).max() / np.abs(kr + 1j * ki).min()
    for divide, scale, want, tol in ((False, np.sqrt(2 * n), u_np, 1e-6), (True, 1 / np.sqrt(2 * n), v_np, 1e-6 * cond)):
        xr, xi = np.ascontiguousarray(y.real), np.ascontiguousarray(y.imag)
        tc_fft.fft_mul_ifft_tc(1, 1, n, kr, ki, xr, xi, divide=divide, scale=scale)
        err = np.linalg.norm((xr + 1j * xi) - want) / np.linalg.norm(want)
        assert err < tol, (divide, err, cond)
