"""Tensor-core transforms: the FFT of bit-reversed input, its inverse and the
Walsh-Hadamard transform with radix-16 steps as BF16 tensor-core products
(three-term BF16 splits, FP32 accumulation).  Same arguments as the FP64
functions minus the twiddle arrays: fft_bro_1d_tc(d1, d2, n_half, xr, xi),
ifft_bro_1d_tc(d1, d2, n_half, xr, xi), fwht_1d_tc(d1, d2, n_half, x), in
place on numpy arrays (copied to the GPU and back) or CUDA float64 tensors.
Relative L2 error about 1e-7 against the FP64 transforms.

fft_mul_ifft_tc(d1, d2, n_half, lam_r, lam_i, xr, xi, divide=False, scale=1.0)
is the fast kernel matrix-vector product (divide=False: ifft(fft(y) * lam) *
scale) or solve (divide=True: ifft(fft(y) / lam) * scale) of the reference's
documentation in one call, fft / ifft being fft_bro_1d_radix2 /
ifft_bro_1d_radix2; lam holds n values for every vector or one per element.
fwht_mul_fwht_tc(d1, d2, n_half, lam, x, ...) is its Walsh-Hadamard analog,
and fft_mul_ifft / fwht_mul_fwht the same two fused forms in FP64."""
import numpy as np

from . import _ffi


def _run(fn_name, d1, d2, n_half, arrays, stream=None):
    import torch
    d1, d2, n_half = int(d1), int(d2), int(n_half)
    count = d1 * d2 * 2 * n_half
    s = stream if stream is not None else torch.cuda.current_stream()
    with torch.cuda.stream(s):  # the copies in on the call's stream, ahead of the kernels
        devs, back = _device_arrays(torch, arrays, count)
        rc = getattr(_ffi.lib(), fn_name)(d1, d2, n_half, *[t.data_ptr() for t in devs], s.cuda_stream)
        _ffi.check(rc, fn_name)
        for a, t in back:
            torch.from_numpy(a.reshape(-1)[:count]).copy_(t)
        _ffi.check(_ffi.lib().qmc_device_error_check(s.cuda_stream), fn_name)


def _device_arrays(torch, arrays, count):
    """CUDA float64 tensors as they are; numpy arrays copied to the device (and listed to copy back)."""
    devs, back = [], []
    for a in arrays:
        if isinstance(a, torch.Tensor):
            if not a.is_cuda or a.dtype != torch.float64 or not a.is_contiguous() or a.numel() < count:
                raise ValueError("need contiguous CUDA float64 tensors of %d elements" % count)
            devs.append(a)
        else:
            if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"] or a.size < count:
                raise ValueError("need C-contiguous float64 arrays of %d elements" % count)
            if not a.flags["WRITEABLE"]:
                raise ValueError("the transforms work in place: a read-only array cannot take the result")
            t = torch.from_numpy(a.reshape(-1)[:count]).cuda()
            devs.append(t)
            back.append((a, t))
    return devs, back


def fft_bro_1d_tc(d1, d2, n_half, xr, xi, stream=None):
    _run("qmc_tc_fft_bro_1d", d1, d2, n_half, [xr, xi], stream)


def ifft_bro_1d_tc(d1, d2, n_half, xr, xi, stream=None):
    _run("qmc_tc_ifft_bro_1d", d1, d2, n_half, [xr, xi], stream)


def fwht_1d_tc(d1, d2, n_half, x, stream=None):
    _run("qmc_tc_fwht_1d", d1, d2, n_half, [x], stream)


def _lam_tensors(torch, arrays, n, count):
    """lam arrays as contiguous CUDA float64 tensors of n or count values, and
    whether they hold one value per element"""
    lam = []
    for a in arrays:
        t = a if isinstance(a, torch.Tensor) else \
            torch.from_numpy(_ffi.writable(np.ascontiguousarray(a, dtype=np.float64)))
        t = t.to(device="cuda", dtype=torch.float64).contiguous().reshape(-1)
        if t.numel() not in (n, count):
            raise ValueError("lam needs n = %d or d1*d2*n = %d values" % (n, count))
        lam.append(t)
    if len({t.numel() for t in lam}) != 1:
        raise ValueError("lam_r and lam_i differ in size")
    return lam, (1 if lam[0].numel() == count and count != n else 0)


def _fused(fn_name, d1, d2, n_half, lams, data, divide, scale, stream, twiddles=False):
    import torch
    d1, d2, n_half = int(d1), int(d2), int(n_half)
    n = 2 * n_half
    count = d1 * d2 * n
    s = stream if stream is not None else torch.cuda.current_stream()
    with torch.cuda.stream(s):  # every copy in on the call's stream, ahead of the kernels
        lam, per_element = _lam_tensors(torch, lams, n, count)
        devs, back = _device_arrays(torch, data, count)
        tw = [torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(2)] if twiddles else []
        L = _ffi.lib()
        args = [d1, d2, n_half] + [t.data_ptr() for t in tw] + [t.data_ptr() for t in lam] + \
            [per_element, 1 if divide else 0, float(scale)] + [t.data_ptr() for t in devs] + [s.cuda_stream]
        _ffi.check(getattr(L, fn_name)(*args), fn_name)
        for a, t in back:
            torch.from_numpy(a.reshape(-1)[:count]).copy_(t)
        _ffi.check(L.qmc_device_error_check(s.cuda_stream), fn_name)


def fft_mul_ifft_tc(d1, d2, n_half, lam_r, lam_i, xr, xi, divide=False, scale=1.0, stream=None):
    """y <- IFFT(FFT(y) * lam) * scale (or / lam) in place on (xr, xi) with the
    tensor-core transforms; lam of n values shared by every vector, or of
    d1*d2*n values (one per element)."""
    _fused("qmc_tc_fft_mul_ifft", d1, d2, n_half, (lam_r, lam_i), (xr, xi), divide, scale, stream)


def fwht_mul_fwht_tc(d1, d2, n_half, lam, x, divide=False, scale=1.0, stream=None):
    """y <- FWHT(FWHT(y) * lam) * scale (or / lam) in place on x with the
    tensor-core WHT; lam real, n values shared by every vector or one per
    element (the reference's fast Walsh kernel product and solve,
    docs/index.md:1929-1978)."""
    _fused("qmc_tc_fwht_mul_fwht", d1, d2, n_half, (lam,), (x,), divide, scale, stream)


def fft_mul_ifft(d1, d2, n_half, lam_r, lam_i, xr, xi, divide=False, scale=1.0, stream=None):
    """The FP64 form of fft_mul_ifft_tc: fft_bro_1d_radix2, the pointwise
    product (or quotient) by lam and ifft_bro_1d_radix2 in one call, with the
    forward transform's last pass, the pointwise step and the inverse's first
    pass fused on each tile (docs/index.md:1825-1884, to FP64 rounding)."""
    _fused("qmc_fft_mul_ifft", d1, d2, n_half, (lam_r, lam_i), (xr, xi), divide, scale, stream, twiddles=True)


def fwht_mul_fwht(d1, d2, n_half, lam, x, divide=False, scale=1.0, stream=None):
    """The FP64 form of fwht_mul_fwht_tc (docs/index.md:1929-1978, to FP64
    rounding)."""
    _fused("qmc_fwht_mul_fwht", d1, d2, n_half, (lam,), (x,), divide, scale, stream)
