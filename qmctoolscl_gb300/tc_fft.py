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
ifft_bro_1d_radix2; lam holds n values for every vector or one per element."""
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


def fft_mul_ifft_tc(d1, d2, n_half, lam_r, lam_i, xr, xi, divide=False, scale=1.0, stream=None):
    """y <- IFFT(FFT(y) * lam) * scale (or / lam) in place on (xr, xi); lam of n values
    shared by every vector, or of d1*d2*n values (one per element)."""
    import torch
    d1, d2, n_half = int(d1), int(d2), int(n_half)
    n = 2 * n_half
    count = d1 * d2 * n
    s = stream if stream is not None else torch.cuda.current_stream()
    with torch.cuda.stream(s):  # every copy in on the call's stream, ahead of the kernels
        lam = []
        for a in (lam_r, lam_i):
            t = a if isinstance(a, torch.Tensor) else \
                torch.from_numpy(_ffi.writable(np.ascontiguousarray(a, dtype=np.float64)))
            t = t.to(device="cuda", dtype=torch.float64).contiguous().reshape(-1)
            if t.numel() not in (n, count):
                raise ValueError("lam needs n = %d or d1*d2*n = %d values" % (n, count))
            lam.append(t)
        if lam[0].numel() != lam[1].numel():
            raise ValueError("lam_r and lam_i differ in size")
        per_element = 1 if lam[0].numel() == count and count != n else 0
        devs, back = _device_arrays(torch, (xr, xi), count)
        L = _ffi.lib()
        _ffi.check(L.qmc_tc_fft_mul_ifft(d1, d2, n_half, lam[0].data_ptr(), lam[1].data_ptr(), per_element,
                                         1 if divide else 0, float(scale), devs[0].data_ptr(), devs[1].data_ptr(),
                                         s.cuda_stream), "tc_fft_mul_ifft")
        for a, t in back:
            torch.from_numpy(a.reshape(-1)[:count]).copy_(t)
        _ffi.check(L.qmc_device_error_check(s.cuda_stream), "tc_fft_mul_ifft")
