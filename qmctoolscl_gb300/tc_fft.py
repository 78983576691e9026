"""Tensor-core transforms: the FFT of bit-reversed input, its inverse and the
Walsh-Hadamard transform with radix-16 steps as BF16 tensor-core products
(three-term BF16 splits, FP32 accumulation).  Same arguments as the FP64
functions minus the twiddle arrays: fft_bro_1d_tc(d1, d2, n_half, xr, xi),
ifft_bro_1d_tc(d1, d2, n_half, xr, xi), fwht_1d_tc(d1, d2, n_half, x), in
place on numpy arrays (copied to the GPU and back) or CUDA float64 tensors.
Relative L2 error about 1e-7 against the FP64 transforms."""
import numpy as np

from . import _ffi


def _run(fn_name, d1, d2, n_half, arrays, stream=None):
    import torch
    d1, d2, n_half = int(d1), int(d2), int(n_half)
    count = d1 * d2 * 2 * n_half
    s = stream if stream is not None else torch.cuda.current_stream()
    devs, back = [], []
    for a in arrays:
        if isinstance(a, torch.Tensor):
            if not a.is_cuda or a.dtype != torch.float64 or not a.is_contiguous() or a.numel() < count:
                raise ValueError("need contiguous CUDA float64 tensors of %d elements" % count)
            devs.append(a)
        else:
            if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"] or a.size < count:
                raise ValueError("need C-contiguous float64 arrays of %d elements" % count)
            t = torch.from_numpy(a.reshape(-1)[:count]).cuda()
            devs.append(t)
            back.append((a, t))
    with torch.cuda.stream(s):
        rc = getattr(_ffi.lib(), fn_name)(d1, d2, n_half, *[t.data_ptr() for t in devs], s.cuda_stream)
        _ffi.check(rc, fn_name)
        for a, t in back:
            torch.from_numpy(a.reshape(-1)[:count]).copy_(t)
        _ffi.check(_ffi.lib().qmc_device_error_check(s.cuda_stream), fn_name)


def fft_bro_1d_tc(d1, d2, n_half, xr, xi, stream=None):
    _run("qmc_tc_fft_bro_1d", d1, d2, n_half, [xr, xi], stream)


def ifft_bro_1d_tc(d1, d2, n_half, xr, xi, stream=None):
    _run("qmc_tc_ifft_bro_1d", d1, d2, n_half, [xr, xi], stream)


def fwht_1d_tc(d1, d2, n_half, x, stream=None):
    _run("qmc_tc_fwht_1d", d1, d2, n_half, [x], stream)
