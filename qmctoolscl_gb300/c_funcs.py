"""The reference's generated ctypes module exposes halton_qrng only as the raw
binding `qmctoolscl.c_funcs.halton_qrng_c` (pdm_build.py:84-94), not through
the wrapped API: this module mirrors that name and contract.

halton_qrng_c(n, d, n0, generalized, res, randu_d_32, dvec): four C ints, then
res (float64, C-contiguous, d*n values, written), randu_d_32 (float64, d*32)
and dvec (C int, d), each checked as np.ctypeslib.ndpointer checks it
(ctypes.ArgumentError otherwise); returns None like the C function.  The
points come from the GPU kernel qmc_halton_qrng (bit for bit the reference's
values); numpy arrays are copied to the device and res back, CUDA tensors
(float64 / int32) are used in place."""
import ctypes

import numpy as np

from . import _ffi

_C_INT_MIN, _C_INT_MAX = -(1 << 31), (1 << 31) - 1


def _c_int(v, pos):
    if isinstance(v, (bool, np.bool_)) or isinstance(v, (float, np.floating)) or not hasattr(v, "__index__"):
        raise ctypes.ArgumentError("argument %d: TypeError: wrong type" % (pos + 1))
    v = int(v) & 0xFFFFFFFF  # c_int keeps the low 32 bits
    return v - (1 << 32) if v > _C_INT_MAX else v


def _is_torch(a):
    return type(a).__module__.startswith("torch") and hasattr(a, "data_ptr")


def _check(a, dtype, pos):
    if _is_torch(a):
        import torch
        want = torch.float64 if dtype == np.float64 else torch.int32
        if a.dtype != want or not a.is_cuda or not a.is_contiguous():
            raise ctypes.ArgumentError("argument %d: TypeError: need a contiguous CUDA %s tensor" % (pos + 1, want))
        return
    if not isinstance(a, np.ndarray):
        raise ctypes.ArgumentError("argument %d: TypeError: argument must be an ndarray" % (pos + 1))
    if a.dtype != dtype:
        raise ctypes.ArgumentError("argument %d: TypeError: array must have data type %s"
                                   % (pos + 1, np.dtype(dtype).name))
    if not a.flags["C_CONTIGUOUS"]:
        raise ctypes.ArgumentError("argument %d: TypeError: array must have flags ['C_CONTIGUOUS']" % (pos + 1))


def halton_qrng_c(n, d, n0, generalized, res, randu_d_32, dvec):
    n, d, n0, generalized = (_c_int(v, k) for k, v in enumerate((n, d, n0, generalized)))
    _check(res, np.float64, 4)
    _check(randu_d_32, np.float64, 5)
    _check(dvec, np.int32, 6)
    if n <= 0 or d <= 0:
        return None
    for a, need, name in ((res, d * n, "res"), (randu_d_32, d * 32, "randu_d_32"), (dvec, d, "dvec")):
        size = a.numel() if _is_torch(a) else a.size
        if size < need:
            raise ValueError("%s has %d elements, halton_qrng needs %d (the reference would read past it)"
                             % (name, size, need))
    import torch
    s = torch.cuda.current_stream()
    dev = []
    for a in (res, randu_d_32, dvec):
        dev.append(a if _is_torch(a) else torch.from_numpy(_ffi.writable(a.reshape(-1))).cuda())
    L = _ffi.lib()
    _ffi.check(L.qmc_halton_qrng(n, d, n0, generalized, dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(),
                                 s.cuda_stream), "halton_qrng")
    if not _is_torch(res):
        torch.from_numpy(res.reshape(-1)).copy_(dev[0])
    _ffi.check(L.qmc_device_error_check(s.cuda_stream), "halton_qrng")
    return None
