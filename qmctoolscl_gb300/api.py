"""The QMCToolsCL call surface, running on the GB300 kernels of libqmcgb.so.

Every function takes the reference's arguments in the reference's order
(qmctoolscl/wrapped_funcs.py as generated by pdm_build.py:51-82: the C
signature without bs_r/bs_n/bs_d) and returns ``(t_perf, t_process)`` like
qmctoolscl/util.py:99-144: the wall-clock time of the call and the host CPU
time it used.

Arrays may be
  * numpy arrays (C-contiguous, exact dtype -- uint64 or float64, checked the
    way np.ctypeslib.ndpointer checks them, raising ctypes.ArgumentError):
    inputs are copied to the GPU, the kernel runs, and outputs are copied back
    into the same arrays, so the reference's in-place semantics hold;
  * CUDA torch tensors (contiguous, int64/uint64 or float64): used in place
    with no copies.

Keyword arguments: ``backend`` is accepted for compatibility ("c" or "cl",
case-insensitive, as the reference asserts) and does not change anything;
the OpenCL-only keywords (global_size, local_size, context, queue, program,
platform_id, device_id, profile) are accepted and ignored.  ``wait``
(default True, as in the reference's OpenCL path) synchronises the stream
before returning; with wait=False and only device tensors the call returns
right after the launch and t_process is -1.  ``stream`` selects a
torch.cuda.Stream (default: the current stream).

Errors.  Where the reference raises (lat_gen_natural's power-of-two check,
util.py:84-86) the same exception is raised.  Where the reference would
read or write outside the given arrays, a ValueError is raised instead
(documented divergence: the reference's behaviour there is undefined).
"""
import ctypes
import time

import numpy as np

from . import _ffi
from ._signatures import SIGNATURES

_torch = None


def _t():
    global _torch
    if _torch is None:
        import torch
        _torch = torch
    return _torch


# Elements each array must hold (the size strings of the reference's
# argument comments, qmctoolscl/c_funcs/*.c:3-16).
NEED = {
    "lat_gen_linear": lambda s: {"g": s["r"] * s["d"], "x": s["r"] * s["n"] * s["d"]},
    "lat_gen_natural": lambda s: {"g": s["r"] * s["d"], "x": s["r"] * s["n"] * s["d"]},
    "lat_gen_gray": lambda s: {"g": s["r"] * s["d"], "x": s["r"] * s["n"] * s["d"]},
    "lat_shift_mod_1": lambda s: {"x": s["r_x"] * s["n"] * s["d"], "shifts": s["r"] * s["d"],
                                  "xr": s["r"] * s["n"] * s["d"]},
    "dnb2_gen_natural": lambda s: {"C": s["r"] * s["d"] * s["mmax"], "xb": s["r"] * s["n"] * s["d"]},
    "dnb2_gen_gray": lambda s: {"C": s["r"] * s["d"] * s["mmax"], "xb": s["r"] * s["n"] * s["d"]},
    "dnb2_digital_shift": lambda s: {"lshifts": s["r_x"], "xb": s["r_x"] * s["n"] * s["d"],
                                     "shiftsb": s["r"] * s["d"], "xrb": s["r"] * s["n"] * s["d"]},
    "dnb2_integer_to_float": lambda s: {"tmaxes": s["r"], "xb": s["r"] * s["n"] * s["d"],
                                        "x": s["r"] * s["n"] * s["d"]},
    "dnb2_linear_matrix_scramble": lambda s: {"S": s["r"] * s["d"] * s["tmax_new"],
                                              "C": s["r_C"] * s["d"] * s["mmax"],
                                              "C_lms": s["r"] * s["d"] * s["mmax"]},
    "dnb2_interlace": lambda s: {"C": s["r"] * s["d"] * s["mmax"], "C_alpha": s["r"] * s["d_alpha"] * s["mmax"]},
    "dnb2_undo_interlace": lambda s: {"C_alpha": s["r"] * s["d_alpha"] * s["mmax"],
                                      "C": s["r"] * s["d"] * s["mmax"]},
    "dnb2_gmat_lsb_to_msb": lambda s: {"tmaxes": s["r"], "C_lsb": s["r"] * s["d"] * s["mmax"],
                                       "C_msb": s["r"] * s["d"] * s["mmax"]},
    "gdn_gen_natural": lambda s: {"bases": s["r_b"] * s["d"], "C": s["r"] * s["d"] * s["mmax"] * s["tmax"],
                                  "xdig": s["r"] * s["n"] * s["d"] * s["tmax"]},
    "gdn_gen_natural_same_base": lambda s: {"C": s["r"] * s["d"] * s["mmax"] * s["tmax"],
                                            "xdig": s["r"] * s["n"] * s["d"] * s["tmax"]},
    "gdn_linear_matrix_scramble": lambda s: {"bases": s["r_b"] * s["d"],
                                             "S": s["r"] * s["d"] * s["tmax_new"] * s["tmax"],
                                             "C": s["r_C"] * s["d"] * s["mmax"] * s["tmax"],
                                             "C_lms": s["r"] * s["d"] * s["mmax"] * s["tmax_new"]},
    "gdn_digital_permutation": lambda s: {"perms": s["r"] * s["d"] * s["tmax_new"] * s["bmax"],
                                          "xdig": s["r_x"] * s["n"] * s["d"] * s["tmax"],
                                          "xdig_new": s["r"] * s["n"] * s["d"] * s["tmax_new"]},
    "gdn_digital_shift": lambda s: {"bases": s["r_b"] * s["d"], "shifts": s["r"] * s["d"] * s["tmax_new"],
                                    "xdig": s["r_x"] * s["n"] * s["d"] * s["tmax"],
                                    "xdig_new": s["r"] * s["n"] * s["d"] * s["tmax_new"]},
    "gdn_integer_to_float": lambda s: {"bases": s["r_b"] * s["d"], "xdig": s["r"] * s["n"] * s["d"] * s["tmax"],
                                       "x": s["r"] * s["n"] * s["d"]},
    "gdn_interlace": lambda s: {"C": s["r"] * s["d"] * s["mmax"] * s["tmax"],
                                "C_alpha": s["r"] * s["d_alpha"] * s["mmax"] * s["tmax_alpha"]},
    "gdn_undo_interlace": lambda s: {"C_alpha": s["r"] * s["d_alpha"] * s["mmax"] * s["tmax_alpha"],
                                     "C": s["r"] * s["d"] * s["mmax"] * s["tmax"]},
    "fft_bro_1d_radix2": lambda s: {"twiddler": 2 * s["n_half"], "twiddlei": 2 * s["n_half"],
                                    "xr": s["d1"] * s["d2"] * 2 * s["n_half"],
                                    "xi": s["d1"] * s["d2"] * 2 * s["n_half"]},
    "ifft_bro_1d_radix2": lambda s: {"twiddler": 2 * s["n_half"], "twiddlei": 2 * s["n_half"],
                                     "xr": s["d1"] * s["d2"] * 2 * s["n_half"],
                                     "xi": s["d1"] * s["d2"] * 2 * s["n_half"]},
    "fwht_1d_radix2": lambda s: {"x": s["d1"] * s["d2"] * 2 * s["n_half"]},
}

# arrays the kernels only write: no host-to-device copy is needed for them
WRITE_ONLY = {"twiddler", "twiddlei"}
IN_PLACE = {"fft_bro_1d_radix2": {"xr", "xi"}, "ifft_bro_1d_radix2": {"xr", "xi"}, "fwht_1d_radix2": {"x"}}

_OPENCL_ONLY = ("global_size", "local_size", "context", "queue", "program", "platform_id", "device_id",
                "profile")


def _parse_kwargs(kwargs):
    # qmctoolscl/util.py:51-56: backend defaults to "c" and must be c or cl
    if "backend" in kwargs:
        kwargs["backend"] = kwargs["backend"].lower()
        assert kwargs["backend"] in ["cl", "c"]
    else:
        kwargs["backend"] = "c"


def _scalar(v, pos):
    if isinstance(v, (bool, np.bool_)) or isinstance(v, (float, np.floating)) or not hasattr(v, "__index__"):
        raise ctypes.ArgumentError("argument %d: TypeError: wrong type" % (pos + 1))
    return int(v) & 0xFFFFFFFFFFFFFFFF  # c_uint64 wraps like this


def _is_torch(a):
    # a torch tensor without importing torch for numpy-only callers
    return type(a).__module__.startswith("torch") and hasattr(a, "data_ptr")


def _check_numpy(a, kind, pos):
    want = np.uint64 if kind == "u64*" else np.float64
    if not isinstance(a, np.ndarray):
        raise ctypes.ArgumentError("argument %d: TypeError: argument must be an ndarray" % (pos + 1))
    if a.dtype != want:
        raise ctypes.ArgumentError("argument %d: TypeError: array must have data type %s"
                                   % (pos + 1, np.dtype(want).name))
    if not a.flags["C_CONTIGUOUS"]:
        raise ctypes.ArgumentError("argument %d: TypeError: array must have flags ['C_CONTIGUOUS']" % (pos + 1))


def _check_tensor(a, kind, pos, need, name):
    torch = _t()
    ok_dtypes = (torch.int64, torch.uint64) if kind == "u64*" else (torch.float64,)
    if a.dtype not in ok_dtypes:
        raise ctypes.ArgumentError("argument %d (%s): tensor must have dtype %s" % (pos + 1, name, ok_dtypes))
    if not a.is_cuda:
        raise ValueError("argument %d (%s): torch tensors must live on a CUDA device" % (pos + 1, name))
    if not a.is_contiguous():
        raise ctypes.ArgumentError("argument %d (%s): tensor must be contiguous" % (pos + 1, name))
    if a.numel() < need:
        raise ValueError("%s has %d elements, the call needs %d" % (name, a.numel(), need))


def _device_of(arrays, kwargs):
    torch = _t()
    for a in arrays:
        if _is_torch(a):
            return a.device
    if "device" in kwargs:
        return torch.device(kwargs["device"])
    if not torch.cuda.is_available():
        raise _ffi.QmcError("no CUDA device is available; qmctoolscl_gb300 runs only on the GPU")
    return torch.device("cuda", torch.cuda.current_device())


def _call(name, args, kwargs):
    spec, outs = SIGNATURES[name]
    if len(args) != len(spec):
        raise TypeError("%s() takes %d positional arguments but %d were given" % (name, len(spec), len(args)))
    _parse_kwargs(kwargs)
    t0_perf = time.perf_counter()
    t0_proc = time.process_time()
    # host-side checks first, in the order the reference meets them: ctypes
    # argument conversion, then the preprocess hook, then array sizes
    scalars, arrays = {}, {}
    for pos, ((an, kind), a) in enumerate(zip(spec, args)):
        if kind == "u64":
            scalars[an] = _scalar(a, pos)
        else:
            if not _is_torch(a):
                _check_numpy(a, kind, pos)
            arrays[an] = (pos, kind, a)
    pre = _PREPROCESS.get(name)
    if pre is not None:
        pre(scalars)
    need = NEED[name](scalars)
    for an, (pos, kind, a) in arrays.items():
        if not _is_torch(a) and a.size < need[an]:
            raise ValueError("%s has %d elements, the call needs %d" % (an, a.size, need[an]))
    lib = _ffi.lib()  # raises if the library is not built
    torch = _t()
    for an, (pos, kind, a) in arrays.items():
        if _is_torch(a):
            _check_tensor(a, kind, pos, need[an], an)
    dev = _device_of([a for (_p, _k, a) in arrays.values()], kwargs)
    stream = kwargs.get("stream")
    if stream is None:
        stream = torch.cuda.current_stream(dev)
    elif not hasattr(stream, "cuda_stream"):
        stream = torch.cuda.ExternalStream(int(stream), device=dev)
    handle = stream.cuda_stream
    wait = kwargs.get("wait", True)
    in_place = IN_PLACE.get(name, set())
    host_out = []  # (numpy flat view, device tensor)
    keep = []
    ptrs = {}
    any_host = False
    with torch.cuda.device(dev), torch.cuda.stream(stream):
        for an, (pos, kind, a) in arrays.items():
            cnt = need[an]
            if _is_torch(a):
                ptrs[an] = a.data_ptr()
                continue
            any_host = True
            tdt = torch.int64 if kind == "u64*" else torch.float64
            flat = a.reshape(-1)[:cnt]
            if an in outs and an not in in_place:
                dbuf = torch.empty(max(cnt, 1), dtype=tdt, device=dev)
            else:
                src = flat.view(np.int64) if kind == "u64*" else flat
                if not src.flags["WRITEABLE"]:
                    src = src.copy()
                dbuf = torch.from_numpy(src).to(dev) if cnt else torch.empty(1, dtype=tdt, device=dev)
            keep.append(dbuf)
            ptrs[an] = dbuf.data_ptr()
            if an in outs and cnt:
                host_out.append((flat, dbuf[:cnt]))
        cargs = [scalars[an] if kind == "u64" else ptrs[an] for an, kind in spec]
        fn = getattr(lib, "qmc_" + name)
        _ffi.check(fn(*cargs, handle), name)
        for flat, dbuf in host_out:
            dst = torch.from_numpy(flat.view(np.int64) if flat.dtype == np.uint64 else flat)
            dst.copy_(dbuf)
        if any_host or wait:
            _ffi.check(lib.qmc_device_error_check(handle), name)
            t_proc = time.process_time() - t0_proc
        else:
            t_proc = -1.0
    return time.perf_counter() - t0_perf, t_proc


def _pre_lat_gen_natural(s):
    # qmctoolscl/util.py:84-86
    n, n_start = s["n"], s["n_start"]
    if not ((n_start == 0 or np.log2(n_start) % 1 == 0) and ((n + n_start) == 0 or np.log2(n + n_start) % 1 == 0)):
        raise Exception("lat_gen_natural requires n_start and n+n_start are either 0 or powers of 2")


_PREPROCESS = {"lat_gen_natural": _pre_lat_gen_natural}

# One-line descriptions and argument meanings (our wording).
_DESC = {
    "lat_gen_linear": "Rank-1 lattice points in linear order, x[l,i,j] = frac(g[l,j]*i/n).",
    "lat_gen_natural": "Rank-1 lattice points in natural (van der Corput) order.",
    "lat_gen_gray": "Rank-1 lattice points in Gray-code order.",
    "lat_shift_mod_1": "Random shift modulo 1 of lattice points.",
    "dnb2_gen_natural": "Integer (binary) points of a base-2 digital net in natural order.",
    "dnb2_gen_gray": "Integer (binary) points of a base-2 digital net in Gray-code order.",
    "dnb2_digital_shift": "Digital (XOR) shift of base-2 digital net points, after a left shift.",
    "dnb2_integer_to_float": "Base-2 digital net integers to floats, x = xb * 2^-tmax.",
    "dnb2_linear_matrix_scramble": "Linear matrix scrambling of base-2 generating matrices over GF(2).",
    "dnb2_interlace": "Digit interlacing of base-2 generating matrices (higher-order nets).",
    "dnb2_undo_interlace": "Inverse of dnb2_interlace.",
    "dnb2_gmat_lsb_to_msb": "Base-2 generating matrices from least- to most-significant-bit-first columns.",
    "gdn_gen_natural": "Digits of a generalized digital net (one base per dimension, e.g. Halton), natural order.",
    "gdn_gen_natural_same_base": "Digits of a generalized digital net with one common base, natural order.",
    "gdn_linear_matrix_scramble": "Linear matrix scrambling of base-b generating matrices.",
    "gdn_digital_permutation": "Per-digit permutation scrambling of generalized digital net digits.",
    "gdn_digital_shift": "Digital shift (digit-wise addition mod b) of generalized digital net digits.",
    "gdn_integer_to_float": "Generalized digital net digits to floats.",
    "gdn_interlace": "Digit-row interlacing of base-b generating matrices.",
    "gdn_undo_interlace": "Inverse of gdn_interlace.",
    "fft_bro_1d_radix2": "Orthonormal FFT along the last axis of bit-reversed-order input (in place), "
                         "natural-order output; also fills the twiddle arrays.",
    "ifft_bro_1d_radix2": "Orthonormal inverse FFT along the last axis (in place), bit-reversed-order output; "
                          "also fills the twiddle arrays.",
    "fwht_1d_radix2": "Orthonormal fast Walsh-Hadamard transform along the last axis (in place).",
}

_ARGDOC = {
    "r": "randomisations (replications)", "n": "number of points", "d": "dimension",
    "n_start": "index of the first point in the sequence", "g": "generating vectors, r*d",
    "x": "points", "r_x": "randomisations present in the input", "shifts": "shifts",
    "xr": "shifted points", "mmax": "columns of each generating matrix", "C": "generating matrices",
    "xb": "integer points, r*n*d", "lshifts": "left shift applied per input randomisation",
    "shiftsb": "digital shifts, r*d", "xrb": "shifted integer points, r*n*d",
    "tmaxes": "bits per integer, one per randomisation", "r_C": "randomisations of C",
    "tmax_new": "bits (digits) after scrambling", "S": "scrambling matrices", "C_lms": "scrambled matrices",
    "d_alpha": "dimension after interlacing", "tmax": "bits (digits) of each column",
    "tmax_alpha": "bits (digits) after interlacing", "alpha": "interlacing factor",
    "C_alpha": "interlaced matrices", "C_lsb": "LSB-first matrices", "C_msb": "MSB-first matrices",
    "r_b": "randomisations of bases", "bases": "base of each dimension, r_b*d", "xdig": "digits",
    "b": "common base", "bmax": "permutation length (largest base)", "perms": "digit permutations",
    "xdig_new": "new digits", "d1": "first batch axis", "d2": "second batch axis",
    "n_half": "half the transform length (n = 2*n_half, a power of two)",
    "twiddler": "real twiddle factors (output, n)", "twiddlei": "imaginary twiddle factors (output, n)",
}


def _make(name):
    spec, _outs = SIGNATURES[name]

    def f(*args, **kwargs):
        return _call(name, args, kwargs)

    f.__name__ = name
    f.__qualname__ = name
    lines = []
    for an, kind in spec:
        typ = "np.uint64" if kind == "u64" else ("np.ndarray of np.uint64" if kind == "u64*"
                                                 else "np.ndarray of np.double")
        lines.append("%s (%s): %s" % (an, typ, _ARGDOC.get(an, an)))
    f.__doc__ = "%s\n\nArgs:\n    %s" % (_DESC[name], "\n    ".join(lines))
    return f


for _name in SIGNATURES:
    globals()[_name] = _make(_name)

__all__ = list(SIGNATURES)
