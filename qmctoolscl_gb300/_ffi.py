"""ctypes binding of libqmcgb.so (declarations in include/qmcgb.h).

The library is the only compute path: if it is missing or cannot be loaded,
every call raises.  There is no CPU fallback.
"""
import ctypes
import os
import threading

from ._signatures import SIGNATURES

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libqmcgb.so")

QMC_OK, QMC_ERR_ARG, QMC_ERR_DOMAIN, QMC_ERR_CUDA, QMC_ERR_DEVICE = 0, -1, -2, -3, -4

_lock = threading.Lock()
_lib = None

U64 = ctypes.c_uint64
PTR = ctypes.c_void_p
INT = ctypes.c_int

# extra entry points beyond the 23 reference functions: name -> argtypes
EXTRA = {
    "qmc_lat_gen_shift": [U64, U64, U64, U64, INT, PTR, PTR, PTR, PTR],
    "qmc_dnb2_gen_fused": [U64, U64, U64, U64, U64, PTR, U64, INT, PTR, U64, PTR, PTR, PTR, PTR, PTR],
    "qmc_tc_fft_bro_1d": [U64, U64, U64, PTR, PTR, PTR],
    "qmc_tc_ifft_bro_1d": [U64, U64, U64, PTR, PTR, PTR],
    "qmc_tc_fwht_1d": [U64, U64, U64, PTR, PTR],
    "qmc_tc_fft_mul_ifft": [U64, U64, U64, PTR, PTR, U64, INT, ctypes.c_double, PTR, PTR, PTR],
    "qmc_tc_fwht_mul_fwht": [U64, U64, U64, PTR, U64, INT, ctypes.c_double, PTR, PTR],
    "qmc_fft_mul_ifft": [U64, U64, U64, PTR, PTR, PTR, PTR, U64, INT, ctypes.c_double, PTR, PTR, PTR],
    "qmc_fwht_mul_fwht": [U64, U64, U64, PTR, U64, INT, ctypes.c_double, PTR, PTR],
    "qmc_halton_qrng": [INT, INT, INT, INT, PTR, PTR, PTR, PTR],
    "qmc_dnb2_nus_workspace_size": [U64, U64, U64, PTR],
    "qmc_dnb2_nested_uniform_scramble": [U64] * 6 + [PTR, U64, PTR, PTR, PTR, PTR, PTR, PTR, PTR, U64, PTR],
    "qmc_lat_get_shifts": [PTR, U64, U64, PTR, PTR],
    "qmc_random_tbit_uint64s": [PTR, U64, U64, PTR, PTR],
    "qmc_dnb2_get_digital_shifts": [PTR, U64, U64, U64, PTR, PTR],
    "qmc_dnb2_get_linear_scramble_matrix": [PTR, U64, U64, U64, U64, PTR, PTR],
    "qmc_gdn_get_linear_scramble_matrix": [PTR, U64, U64, U64, U64, U64, PTR, PTR, PTR],
    "qmc_gdn_get_digital_shifts": [PTR, U64, U64, U64, U64, PTR, PTR, PTR],
    "qmc_gdn_get_digital_permutations": [PTR, U64, U64, U64, U64, PTR, U64, PTR, PTR],
    "qmc_random_uint64_permutations": [PTR, U64, U64, PTR, PTR],
    "qmc_gdn_nus_workspace_size": [U64, U64, U64, PTR],
    "qmc_gdn_nested_uniform_scramble": [U64] * 7 + [PTR, PTR, U64, PTR, PTR, PTR, PTR, PTR, PTR, PTR, U64, PTR,
                                                     PTR, PTR, U64, PTR],
}


class LibraryMissing(RuntimeError):
    pass


def lib():
    """Load libqmcgb.so once; raise if it is not built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise LibraryMissing(
                "libqmcgb.so is not built (expected at %s); run "
                "`python -m qmctoolscl_gb300._build` or __graft_entry__.build()" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (args, _outs) in SIGNATURES.items():
            fn = getattr(L, "qmc_" + name)
            fn.argtypes = [U64 if k == "u64" else PTR for _a, k in args] + [PTR]
            fn.restype = INT
        for name, types in EXTRA.items():
            fn = getattr(L, name)
            fn.argtypes = types
            fn.restype = INT
        L.qmc_last_error.restype = ctypes.c_char_p
        L.qmc_last_error.argtypes = []
        L.qmc_version.restype = INT
        L.qmc_device_error_check.argtypes = [PTR]
        L.qmc_device_error_check.restype = INT
        L.qmc_device_error_reset.argtypes = [PTR]
        L.qmc_device_error_reset.restype = INT
        L.qmc_host_pointer_for_device.argtypes = [PTR, ctypes.POINTER(ctypes.c_void_p)]
        L.qmc_host_pointer_for_device.restype = INT
        L.qmc_device_attributes.argtypes = [ctypes.POINTER(INT)] * 3
        L.qmc_device_attributes.restype = INT
        _lib = L
        return _lib


def last_error():
    return lib().qmc_last_error().decode(errors="replace")


def device_pointer_of_host(ptr):
    """Device address of pinned host memory at ptr, or None if it is not pinned."""
    out = ctypes.c_void_p()
    if lib().qmc_host_pointer_for_device(ctypes.c_void_p(ptr), ctypes.byref(out)) == QMC_OK:
        return out.value
    return None


def device_attributes():
    a, b, c = INT(), INT(), INT()
    check(lib().qmc_device_attributes(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)), "device_attributes")
    return {"pageable_access": a.value, "uses_host_page_tables": b.value, "sms": c.value}


def writable(a):
    """`a` itself when numpy marks it writeable, else a copy of it:
    torch.from_numpy takes writeable arrays only (a read-only array would be
    shared with a tensor that claims it may write)."""
    return a if a.flags["WRITEABLE"] else a.copy()


class QmcError(RuntimeError):
    """A CUDA-side failure reported by libqmcgb."""


def check(rc, what):
    if rc == QMC_OK:
        return
    msg = "%s: %s" % (what, last_error())
    if rc in (QMC_ERR_ARG, QMC_ERR_DOMAIN):
        raise ValueError(msg)
    raise QmcError(msg)
