"""Parity oracle for the QMCToolsCL hot path.

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker, and by bench.py for its CPU-baseline leg.  The product package
(qmctoolscl_gb300) never imports this module.

Two CPU implementations live here:

* ``liboracle.so`` -- qmc_oracle.c, our C restatement of the reference C
  backend (each function cites the reference file:line it follows).  Built by
  ``make -C oracle``; it builds on any host with gcc (x86-64 or aarch64).
* ``_ref/c_lib.so`` -- the reference's own C sources compiled where they lie
  (``make -C oracle ref``); only available where the reference checkout is.
  Used to pin the restatement and to make the golden fixtures.

Both are called with numpy arrays in the reference's argument order (without
the batch-size arguments): ``oracle.call("lat_gen_gray", r, n, d, n_start,
g, x)``.
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

from qmctoolscl_gb300._signatures import SIGNATURES

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "c_lib.so")

_lock = threading.Lock()
_libs = {}


def build(ref=False, ref_dir=None):
    """Compile the oracle (and, with ref=True, the reference C backend from the
    QMCToolsCL checkout at ref_dir, or at $QMCTOOLSCL_REF when ref_dir is None)."""
    extra = ["ref"] if ref else []
    if ref and ref_dir:
        extra.append("REF_DIR=%s" % ref_dir)
    subprocess.run(["make", "-s", "-C", HERE] + extra, check=True)


def _argtype(kind):
    if kind == "u64":
        return ctypes.c_uint64
    if kind == "u64*":
        return np.ctypeslib.ndpointer(ctypes.c_uint64, flags="C_CONTIGUOUS")
    return np.ctypeslib.ndpointer(ctypes.c_double, flags="C_CONTIGUOUS")


def _load(path, prefix, with_bs):
    lib = ctypes.CDLL(path)
    funcs = {}
    for name, (args, _outs) in SIGNATURES.items():
        fn = getattr(lib, prefix + name)
        types = [_argtype(k) for _a, k in args]
        if with_bs:  # the reference repeats the three leading extents as batch sizes
            types = types[:3] + [ctypes.c_uint64] * 3 + types[3:]
        fn.argtypes = types
        fn.restype = None
        funcs[name] = fn
    return funcs


def oracle_lib():
    with _lock:
        if "oracle" not in _libs:
            if not os.path.exists(ORACLE_SO):
                build()
            _libs["oracle"] = _load(ORACLE_SO, "oracle_", with_bs=False)
        return _libs["oracle"]


def ref_available():
    return os.path.exists(REF_SO)


def ref_lib():
    with _lock:
        if "ref" not in _libs:
            _libs["ref"] = _load(REF_SO, "", with_bs=True)
        return _libs["ref"]


def call(name, *args):
    """Run the oracle restatement of ``name`` in place on numpy arrays."""
    oracle_lib()[name](*args)


def call_ref(name, *args):
    """Run the compiled reference C function ``name`` (bs_* set to the extents)."""
    a = list(args)
    ref_lib()[name](*(a[:3] + a[:3] + a[3:]))


_QRNG_ARGTYPES = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                  np.ctypeslib.ndpointer(ctypes.c_double, flags="C_CONTIGUOUS"),
                  np.ctypeslib.ndpointer(ctypes.c_double, flags="C_CONTIGUOUS"),
                  np.ctypeslib.ndpointer(ctypes.c_int, flags="C_CONTIGUOUS")]


def _qrng(path, symbol):
    fn = getattr(ctypes.CDLL(path), symbol)
    fn.argtypes = _QRNG_ARGTYPES
    fn.restype = None
    return fn


def halton_qrng(n, d, n0, generalized, res, randu_d_32, dvec):
    """The oracle restatement of halton_qrng (qmctoolscl/c_funcs/halton_qrng.c:3-162):
    res (d x n) filled in place."""
    if not os.path.exists(ORACLE_SO):
        build()
    _qrng(ORACLE_SO, "oracle_halton_qrng")(n, d, n0, generalized, res, randu_d_32, dvec)


def halton_qrng_ref(n, d, n0, generalized, res, randu_d_32, dvec):
    """The reference's own compiled halton_qrng (where oracle/_ref is built)."""
    _qrng(REF_SO, "halton_qrng")(n, d, n0, generalized, res, randu_d_32, dvec)


_U64P = np.ctypeslib.ndpointer(ctypes.c_uint64, flags="C_CONTIGUOUS")


def _nus_lib():
    if not os.path.exists(ORACLE_SO):
        build()
    lib = ctypes.CDLL(ORACLE_SO)
    lib.oracle_nus_forest_new.argtypes = [ctypes.c_uint64]
    lib.oracle_nus_forest_new.restype = ctypes.c_void_p
    lib.oracle_nus_forest_free.argtypes = [ctypes.c_void_p]
    lib.oracle_nus_forest_free.restype = None
    lib.oracle_dnb2_nested_uniform_scramble.argtypes = [ctypes.c_uint64] * 6 + [_U64P, ctypes.c_void_p, _U64P, _U64P]
    lib.oracle_dnb2_nested_uniform_scramble.restype = None
    return lib


class NusForest:
    """The oracle restatement of dnb2_nested_uniform_scramble
    (qmctoolscl/rand_funcs.py:155-253): r*d scrambling trees kept between
    calls, as the reference keeps its root nodes.  ``states`` holds six words
    per generator (a, b, c, w, has_uint32, uinteger of numpy's SFC64) and is
    advanced in place."""

    def __init__(self, ntrees):
        self._lib = _nus_lib()
        self._h = self._lib.oracle_nus_forest_new(ntrees)

    def scramble(self, r, n, d, r_x, tmax, tmax_new, states, xb, xrb):
        self._lib.oracle_dnb2_nested_uniform_scramble(r, n, d, r_x, tmax, tmax_new, states, self._h,
                                                      np.ascontiguousarray(xb, dtype=np.uint64), xrb)

    def close(self):
        if self._h:
            self._lib.oracle_nus_forest_free(self._h)
            self._h = None

    def __del__(self):
        self.close()


def _gdn_nus_lib():
    lib = _nus_lib()
    lib.oracle_gdn_forest_new.argtypes = [ctypes.c_uint64]
    lib.oracle_gdn_forest_new.restype = ctypes.c_void_p
    lib.oracle_gdn_forest_free.argtypes = [ctypes.c_void_p]
    lib.oracle_gdn_forest_free.restype = None
    lib.oracle_gdn_nested_uniform_scramble.argtypes = [ctypes.c_uint64] * 7 + [_U64P, ctypes.c_void_p, _U64P, _U64P,
                                                                               _U64P]
    lib.oracle_gdn_nested_uniform_scramble.restype = ctypes.c_int
    return lib


class GdnNusForest:
    """The oracle restatement of gdn_nested_uniform_scramble
    (qmctoolscl/rand_funcs.py:262-356): r*d base-b scrambling trees kept
    between calls.  ``states`` as for NusForest.  ``scramble`` returns 0, or 1
    where the reference raises IndexError (a digit at or above its base; a
    walk that runs out of digits, which happens for tmax_new = tmax)."""

    def __init__(self, ntrees):
        self._lib = _gdn_nus_lib()
        self._h = self._lib.oracle_gdn_forest_new(ntrees)

    def scramble(self, r, n, d, r_x, r_b, tmax, tmax_new, states, bases, xdig, xrdig):
        return self._lib.oracle_gdn_nested_uniform_scramble(
            r, n, d, r_x, r_b, tmax, tmax_new, states, self._h, np.ascontiguousarray(bases, dtype=np.uint64),
            np.ascontiguousarray(xdig, dtype=np.uint64), xrdig)

    def close(self):
        if self._h:
            self._lib.oracle_gdn_forest_free(self._h)
            self._h = None

    def __del__(self):
        self.close()
