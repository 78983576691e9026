"""The C-ABI library: it builds for sm_103a, loads without a GPU, and exports
every entry point include/qmcgb.h declares (no compute calls here)."""
import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for fn in sorted(os.listdir(os.path.join(REPO, "include"))):
        if fn.endswith(".h"):
            with open(os.path.join(REPO, "include", fn)) as f:
                text = re.sub(r"/\*.*?\*/", "", f.read(), flags=re.S)
            names += re.findall(r"\b(qmc_\w+)\s*\(", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from qmctoolscl_gb300 import _build
    path = _build.build()
    return ctypes.CDLL(path)


def test_header_declares_all_reference_functions():
    from qmctoolscl_gb300._signatures import NAMES
    syms = declared_symbols()
    for name in NAMES:
        assert "qmc_" + name in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert missing == []


def test_library_reports_version_and_empty_error(lib):
    lib.qmc_version.restype = ctypes.c_int
    assert lib.qmc_version() >= 10000
    lib.qmc_last_error.restype = ctypes.c_char_p
    assert lib.qmc_last_error() == b""


def test_ffi_binds_all_entry_points(lib):
    from qmctoolscl_gb300 import _ffi
    L = _ffi.lib()
    for s in declared_symbols():
        getattr(L, s)


def test_argument_errors_need_no_gpu(lib):
    """Argument checks run on the host before any CUDA call."""
    from qmctoolscl_gb300 import _ffi
    L = _ffi.lib()
    # lat_gen_natural with n_start not a power of two: rejected before launch
    rc = L.qmc_lat_gen_natural(1, 3, 2, 3, None, None, None)
    assert rc == _ffi.QMC_ERR_ARG
    assert b"powers of 2" in L.qmc_last_error()
    # non-power-of-two transform length
    rc = L.qmc_fwht_1d_radix2(1, 1, 3, None, None)
    assert rc == _ffi.QMC_ERR_DOMAIN


def test_no_alloc_scratch_limit_holds_when_sizes_would_wrap(lib):
    """qmc_net_gen_noalloc bounds r*d*mmax factor by factor: sizes whose
    64-bit product wraps to 0 (r = 2^34, d = 2^30, mmax = 1) are refused on
    the host like any request above the fixed scratch, before any CUDA call
    and without touching the (fake) array pointers."""
    from qmctoolscl_gb300 import _ffi, batch
    L = _ffi.lib()
    L.qmc_net_gen_noalloc.argtypes = [ctypes.POINTER(batch.NetRequest), ctypes.c_void_p]
    L.qmc_net_gen_noalloc.restype = ctypes.c_int
    fake = 0x1000
    for r, d, alpha in ((1 << 34, 1 << 30, 1), (1, 1 << 63, 2)):
        req = batch.NetRequest(r=r, n=2, d=d, n_start=0, mmax=1, d_pre=(d * alpha) % (1 << 64), alpha=alpha, tmax=1,
                               tmax_new=1, tmax_alpha=1, r_C=1, gray=0, C=fake, S=fake, lshifts=None, shifts=None,
                               tmaxes=None, xb=fake, x=None)
        assert L.qmc_net_gen_noalloc(ctypes.byref(req), None) == _ffi.QMC_ERR_ARG
    assert b"131072" in L.qmc_last_error() or b"d_pre" in L.qmc_last_error()


def test_generalized_net_plan_argument_errors_need_no_gpu(lib):
    """qmc_halton_plan_create validates every dimension on the host, before
    any allocation; the array pointers are never dereferenced there."""
    from qmctoolscl_gb300 import _ffi, halton
    L = halton._lib()
    fake = ctypes.c_void_p(0x1000)
    x = ctypes.c_void_p(0x2000)

    def create(dims, r=1, n=8, n_start=0):
        arr = (halton.GdnDim * len(dims))(*dims)
        h = ctypes.c_void_p()
        rc = L.qmc_halton_plan_create(r, n, n_start, len(dims), arr, x, ctypes.byref(h))
        assert h.value is None
        return rc, L.qmc_last_error()

    def dim(b=3, tmax=4, mmax=3, **kw):
        args = dict(b=b, tmax=tmax, mmax=mmax, S=fake, C=fake, perms=fake, shifts=fake)
        args.update(kw)
        return halton.GdnDim(**args)

    assert create([dim(b=1)])[0] == _ffi.QMC_ERR_DOMAIN             # the reference never ends its digit loop
    assert create([dim(b=2048)])[0] == _ffi.QMC_ERR_ARG
    assert create([dim(tmax=0)])[0] == _ffi.QMC_ERR_ARG
    assert create([dim(mmax=65)])[0] == _ffi.QMC_ERR_ARG
    rc, msg = create([dim(b=2, mmax=2)], n=8)                       # index 7 has 3 binary digits
    assert rc == _ffi.QMC_ERR_ARG and b"digits" in msg
    rc, msg = create([dim(), dim(S=None)])                          # LMS for some dimensions only
    assert rc == _ffi.QMC_ERR_ARG and b"all dimensions" in msg
    assert create([dim()], n=1, n_start=(1 << 32))[0] == _ffi.QMC_ERR_ARG
    assert create([dim(C=None)])[0] == _ffi.QMC_ERR_ARG


def test_header_compiles_as_c_and_links(lib, tmp_path):
    """include/qmcgb.h is plain C (C99) and a C caller links libqmcgb.so and
    calls it (version, last error, an argument error), as a C integrator
    would -- no GPU needed."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "caller.c"
    src.write_text(
        '#include "qmcgb.h"\n'
        "#include <stdio.h>\n"
        "int main(void) {\n"
        "    if (qmc_version() < 10000) return 2;\n"
        "    int rc = qmc_fwht_1d_radix2(1, 1, 3, 0, 0);\n"
        "    if (rc != QMC_ERR_DOMAIN) return 3;\n"
        '    printf("%s\\n", qmc_last_error());\n'
        "    return 0;\n"
        "}\n")
    libdir = os.path.dirname(lib._name)
    exe = tmp_path / "caller"
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(REPO, "include"), str(src), "-L", libdir,
                    "-lqmcgb", "-Wl,-rpath," + libdir, "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out
    assert out.stdout.strip() != ""
