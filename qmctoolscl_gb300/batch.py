"""Fused pipelines beyond the reference's one-function-per-call surface.

lattice_gen_shift
    rank-1 lattice points in natural or Gray order followed by the mod-1
    shift, in one kernel that writes only the shifted points -- the result
    of lat_gen_{natural,gray} then lat_shift_mod_1 (r_x = r), bit for bit,
    with a third of the memory traffic and no intermediate array.
dnb2_gen_fused
    base-2 digital net generation followed by the digital shift and/or the
    integer-to-float conversion, in one kernel.

Arrays may be numpy arrays (copied to and from the GPU, as in the drop-in
API) or CUDA torch tensors (used in place, nothing copied).
"""
import numpy as np

from . import _ffi


def _t():
    import torch
    return torch


class _Args:
    """Collects device pointers for one call, copying numpy inputs in and
    remembering numpy outputs to copy back."""

    def __init__(self, stream=None, device=None, direct_out=True):
        torch = _t()
        self.torch = torch
        self.dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.stream = torch.cuda.current_stream(self.dev) if stream is None else stream
        self.keep, self.back = [], []
        self.h2d_bytes = self.d2h_bytes = 0
        self.direct_out = direct_out
        self.direct = False

    def ptr(self, a, dtype, count, out=False, name="array"):
        torch = self.torch
        if a is None:
            return None
        if isinstance(a, torch.Tensor):
            if not a.is_cuda or not a.is_contiguous() or a.numel() < count:
                raise ValueError("%s: need a contiguous CUDA tensor with at least %d elements" % (name, count))
            return a.data_ptr()
        a = np.asarray(a)
        if a.dtype != dtype or not a.flags["C_CONTIGUOUS"]:
            raise TypeError("%s must be a C-contiguous %s array" % (name, np.dtype(dtype).name))
        if a.size < count:
            raise ValueError("%s has %d elements, the call needs %d" % (name, a.size, count))
        flat = a.reshape(-1)[:count]
        tdt = torch.int64 if dtype == np.uint64 else torch.float64
        if out and self.direct_out and count:
            # pinned host output: the kernel writes it directly over the
            # CPU-GPU link, no staging buffer and no separate copy
            dptr = _ffi.device_pointer_of_host(flat.ctypes.data)
            if dptr is not None:
                self.direct = True
                self.d2h_bytes += flat.nbytes
                return dptr
        if out:
            d = torch.empty(max(count, 1), dtype=tdt, device=self.dev)
            self.back.append((flat, d[:count]))
            self.d2h_bytes += flat.nbytes
        else:
            src = flat.view(np.int64) if dtype == np.uint64 else flat
            d = torch.from_numpy(_ffi.writable(np.ascontiguousarray(src))).to(self.dev, non_blocking=True)
            self.h2d_bytes += flat.nbytes
        self.keep.append(d)
        return d.data_ptr()

    def finish(self):
        torch = self.torch
        for flat, d in self.back:
            dst = torch.from_numpy(flat.view(np.int64) if flat.dtype == np.uint64 else flat)
            dst.copy_(d, non_blocking=False)
        if self.direct:
            self.stream.synchronize()  # results written straight to host memory


def lattice_gen_shift(r, n, d, n_start, g, shifts, xr, order="gray", stream=None, direct_out=True):
    """xr[l,i,j] = fmod(lattice point (l,i,j) + shifts[l,j], 1), points in
    natural or Gray order from generating vectors g (r*d); equals
    lat_gen_<order>(r,n,d,n_start,g,x) then lat_shift_mod_1(r,n,d,r,x,shifts,xr).

    With direct_out (default) a pinned numpy output (e.g. from
    qmctoolscl_gb300.batch.pinned_empty) is written by the kernel in place over
    the CPU-GPU link; other numpy outputs are staged in device memory and
    copied back."""
    torch = _t()
    r, n, d, n_start = int(r), int(n), int(d), int(n_start)
    if order not in ("gray", "natural"):
        raise ValueError("order must be 'gray' or 'natural'")
    A = _Args(stream, direct_out=direct_out)
    with torch.cuda.stream(A.stream):
        pg = A.ptr(g, np.uint64, r * d, name="g")
        ps = A.ptr(shifts, np.float64, r * d, name="shifts")
        px = A.ptr(xr, np.float64, r * n * d, out=True, name="xr")
        rc = _ffi.lib().qmc_lat_gen_shift(r, n, d, n_start, 1 if order == "gray" else 0, pg, ps, px,
                                          A.stream.cuda_stream)
        _ffi.check(rc, "lattice_gen_shift")
        A.finish()
    return A


def pinned_empty(shape, dtype=np.float64):
    """A numpy array in pinned (page-locked) host memory, which kernels can
    write directly and copies reach at full link speed."""
    torch = _t()
    tdt = {np.dtype(np.float64): torch.float64, np.dtype(np.uint64): torch.int64}[np.dtype(dtype)]
    a = torch.empty(shape, dtype=tdt, pin_memory=True).numpy()  # the array keeps the tensor alive
    return a.view(np.uint64) if np.dtype(dtype) == np.uint64 else a


def dnb2_gen_fused(r, n, d, n_start, mmax, C, r_C=None, order="natural", lshifts=None, r_x=None, shiftsb=None,
                   tmaxes=None, xrb=None, x=None, stream=None):
    """Digital net generation (natural or Gray order), then the digital shift
    (when shiftsb is given: (point << lshifts[l % r_x]) ^ shiftsb[l,j]), then
    the conversion ldexp(value, -tmaxes[l]) (when x is given).  xrb receives
    the integers (optional when x is given)."""
    torch = _t()
    r, n, d, n_start, mmax = int(r), int(n), int(d), int(n_start), int(mmax)
    r_C = r if r_C is None else int(r_C)
    r_x = r if r_x is None else int(r_x)
    A = _Args(stream)
    with torch.cuda.stream(A.stream):
        pC = A.ptr(C, np.uint64, r_C * d * mmax, name="C")
        pl = A.ptr(lshifts, np.uint64, r_x, name="lshifts")
        ps = A.ptr(shiftsb, np.uint64, r * d, name="shiftsb")
        pt = A.ptr(tmaxes, np.uint64, r, name="tmaxes")
        pxb = A.ptr(xrb, np.uint64, r * n * d, out=True, name="xrb")
        px = A.ptr(x, np.float64, r * n * d, out=True, name="x")
        rc = _ffi.lib().qmc_dnb2_gen_fused(r, n, d, n_start, mmax, pC, r_C, 1 if order == "gray" else 0, pl, r_x,
                                           ps, pt, pxb, px, A.stream.cuda_stream)
        _ffi.check(rc, "dnb2_gen_fused")
        A.finish()
    return A


# --------------------------------------------------------------------------
# batched plans: many requests of uneven size, one persistent launch

import ctypes as _ct
import json as _json
import os as _os
import threading as _threading

_U64, _I32, _P = _ct.c_uint64, _ct.c_int32, _ct.c_void_p


class NetRequest(_ct.Structure):
    """qmc_net_request (include/qmcgb.h): LMS -> interlace -> generation ->
    digital shift -> float, per request, r randomisations each."""
    _fields_ = [("r", _U64), ("n", _U64), ("d", _U64), ("n_start", _U64), ("mmax", _U64), ("d_pre", _U64),
                ("alpha", _U64), ("tmax", _U64), ("tmax_new", _U64), ("tmax_alpha", _U64), ("r_C", _U64),
                ("gray", _I32), ("reserved", _I32), ("C", _P), ("S", _P), ("lshifts", _P), ("shifts", _P),
                ("tmaxes", _P), ("xb", _P), ("x", _P)]


class LatRequest(_ct.Structure):
    """qmc_lat_request (include/qmcgb.h): lattice generation -> shift mod 1."""
    _fields_ = [("r", _U64), ("n", _U64), ("d", _U64), ("n_start", _U64), ("gray", _I32), ("reserved", _I32),
                ("g", _P), ("shifts", _P), ("x", _P)]


def _plan_lib():
    L = _ffi.lib()
    if not getattr(L, "_plan_bound", False):
        L.qmc_net_plan_create.argtypes = [_ct.POINTER(NetRequest), _ct.c_int, _ct.POINTER(_P)]
        L.qmc_lat_plan_create.argtypes = [_ct.POINTER(LatRequest), _ct.c_int, _ct.POINTER(_P)]
        for fn in ("qmc_net_plan_create", "qmc_lat_plan_create", "qmc_plan_run", "qmc_plan_graph_launch",
                   "qmc_plan_set_tuning", "qmc_plan_info", "qmc_plan_destroy"):
            getattr(L, fn).restype = _ct.c_int
        L.qmc_plan_run.argtypes = [_P, _P]
        L.qmc_plan_graph_launch.argtypes = [_P, _P]
        L.qmc_plan_set_tuning.argtypes = [_P, _ct.c_int, _ct.c_int, _U64]
        L.qmc_plan_info.argtypes = [_P, _ct.POINTER(_U64), _ct.POINTER(_U64), _ct.POINTER(_U64),
                                    _ct.POINTER(_ct.c_int)]
        L.qmc_plan_destroy.argtypes = [_P]
        L._plan_bound = True
    return L


def _dptr(t):
    return None if t is None else t.data_ptr()


def _need(q, key, count, dtypes, optional=True):
    """Check that request field `key` is a contiguous CUDA tensor of one of
    `dtypes` with at least `count` elements (kernels get raw pointers and
    would otherwise read or write past it)."""
    t = q.get(key)
    if t is None:
        if optional:
            return
        raise ValueError("request field %s is required" % key)
    torch = _t()
    if not isinstance(t, torch.Tensor) or not t.is_cuda or not t.is_contiguous():
        raise TypeError("request field %s must be a contiguous CUDA tensor" % key)
    if t.dtype not in dtypes:
        raise TypeError("request field %s has dtype %s" % (key, t.dtype))
    if t.numel() < count:
        raise ValueError("request field %s has %d elements, needs %d" % (key, t.numel(), count))


class Plan:
    """A batched plan over device tensors (see NetPlan / LatPlan).

    run(stream)          -- launch (net plans: matrix preparation + generation;
                            lattice plans: generation), asynchronous
    graph_launch(stream) -- the same from a CUDA graph captured at the first call
                            (stream must not be the default stream)
    tune()               -- pick the launch shape with the autotuner
    The tensors the requests refer to are kept alive by the plan; their
    contents may change between runs, their storage may not."""

    kind = None

    def __init__(self, structs, keep):
        L = _plan_lib()
        arr = (self.struct_type * max(len(structs), 1))(*structs)
        h = _P()
        create = L.qmc_net_plan_create if self.kind == "net" else L.qmc_lat_plan_create
        _ffi.check(create(arr, len(structs), _ct.byref(h)), "plan_create")
        self._h = h
        self._keep = keep
        self.nreq = len(structs)
        self.tuning = None

    def run(self, stream=None):
        s = stream if stream is not None else _t().cuda.current_stream()
        _ffi.check(_plan_lib().qmc_plan_run(self._h, s.cuda_stream), "plan_run")

    def graph_launch(self, stream):
        _ffi.check(_plan_lib().qmc_plan_graph_launch(self._h, stream.cuda_stream), "plan_graph_launch")

    def set_tuning(self, ctas_per_sm=0, chunk=0, tile_coords=0):
        _ffi.check(_plan_lib().qmc_plan_set_tuning(self._h, int(ctas_per_sm), int(chunk), int(tile_coords)),
                   "plan_set_tuning")
        self.tuning = (ctas_per_sm, chunk, tile_coords)

    def info(self):
        t, c, b, l_ = _U64(), _U64(), _U64(), _ct.c_int()
        _ffi.check(_plan_lib().qmc_plan_info(self._h, _ct.byref(t), _ct.byref(c), _ct.byref(b), _ct.byref(l_)),
                   "plan_info")
        return {"tiles": t.value, "coords": c.value, "bytes_out": b.value, "launches": l_.value}

    def shape_class(self):
        inf = self.info()
        coords = max(inf["coords"], 1)
        mean_d = coords / max(sum(self._rows), 1)
        return "%s|coords2^%d|d2^%d|req2^%d|%s" % (self.kind, int(np.log2(coords)), int(np.log2(max(mean_d, 1))),
                                                  int(np.log2(max(self.nreq, 1))), _device_name())

    def tune(self, stream=None, reps=3, use_cache=True):
        return autotune(self, stream=stream, reps=reps, use_cache=use_cache)

    def close(self):
        if getattr(self, "_h", None):
            _plan_lib().qmc_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class NetPlan(Plan):
    """Digital-net plan.  Each request is a dict with the fields of
    NetRequest; arrays are CUDA tensors (int64/uint64 for integer arrays,
    float64 for x).  Missing optional arrays (S, shifts, lshifts, tmaxes, xb,
    x) are None."""
    kind = "net"
    struct_type = NetRequest

    def __init__(self, requests):
        torch = _t()
        ints, flts = (torch.int64, torch.uint64), (torch.float64,)
        structs, keep, self._rows = [], [], []
        for q in requests:
            q = dict(q)
            alpha = int(q.get("alpha", 1))
            d = int(q["d"])
            r, n, mmax = int(q["r"]), int(q["n"]), int(q["mmax"])
            d_pre = int(q.get("d_pre", d * alpha))
            _need(q, "C", int(q.get("r_C", 1)) * d_pre * mmax, ints, optional=False)
            _need(q, "S", r * d_pre * int(q.get("tmax_new", q.get("tmax", 64))), ints)
            _need(q, "shifts", r * d, ints)
            _need(q, "lshifts", r if q.get("shifts") is not None else 0, ints)
            _need(q, "tmaxes", r if q.get("x") is not None else 0, ints)
            _need(q, "xb", r * n * d, ints)
            _need(q, "x", r * n * d, flts)
            st = NetRequest(r=int(q["r"]), n=int(q["n"]), d=d, n_start=int(q.get("n_start", 0)),
                            mmax=int(q["mmax"]), d_pre=int(q.get("d_pre", d * alpha)), alpha=alpha,
                            tmax=int(q.get("tmax", 64)), tmax_new=int(q.get("tmax_new", q.get("tmax", 64))),
                            tmax_alpha=int(q.get("tmax_alpha", min(alpha * int(q.get("tmax_new", q.get("tmax", 64))),
                                                                   64))),
                            r_C=int(q.get("r_C", 1)), gray=1 if q.get("order", "natural") == "gray" else 0,
                            C=_dptr(q["C"]), S=_dptr(q.get("S")), lshifts=_dptr(q.get("lshifts")),
                            shifts=_dptr(q.get("shifts")), tmaxes=_dptr(q.get("tmaxes")), xb=_dptr(q.get("xb")),
                            x=_dptr(q.get("x")))
            structs.append(st)
            keep.append(q)
            self._rows.append(int(q["r"]) * int(q["n"]))
        super().__init__(structs, keep)


class LatPlan(Plan):
    """Rank-1 lattice plan.  Each request: dict(r, n, d, n_start=0,
    order='gray'|'natural', g=<r*d int tensor>, shifts=<r*d float tensor or
    None>, x=<r*n*d float tensor>)."""
    kind = "lat"
    struct_type = LatRequest

    def __init__(self, requests):
        torch = _t()
        structs, keep, self._rows = [], [], []
        for q in requests:
            q = dict(q)
            r, n, d = int(q["r"]), int(q["n"]), int(q["d"])
            _need(q, "g", r * d, (torch.int64, torch.uint64), optional=False)
            _need(q, "shifts", r * d, (torch.float64,))
            _need(q, "x", r * n * d, (torch.float64,), optional=False)
            st = LatRequest(r=int(q["r"]), n=int(q["n"]), d=int(q["d"]), n_start=int(q.get("n_start", 0)),
                            gray=1 if q.get("order", "gray") == "gray" else 0, g=_dptr(q["g"]),
                            shifts=_dptr(q.get("shifts")), x=_dptr(q["x"]))
            structs.append(st)
            keep.append(q)
            self._rows.append(int(q["r"]) * int(q["n"]))
        super().__init__(structs, keep)


# --------------------------------------------------------------------------
# autotuner: launch shapes of the persistent kernel, cached per shape class

TUNE_CTAS = (2, 4, 8)
TUNE_CHUNK = (1, 4, 16)
TUNE_TILE = (1 << 14, 1 << 16, 1 << 18)
_cache_lock = _threading.Lock()


def _device_name():
    torch = _t()
    return torch.cuda.get_device_name().replace(" ", "_") if torch.cuda.is_available() else "nogpu"


def _cache_path():
    return _os.environ.get("QMCGB_TUNE_CACHE",
                           _os.path.join(_os.path.expanduser("~"), ".cache", "qmctoolscl_gb300", "autotune.json"))


def _load_cache():
    try:
        with open(_cache_path()) as f:
            return _json.load(f)
    except (OSError, ValueError):
        return {}


def _store_cache(key, value):
    with _cache_lock:
        c = _load_cache()
        c[key] = value
        path = _cache_path()
        try:
            _os.makedirs(_os.path.dirname(path), exist_ok=True)
            tmp = path + ".tmp%d" % _os.getpid()
            with open(tmp, "w") as f:
                _json.dump(c, f, indent=1)
            _os.replace(tmp, path)
        except OSError:
            pass


def time_plan(plan, stream, reps):
    """Average milliseconds of one plan run, CUDA events on `stream`."""
    torch = _t()
    with torch.cuda.stream(stream):
        plan.run(stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            plan.run(stream)
        e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def autotune(plan, stream=None, reps=3, use_cache=True):
    """Try every (CTAs per SM, tiles per grab, coordinates per tile) of the
    candidate grid on this plan, keep the fastest, and remember it for plans
    of the same shape class.  Returns (ctas_per_sm, chunk, tile_coords, ms)."""
    torch = _t()
    stream = stream if stream is not None else torch.cuda.current_stream()
    key = plan.shape_class()
    if use_cache:
        hit = _load_cache().get(key)
        if hit:
            plan.set_tuning(*hit[:3])
            return tuple(hit)
    best = None
    for tile in TUNE_TILE:
        for ctas in TUNE_CTAS:
            for chunk in TUNE_CHUNK:
                plan.set_tuning(ctas, chunk, tile)
                ms = time_plan(plan, stream, reps)
                if best is None or ms < best[3]:
                    best = (ctas, chunk, tile, ms)
    plan.set_tuning(*best[:3])
    if use_cache:
        _store_cache(key, list(best))
    return best
