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

    def __init__(self, stream=None, device=None):
        torch = _t()
        self.torch = torch
        self.dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.stream = torch.cuda.current_stream(self.dev) if stream is None else stream
        self.keep, self.back = [], []
        self.h2d_bytes = self.d2h_bytes = 0

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
        if out:
            d = torch.empty(max(count, 1), dtype=tdt, device=self.dev)
            self.back.append((flat, d[:count]))
            self.d2h_bytes += flat.nbytes
        else:
            src = flat.view(np.int64) if dtype == np.uint64 else flat
            d = torch.from_numpy(np.ascontiguousarray(src)).to(self.dev, non_blocking=True)
            self.h2d_bytes += flat.nbytes
        self.keep.append(d)
        return d.data_ptr()

    def finish(self):
        torch = self.torch
        for flat, d in self.back:
            dst = torch.from_numpy(flat.view(np.int64) if flat.dtype == np.uint64 else flat)
            dst.copy_(d, non_blocking=False)


def lattice_gen_shift(r, n, d, n_start, g, shifts, xr, order="gray", stream=None):
    """xr[l,i,j] = fmod(lattice point (l,i,j) + shifts[l,j], 1), points in
    natural or Gray order from generating vectors g (r*d); equals
    lat_gen_<order>(r,n,d,n_start,g,x) then lat_shift_mod_1(r,n,d,r,x,shifts,xr)."""
    torch = _t()
    r, n, d, n_start = int(r), int(n), int(d), int(n_start)
    if order not in ("gray", "natural"):
        raise ValueError("order must be 'gray' or 'natural'")
    A = _Args(stream)
    with torch.cuda.stream(A.stream):
        pg = A.ptr(g, np.uint64, r * d, name="g")
        ps = A.ptr(shifts, np.float64, r * d, name="shifts")
        px = A.ptr(xr, np.float64, r * n * d, out=True, name="xr")
        rc = _ffi.lib().qmc_lat_gen_shift(r, n, d, n_start, 1 if order == "gray" else 0, pg, ps, px,
                                          A.stream.cuda_stream)
        _ffi.check(rc, "lattice_gen_shift")
        A.finish()
    return A


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
