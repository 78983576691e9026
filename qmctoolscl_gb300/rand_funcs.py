"""Host-side generators of randomisation inputs (shifts, scrambling matrices,
permutations), part of the QMCToolsCL call surface (qmctoolscl/rand_funcs.py:4-153).

These produce the inputs that the GPU kernels consume.  Their outputs are
defined by numpy's random streams, so each helper draws from the Generator
with the same calls, shapes, bounds and dtypes, in the same order, as the
reference helper of the same name: given a Generator in the same state they
return identical arrays (checked against fixtures recorded from the
reference).  The nested-uniform-scrambling routines of the reference
(rand_funcs.py:155-356) run on the GPU and live in nus.py.

On the GPU.  Every helper that draws takes the keyword ``device`` (a torch
device, "cuda" or a device index): the same draws then run on the GPU, bit for
bit (libqmcgb's qmc_<helper> entry points), and the helper returns a CUDA
tensor of the same shape -- float64 for lat_get_shifts, the uint64 bits as
int64 otherwise -- instead of a numpy array.  The Generator must sit on an
SFC64 bit generator (the reference's own family); its state is read before
and set after the call, exactly as numpy would leave it.  For a sequence of
calls, wrap the Generator in a ``DeviceGenerator``: its state then stays on
the GPU between calls (no host round trip per call) and goes back to the
Generator at ``sync()``.  Domain of the GPU form: permutations of at most
65536 entries; otherwise as numpy (the same exception types for the inputs
numpy refuses, raised before any draw).
"""
import numpy as np

__all__ = ["random_tbit_uint64s", "random_uint64_permutations", "lat_get_shifts", "dnb2_get_digital_shifts",
           "dnb2_get_linear_scramble_matrix", "gdn_get_linear_scramble_matrix", "gdn_get_halton_generating_matrix",
           "gdn_get_digital_shifts", "gdn_get_digital_permutations", "DeviceGenerator"]

PERM_MAX = 65536  # the GPU form's largest permutation (16-bit entries in shared memory)


class DeviceGenerator(object):
    """A numpy Generator (SFC64) whose state lives in device memory across
    helper calls: pass it as the helpers' ``rng`` and they draw on the GPU
    with no host round trip; ``sync()`` checks the calls and sets the
    Generator's state to where the draws left it.  Until then the Generator
    itself must not be drawn from."""

    def __init__(self, rng, device="cuda", stream=None):
        import torch
        from .nus import sfc64_state_words
        self.rng = rng
        self.dev = torch.device(device) if not isinstance(device, int) else torch.device("cuda", device)
        if self.dev.index is None:
            self.dev = torch.device("cuda", torch.cuda.current_device())
        self.stream = stream or torch.cuda.current_stream(self.dev)
        words = sfc64_state_words(rng)
        with torch.cuda.device(self.dev), torch.cuda.stream(self.stream):
            self.state = torch.from_numpy(words.view(np.int64).copy()).to(self.dev)

    def sync(self):
        """Check the device error word and write the state back to the Generator."""
        from . import _ffi
        from .nus import set_sfc64_state
        lib = _ffi.lib()
        _ffi.check(lib.qmc_device_error_check(self.stream.cuda_stream), "randomisation helpers on the GPU")
        set_sfc64_state(self.rng, self.state.cpu().numpy().view(np.uint64))
        return self.rng


def _on_gpu(rng, device):
    return device is not None or isinstance(rng, DeviceGenerator)


def _gpu_call(rng, device, shape, dtype, launch):
    """Run `launch(lib, state_ptr, out_tensor, stream_handle)` -> rc on the GPU
    with rng's stream; returns the output tensor of `shape`."""
    import torch
    from . import _ffi
    own = not isinstance(rng, DeviceGenerator)
    dg = DeviceGenerator(rng, device if device is not None else "cuda") if own else rng
    lib = _ffi.lib()
    with torch.cuda.device(dg.dev), torch.cuda.stream(dg.stream):
        out = torch.empty(tuple(int(v) for v in shape), dtype=dtype, device=dg.dev)
        _ffi.check(launch(lib, dg.state.data_ptr(), out, dg.stream.cuda_stream), "randomisation helper")
        if own:
            dg.sync()
    return out


def _dev_bases(bases, rng, device):
    import torch
    dev = rng.dev if isinstance(rng, DeviceGenerator) else (torch.device(device) if not isinstance(device, int)
                                                           else torch.device("cuda", device))
    b = np.ascontiguousarray(np.atleast_2d(np.asarray(bases, dtype=np.uint64)))
    return b, torch.from_numpy(b.reshape(-1).view(np.int64).copy()).to(dev)

_TOP = np.uint64(1) << np.uint64(63)


def random_tbit_uint64s(rng, t, shape, device=None):
    """Uniform random integers with t bits (0 <= t <= 64).

Args:
    rng (np.random._generator.Generator): random number generator
    t (int): number of bits, 0 <= t <= 64
    shape (tuple of ints): shape of the result"""
    assert 0 <= t <= 64, "t must be between 0 and 64"
    if _on_gpu(rng, device):
        import torch
        shp = (shape,) if np.isscalar(shape) else tuple(shape)
        cnt = int(np.prod(shp, dtype=np.int64))
        return _gpu_call(rng, device, shp, torch.int64,
                         lambda L, st, out, h: L.qmc_random_tbit_uint64s(st, int(t), cnt, out.data_ptr(), h))
    if t < 64:
        return rng.integers(0, 1 << int(t), shape, dtype=np.uint64)
    # full 64-bit words: draw signed words and move them up by 2^63, which
    # maps [-2^63, 2^63) onto [0, 2^64) (rand_funcs.py:14-19)
    signed = rng.integers(-(1 << 63), 1 << 63, shape, dtype=np.int64)
    return signed.view(np.uint64) ^ _TOP


def random_uint64_permutations(rng, n, b, device=None):
    """n random permutations of 0,...,b-1 as an (n, b) uint64 array.

Args:
    rng (np.random._generator.Generator): random number generator
    n (int): number of permutations
    b (int): permutation length"""
    if _on_gpu(rng, device):
        import torch
        if int(b) > PERM_MAX:
            raise ValueError("permutations on the GPU have at most %d entries (b = %d)" % (PERM_MAX, int(b)))
        return _gpu_call(rng, device, (int(n), int(b)), torch.int64,
                         lambda L, st, out, h: L.qmc_random_uint64_permutations(st, int(n), int(b), out.data_ptr(),
                                                                                h))
    out = np.empty((n, b), dtype=np.uint64)
    for i in range(n):
        out[i] = rng.permutation(b)
    return out


def lat_get_shifts(rng, r, d, device=None):
    """Uniform shifts in [0, 1) for lattice randomisation, shape (r, d).

Args:
    rng (np.random._generator.Generator): random number generator
    r (np.uint64): randomisations
    d (np.uint64): dimension"""
    if _on_gpu(rng, device):
        import torch
        return _gpu_call(rng, device, (int(r), int(d)), torch.float64,
                         lambda L, st, out, h: L.qmc_lat_get_shifts(st, int(r), int(d), out.data_ptr(), h))
    return rng.random((r, d))


def dnb2_get_digital_shifts(rng, r, d, tmax_new, device=None):
    """Random tmax_new-bit digital shifts, shape (r, d).

Args:
    rng (np.random._generator.Generator): random number generator
    r (np.uint64): randomisations
    d (np.uint64): dimension
    tmax_new (np.uint64): bits per shift"""
    return random_tbit_uint64s(rng, tmax_new, (r, d), device=device)


def dnb2_get_linear_scramble_matrix(rng, r, d, tmax, tmax_new, print_mats, device=None):
    """Random lower-unit-triangular GF(2) scrambling matrices, one tmax-bit
row per integer, shape (r, d, tmax_new).

Args:
    rng (np.random._generator.Generator): random number generator
    r (np.uint64): randomisations
    d (np.uint64): dimension
    tmax (np.uint64): bits per integer of the input matrices
    tmax_new (np.uint64): bits per integer after scrambling
    print_mats (np.uint8): print the matrices as bit rows"""
    tmin = int(min(tmax_new, tmax))
    if _on_gpu(rng, device):
        import torch
        assert 0 <= tmin <= 64, "t must be between 0 and 64"
        if not (1 <= int(tmax) <= int(tmax_new)):  # numpy's broadcasting refuses the other shapes
            raise ValueError("dnb2_get_linear_scramble_matrix needs 1 <= tmax <= tmax_new (tmax=%d, tmax_new=%d)"
                             % (int(tmax), int(tmax_new)))
        S = _gpu_call(rng, device, (int(r), int(d), int(tmax_new)), torch.int64,
                      lambda L, st, out, h: L.qmc_dnb2_get_linear_scramble_matrix(st, int(r), int(d), int(tmax),
                                                                                  int(tmax_new), out.data_ptr(), h))
        if print_mats:
            _print_bit_rows(S.cpu().numpy().view(np.uint64), r, d, tmax, tmax_new)
        return S
    S = random_tbit_uint64s(rng, tmin, (r, d, tmax_new))
    # row t keeps only bits above position tmin-t (strictly lower triangle)
    # and gets its diagonal bit at position tmax-1-t
    drop = np.arange(tmin, 0, -1, dtype=np.uint64)
    S[:, :, :tmin] >>= drop
    S[:, :, :tmin] <<= drop
    S[:, :, :tmin] += np.uint64(1) << np.arange(int(tmax) - 1, -1, -1, dtype=np.uint64)
    if print_mats:
        _print_bit_rows(S, r, d, tmax, tmax_new)
    return S


def _print_bit_rows(S, r, d, tmax, tmax_new):
    print("S with shape (r=%d, d=%d, tmax_new=%d)" % (r, d, tmax_new))
    for l in range(r):
        print("l = %d" % l)
        for j in range(d):
            print("    j = %d" % j)
            for t in range(tmax_new):
                bits = bin(S[l, j, t])[2:]
                print("        " + "0" * int(tmax - len(bits)) + bits)


def gdn_get_linear_scramble_matrix(rng, r, d, tmax, tmax_new, r_b, bases, device=None):
    """Random lower-triangular base-b scrambling matrices with nonzero
diagonal, shape (r, d, tmax_new, tmax).

Args:
    rng (np.random._generator.Generator): random number generator
    r (np.uint64): randomisations
    d (np.uint64): dimension
    tmax (np.uint64): digits per column of the input matrices
    tmax_new (np.uint64): digits per column after scrambling
    r_b (np.uint64): randomisations of bases
    bases (np.ndarray of np.uint64): bases, r_b*d"""
    if _on_gpu(rng, device):
        import torch
        b2, db = _dev_bases(bases, rng, device)
        used = _used_bases(b2, r, r_b, d)
        if int(tmax_new) < int(tmax):  # numpy's boolean assignment refuses it
            raise ValueError("gdn_get_linear_scramble_matrix needs tmax <= tmax_new")
        if used.size and used.min() < 2:
            raise ValueError("high <= low: the diagonal is drawn from integers(1, b)")
        return _gpu_call(rng, device, (int(r), int(d), int(tmax_new), int(tmax)), torch.int64,
                         lambda L, st, out, h: L.qmc_gdn_get_linear_scramble_matrix(
                             st, int(r), int(d), int(tmax), int(tmax_new), int(r_b), db.data_ptr(), out.data_ptr(),
                             h))
    S = np.empty((r, d, tmax_new, tmax), dtype=np.uint64)
    bases_2d = np.atleast_2d(bases)
    below = np.tri(int(tmax_new), int(tmax), k=-1, dtype=bool)
    n_below = below.sum()
    diag = np.eye(tmax_new, tmax, dtype=bool)
    for l in range(r):
        lb = int(l % r_b)
        for j in range(d):
            b = bases_2d[lb, j]
            M = np.zeros((tmax_new, tmax), dtype=np.uint64)
            M[below] = rng.integers(0, b, n_below)
            M[diag] = rng.integers(1, b, tmax)
            S[l, j] = M
    return S


def gdn_get_halton_generating_matrix(r, d, mmax):
    """Identity generating matrices of the Halton sequence, shape (r, d, mmax, mmax).

Args:
    r (np.uint64): randomisations
    d (np.uint64): dimension
    mmax (np.uint64): rows and columns of each matrix"""
    return np.tile(np.eye(mmax, dtype=np.uint64)[None, None, :, :], (int(r), int(d), 1, 1))


def gdn_get_digital_shifts(rng, r, d, tmax_new, r_b, bases, device=None):
    """Random base-b digital shifts, shape (r, d, tmax_new).

Args:
    rng (np.random._generator.Generator): random number generator
    r (np.uint64): randomisations
    d (np.uint64): dimension
    tmax_new (np.uint64): digits per shift
    r_b (np.uint64): randomisations of bases
    bases (np.ndarray of np.uint64): bases, r_b*d"""
    if _on_gpu(rng, device):
        import torch
        b2, db = _dev_bases(bases, rng, device)
        used = _used_bases(b2, r, r_b, d)
        if used.size and used.min() < 1:
            raise ValueError("high <= low: shifts are drawn from integers(0, b)")
        return _gpu_call(rng, device, (int(r), int(d), int(tmax_new)), torch.int64,
                         lambda L, st, out, h: L.qmc_gdn_get_digital_shifts(
                             st, int(r), int(d), int(tmax_new), int(r_b), db.data_ptr(), out.data_ptr(), h))
    out = np.empty((r, d, tmax_new), dtype=np.uint64)
    bases_2d = np.atleast_2d(bases)
    for l in range(r):
        lb = int(l % r_b)
        for j in range(d):
            out[l, j] = rng.integers(0, bases_2d[lb, j], tmax_new, dtype=np.uint64)
    return out


def gdn_get_digital_permutations(rng, r, d, tmax_new, r_b, bases, device=None):
    """Random per-digit permutations of 0..b-1, zero-padded to the largest
base, shape (r, d, tmax_new, bmax).

Args:
    rng (np.random._generator.Generator): random number generator
    r (np.uint64): randomisations
    d (np.uint64): dimension
    tmax_new (np.uint64): digits
    r_b (np.uint64): randomisations of bases
    bases (np.ndarray of np.uint64): bases, r_b*d"""
    if _on_gpu(rng, device):
        import torch
        b2, db = _dev_bases(bases, rng, device)
        bmax = int(b2.max())
        if bmax > PERM_MAX:
            raise ValueError("permutations on the GPU have at most %d entries (largest base %d)" % (PERM_MAX, bmax))
        return _gpu_call(rng, device, (int(r), int(d), int(tmax_new), bmax), torch.int64,
                         lambda L, st, out, h: L.qmc_gdn_get_digital_permutations(
                             st, int(r), int(d), int(tmax_new), int(r_b), db.data_ptr(), bmax, out.data_ptr(), h))
    bases_2d = np.atleast_2d(bases)
    bmax = bases_2d.max()
    out = np.zeros((r, d, tmax_new, bmax), dtype=np.uint64)
    for l in range(r):
        lb = int(l % r_b)
        for j in range(d):
            b = bases_2d[lb, j]
            for t in range(tmax_new):
                out[l, j, t, :b] = rng.permutation(b)
    return out


def _used_bases(b2, r, r_b, d):
    """the bases the (l, j) loops of the helpers read: rows l % r_b for l < r"""
    rows = sorted({int(l % int(r_b)) for l in range(min(int(r), int(r_b)))})
    return b2[rows, :int(d)] if rows else np.zeros(0, np.uint64)
