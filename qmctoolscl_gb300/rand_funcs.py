"""Host-side generators of randomisation inputs (shifts, scrambling matrices,
permutations), part of the QMCToolsCL call surface (qmctoolscl/rand_funcs.py:4-153).

These produce the inputs that the GPU kernels consume.  Their outputs are
defined by numpy's random streams, so each helper draws from the Generator
with the same calls, shapes, bounds and dtypes, in the same order, as the
reference helper of the same name: given a Generator in the same state they
return identical arrays (checked against fixtures recorded from the
reference).  The nested-uniform-scrambling routines of the reference
(rand_funcs.py:155-356) run on the GPU and live in nus.py.
"""
import numpy as np

__all__ = ["random_tbit_uint64s", "random_uint64_permutations", "lat_get_shifts", "dnb2_get_digital_shifts",
           "dnb2_get_linear_scramble_matrix", "gdn_get_linear_scramble_matrix", "gdn_get_halton_generating_matrix",
           "gdn_get_digital_shifts", "gdn_get_digital_permutations"]

_TOP = np.uint64(1) << np.uint64(63)


def random_tbit_uint64s(rng, t, shape):
    """Uniform random integers with t bits (0 <= t <= 64).

Args:
    rng (np.random._generator.Generator): random number generator
    t (int): number of bits, 0 <= t <= 64
    shape (tuple of ints): shape of the result"""
    assert 0 <= t <= 64, "t must be between 0 and 64"
    if t < 64:
        return rng.integers(0, 1 << int(t), shape, dtype=np.uint64)
    # full 64-bit words: draw signed words and move them up by 2^63, which
    # maps [-2^63, 2^63) onto [0, 2^64) (rand_funcs.py:14-19)
    signed = rng.integers(-(1 << 63), 1 << 63, shape, dtype=np.int64)
    return signed.view(np.uint64) ^ _TOP


def random_uint64_permutations(rng, n, b):
    """n random permutations of 0,...,b-1 as an (n, b) uint64 array.

Args:
    rng (np.random._generator.Generator): random number generator
    n (int): number of permutations
    b (int): permutation length"""
    out = np.empty((n, b), dtype=np.uint64)
    for i in range(n):
        out[i] = rng.permutation(b)
    return out


def lat_get_shifts(rng, r, d):
    """Uniform shifts in [0, 1) for lattice randomisation, shape (r, d).

Args:
    rng (np.random._generator.Generator): random number generator
    r (np.uint64): randomisations
    d (np.uint64): dimension"""
    return rng.random((r, d))


def dnb2_get_digital_shifts(rng, r, d, tmax_new):
    """Random tmax_new-bit digital shifts, shape (r, d).

Args:
    rng (np.random._generator.Generator): random number generator
    r (np.uint64): randomisations
    d (np.uint64): dimension
    tmax_new (np.uint64): bits per shift"""
    return random_tbit_uint64s(rng, tmax_new, (r, d))


def dnb2_get_linear_scramble_matrix(rng, r, d, tmax, tmax_new, print_mats):
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
    S = random_tbit_uint64s(rng, tmin, (r, d, tmax_new))
    # row t keeps only bits above position tmin-t (strictly lower triangle)
    # and gets its diagonal bit at position tmax-1-t
    drop = np.arange(tmin, 0, -1, dtype=np.uint64)
    S[:, :, :tmin] >>= drop
    S[:, :, :tmin] <<= drop
    S[:, :, :tmin] += np.uint64(1) << np.arange(int(tmax) - 1, -1, -1, dtype=np.uint64)
    if print_mats:
        print("S with shape (r=%d, d=%d, tmax_new=%d)" % (r, d, tmax_new))
        for l in range(r):
            print("l = %d" % l)
            for j in range(d):
                print("    j = %d" % j)
                for t in range(tmax_new):
                    bits = bin(S[l, j, t])[2:]
                    print("        " + "0" * int(tmax - len(bits)) + bits)
    return S


def gdn_get_linear_scramble_matrix(rng, r, d, tmax, tmax_new, r_b, bases):
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


def gdn_get_digital_shifts(rng, r, d, tmax_new, r_b, bases):
    """Random base-b digital shifts, shape (r, d, tmax_new).

Args:
    rng (np.random._generator.Generator): random number generator
    r (np.uint64): randomisations
    d (np.uint64): dimension
    tmax_new (np.uint64): digits per shift
    r_b (np.uint64): randomisations of bases
    bases (np.ndarray of np.uint64): bases, r_b*d"""
    out = np.empty((r, d, tmax_new), dtype=np.uint64)
    bases_2d = np.atleast_2d(bases)
    for l in range(r):
        lb = int(l % r_b)
        for j in range(d):
            out[l, j] = rng.integers(0, bases_2d[lb, j], tmax_new, dtype=np.uint64)
    return out


def gdn_get_digital_permutations(rng, r, d, tmax_new, r_b, bases):
    """Random per-digit permutations of 0..b-1, zero-padded to the largest
base, shape (r, d, tmax_new, bmax).

Args:
    rng (np.random._generator.Generator): random number generator
    r (np.uint64): randomisations
    d (np.uint64): dimension
    tmax_new (np.uint64): digits
    r_b (np.uint64): randomisations of bases
    bases (np.ndarray of np.uint64): bases, r_b*d"""
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
