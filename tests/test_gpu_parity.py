"""GPU parity: the CUDA kernels, called through the drop-in API (and so
through the C ABI of libqmcgb.so), against the golden fixtures recorded from
the reference C backend and against the oracle on seeded random inputs.

Integer, lattice and float-conversion outputs must match bit for bit.  The
FP64 transforms must match to a relative error of 1e-12 (they run a
different but equally accurate operation order); the twiddle tables to
1e-15 absolute.
"""
import numpy as np
import pytest

import oracle
import qmctoolscl_gb300 as q
from qmctoolscl_gb300._signatures import SIGNATURES
from tests import _golden

pytestmark = pytest.mark.gpu
U = np.uint64
cases, _ = _golden.load()


def run_gpu(name, args):
    getattr(q, name)(*args)


def same_bits(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.dtype == np.float64:
        return np.array_equal(a.view(np.uint64), b.view(np.uint64))
    return np.array_equal(a, b)


@pytest.mark.parametrize("cid", _golden.case_ids(), ids=lambda c: "%s-%d" % (cases[c]["name"], c))
def test_golden_case(cid):
    case = cases[cid]
    args = _golden.build_args(case)
    run_gpu(case["name"], args)
    if case["name"] in _golden.TRANSFORMS:
        names = [a for a, _k in SIGNATURES[case["name"]][0]]
        for an, want in _golden.expected(case).items():
            got = np.asarray(args[names.index(an)])
            if an in _golden.TWIDDLES:
                got = got.reshape(-1)[:want.size]
                assert np.allclose(got, want, rtol=0, atol=1e-15), an
            else:
                got = got.reshape(want.shape)
                err = np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-300)
                assert err < 1e-12, (an, err)
    else:
        assert _golden.check_outputs(case, args, exact=True) == []


# ---------------------------------------------------------------- random

def both(name, args, out_names):
    """Run the oracle and the GPU on copies of the same arguments; return
    {out: (gpu, oracle)}."""
    names = [a for a, _k in SIGNATURES[name][0]]
    a_gpu = [a.copy() if isinstance(a, np.ndarray) else a for a in args]
    a_orc = [a.copy() if isinstance(a, np.ndarray) else a for a in args]
    run_gpu(name, a_gpu)
    oracle.call(name, *a_orc)
    return {o: (a_gpu[names.index(o)], a_orc[names.index(o)]) for o in out_names}


def poison(shape, dt):
    a = np.empty(shape, dt)
    a.view(np.uint64)[...] = U(0x7FF4DEADBEEF0001)
    return a


@pytest.mark.parametrize("order", ["linear", "natural", "gray"])
@pytest.mark.parametrize("bits", [20, 33, 52, 64])
def test_lattice_random(order, bits):
    rng = np.random.Generator(np.random.SFC64(100 + bits))
    r, d = 3, 7
    n = 4096 if order != "linear" else 3000  # non-power-of-two linear n takes the FP64 path
    g = (rng.integers(0, 1 << (bits - 1), (r, d), dtype=U) * U(2) + U(1))
    g[0, 0] = U(1)
    if order == "linear":
        res = both("lat_gen_linear", [U(r), U(n), U(d), g, poison((r, n, d), np.float64)], ["x"])
    elif order == "natural":
        res = both("lat_gen_natural", [U(r), U(n), U(d), U(0), g, poison((r, n, d), np.float64)], ["x"])
    else:
        res = both("lat_gen_gray", [U(r), U(n), U(d), U(77), g, poison((r, n, d), np.float64)], ["x"])
    gpu, orc = res["x"]
    assert same_bits(gpu, orc)


def test_lattice_linear_pow2_fast_path():
    rng = np.random.Generator(np.random.SFC64(5))
    g = rng.integers(0, 1 << 20, (2, 9), dtype=U) * U(2) + U(1)
    gpu, orc = both("lat_gen_linear", [U(2), U(1 << 14), U(9), g, poison((2, 1 << 14, 9), np.float64)], ["x"])["x"]
    assert same_bits(gpu, orc)


@pytest.mark.parametrize("kind", ["lattice", "uniform", "odd_bits", "wild"])
@pytest.mark.parametrize("r_x", [1, 4])
def test_shift_mod_1_random(kind, r_x):
    rng = np.random.Generator(np.random.SFC64(7))
    r, n, d = 4, 1000, 6
    if kind == "lattice":
        x = (rng.integers(0, 1 << 20, (r_x, n, d)) / float(1 << 20))
    elif kind == "uniform":
        x = rng.random((r_x, n, d))
    elif kind == "odd_bits":  # multiples of 2^-64 that are not multiples of 2^-53
        x = rng.integers(0, 1 << 62, (r_x, n, d)).astype(np.float64) * 2.0 ** -62
        x[..., 0] = 2.0 ** -64 * 3
    else:  # negative, >= 1, tiny, subnormal, inf/nan-free
        x = rng.standard_normal((r_x, n, d)) * 3
        x[0, 0, :] = [0.0, -0.0, 1.0, -1.0, 5e-324, 2.0 ** 60][:d]
    shifts = rng.random((r, d))
    if kind == "odd_bits":
        shifts[:, 0] = 1 - 2.0 ** -60
    if kind == "wild":
        shifts[0, :2] = [-0.25, 2.5]
    gpu, orc = both("lat_shift_mod_1", [U(r), U(n), U(d), U(r_x), x, shifts, poison((r, n, d), np.float64)],
                    ["xr"])["xr"]
    assert same_bits(gpu, orc)


@pytest.mark.parametrize("natural", [True, False])
@pytest.mark.parametrize("n_start,n,mmax,d", [(0, 1 << 12, 12, 5), (0, 1 << 15, 20, 64), (8, 8, 4, 3),
                                              (1 << 10, 1 << 10, 11, 70), (2, 14, 4, 2), (0, 100, 7, 33),
                                              (0, 1 << 12, 12, 12), (1 << 12, 1 << 12, 14, 36),
                                              (1 << 31, 1 << 10, 32, 8), ((1 << 31) - (1 << 10), 1 << 11, 32, 16)])
def test_dnb2_gen_random(natural, n_start, n, mmax, d):
    rng = np.random.Generator(np.random.SFC64(n + mmax + d))
    r = 3
    C = q.random_tbit_uint64s(rng, 64, (r, d, mmax))
    if natural and n_start == 0 and n == 100:
        n = 128  # natural order needs a Gray-closed range
    if natural and n_start >= 1 << 30:
        pytest.skip("natural order needs a Gray-closed range; these ranges exercise 64-bit indices in Gray order")
    name = "dnb2_gen_natural" if natural else "dnb2_gen_gray"
    gpu, orc = both(name, [U(r), U(n), U(d), U(n_start), U(mmax), C, poison((r, n, d), U)], ["xb"])["xb"]
    assert same_bits(gpu, orc)


def test_dnb2_gen_rejects_open_range():
    C = np.ones((1, 2, 4), U)
    with pytest.raises(ValueError, match="Gray code"):
        q.dnb2_gen_natural(U(1), U(5), U(2), U(0), U(4), C, np.empty((1, 5, 2), U))
    with pytest.raises(ValueError, match="mmax"):
        q.dnb2_gen_gray(U(1), U(17), U(2), U(0), U(4), C, np.empty((1, 17, 2), U))


@pytest.mark.parametrize("r_x", [1, 3])
def test_dnb2_shift_and_float_random(r_x):
    rng = np.random.Generator(np.random.SFC64(9))
    r, n, d = 3, 2000, 5
    xb = q.random_tbit_uint64s(rng, 64, (r_x, n, d))
    lsh = np.array([0, 13, 63][:r_x], U)
    sb = q.dnb2_get_digital_shifts(rng, r, d, 64)
    gpu, orc = both("dnb2_digital_shift", [U(r), U(n), U(d), U(r_x), lsh, xb, sb, poison((r, n, d), U)],
                    ["xrb"])["xrb"]
    assert same_bits(gpu, orc)
    tm = np.array([64, 1, 1100][:r] if r == 3 else [64] * r, U)
    xb2 = q.random_tbit_uint64s(rng, 64, (r, n, d))
    xb2[0, 0, :] = [0, 1, (1 << 64) - 1, (1 << 53) + 1, (1 << 54) + 6]
    gpu, orc = both("dnb2_integer_to_float", [U(r), U(n), U(d), tm, xb2, poison((r, n, d), np.float64)],
                    ["x"])["x"]
    assert same_bits(gpu, orc)


@pytest.mark.parametrize("tmax,tnew", [(20, 32), (64, 64), (10, 70)])
def test_dnb2_matrix_side_random(tmax, tnew):
    rng = np.random.Generator(np.random.SFC64(tmax * 100 + tnew))
    r, r_C, d, mmax = 5, 1, 12, 20  # d divisible by both interlacing factors
    C = q.random_tbit_uint64s(rng, tmax, (r_C, d, mmax))
    S = q.random_tbit_uint64s(rng, 64, (r, d, tnew))
    gpu, orc = both("dnb2_linear_matrix_scramble", [U(r), U(d), U(mmax), U(r_C), U(tnew), S, C,
                                                    poison((r, d, mmax), U)], ["C_lms"])["C_lms"]
    assert same_bits(gpu, orc)
    for alpha in (2, 3):
        da = d // alpha
        ta = min(alpha * tmax, 64)
        Cb = q.random_tbit_uint64s(rng, tmax, (r, d, mmax))
        gpu, orc = both("dnb2_interlace", [U(r), U(da), U(mmax), U(d), U(tmax), U(ta), U(alpha), Cb,
                                           poison((r, da, mmax), U)], ["C_alpha"])["C_alpha"]
        assert same_bits(gpu, orc)
        gpu2, orc2 = both("dnb2_undo_interlace", [U(r), U(d), U(mmax), U(da), U(tmax), U(ta), U(alpha), gpu,
                                                  poison((r, d, mmax), U)], ["C"])["C"]
        assert same_bits(gpu2, orc2)
    tm = np.array([tmax] * r, U)
    Cl = q.random_tbit_uint64s(rng, min(tmax, 63), (r, d, mmax))
    gpu, orc = both("dnb2_gmat_lsb_to_msb", [U(r), U(d), U(mmax), tm, Cl, poison((r, d, mmax), U)],
                    ["C_msb"])["C_msb"]
    assert same_bits(gpu, orc)


PRIMES = np.array([2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 67, 71, 73, 79, 83, 89,
                   97, 101, 103, 107, 109, 113, 127, 131, 137, 139, 149, 151, 157, 163, 167, 173, 179, 181, 191,
                   193, 197, 199, 211, 223, 227, 229, 233, 239, 241, 251, 257, 263, 269, 271, 277, 281, 283, 293,
                   307, 311, 313, 317, 331, 337, 347, 349, 353, 359, 367, 373, 379, 383, 389, 397, 401, 409, 419,
                   421, 431, 433, 439, 443, 449, 457, 461, 463, 467, 479, 487, 491, 499, 503, 509, 521, 523, 541],
                  dtype=U)


@pytest.mark.parametrize("big_c", [False, True])
def test_gdn_pipeline_random(big_c):
    """LMS -> generation -> permutation -> shift -> float on prime bases,
    each step against the oracle on the same inputs."""
    rng = np.random.Generator(np.random.SFC64(4 + big_c))
    r, r_b, d, n, n_start = 3, 1, 12, 700, 13
    bases = PRIMES[np.array([0, 1, 2, 3, 4, 10, 25, 50, 75, 97, 98, 99])][None, :]
    mmax, tmax, tnew = 10, 12, 14  # 2^10 > n_start+n: every base has enough columns
    C = q.gdn_get_halton_generating_matrix(1, d, tmax)[:, :, :mmax, :]
    C = np.ascontiguousarray(C)
    if big_c:
        C = C + q.random_tbit_uint64s(rng, 60, C.shape)  # entries far above the base: 64-bit path
    S = q.gdn_get_linear_scramble_matrix(rng, r, d, tmax, tnew, r_b, bases)
    C_lms = both("gdn_linear_matrix_scramble", [U(r), U(d), U(mmax), U(1), U(r_b), U(tmax), U(tnew), bases, S, C,
                                                poison((r, d, mmax, tnew), U)], ["C_lms"])["C_lms"]
    assert same_bits(*C_lms)
    xdig = both("gdn_gen_natural", [U(r), U(n), U(d), U(r_b), U(mmax), U(tnew), U(n_start), bases, C_lms[1],
                                    poison((r, n, d, tnew), U)], ["xdig"])["xdig"]
    assert same_bits(*xdig)
    perms = q.gdn_get_digital_permutations(rng, r, d, tnew + 2, r_b, bases)
    bmax = U(bases.max())
    xp = both("gdn_digital_permutation", [U(r), U(n), U(d), U(r), U(r_b), U(tnew), U(tnew + 2), bmax, perms,
                                          xdig[1], poison((r, n, d, tnew + 2), U)], ["xdig_new"])["xdig_new"]
    assert same_bits(*xp)
    sh = q.gdn_get_digital_shifts(rng, r, d, tnew + 4, r_b, bases)
    xs = both("gdn_digital_shift", [U(r), U(n), U(d), U(r), U(r_b), U(tnew + 2), U(tnew + 4), bases, sh, xp[1],
                                    poison((r, n, d, tnew + 4), U)], ["xdig_new"])["xdig_new"]
    assert same_bits(*xs)
    xf = both("gdn_integer_to_float", [U(r), U(n), U(d), U(r_b), U(tnew + 4), bases, xs[1],
                                       poison((r, n, d), np.float64)], ["x"])["x"]
    assert same_bits(*xf)


@pytest.mark.parametrize("b", [2, 3, 5, 31, 32, 33, 541, 1021, 4093])
@pytest.mark.parametrize("d,n_start", [(1, 0), (1, 45), (3, 1000)])
def test_gdn_gen_natural_tiled_forms(b, d, n_start):
    """gdn_gen_natural on a base-b Halton-like matrix with random unit-triangular
    scrambling, tmax = ceil(64/log2 b): the low-digit table form (b^K * tmax
    small), the staged form (large b) and both output layouts (d = 1: the
    group's words in order; d > 1: runs per point), ragged n, against the
    oracle bit for bit."""
    rng = np.random.Generator(np.random.SFC64(b * 7 + d))
    r, n = 2, (1 << 13) + 17
    tmax = int(np.ceil(64 / np.log2(b)))
    mmax = 1
    while b ** mmax < n_start + n:
        mmax += 1
    bases = np.full((1, d), b, U)
    C = rng.integers(0, b, (r, d, mmax, tmax), dtype=U)
    x = both("gdn_gen_natural", [U(r), U(n), U(d), U(1), U(mmax), U(tmax), U(n_start), bases, C,
                                 poison((r, n, d, tmax), U)], ["xdig"])["xdig"]
    assert same_bits(*x)


@pytest.mark.parametrize("tmax", [1, 12, 64, 80])
def test_gdn_integer_to_float_depths(tmax):
    rng = np.random.Generator(np.random.SFC64(tmax))
    r, n, d = 2, 300, 6
    bases = np.array([[2, 3, 5, 7, 541, 1000003]], U)
    xdig = np.empty((r, n, d, tmax), U)
    for j in range(d):
        xdig[:, :, j] = rng.integers(0, bases[0, j], (r, n, tmax), dtype=U)
    xdig[0, 0, 0, 0] = U(1 << 40)  # a digit outside the emulated range
    gpu, orc = both("gdn_integer_to_float", [U(r), U(n), U(d), U(1), U(tmax), bases, xdig,
                                             poison((r, n, d), np.float64)], ["x"])["x"]
    assert same_bits(gpu, orc)


@pytest.mark.parametrize("bases,tmax,r_b", [([2], 64, 1), ([2], 53, 1), ([2], 54, 1), ([2], 55, 1), ([2], 7, 1),
                                           ([2, 3], 60, 2), ([3], 41, 1), ([541], 3, 1), ([251], 8, 1),
                                           ([2, 3, 5, 7], 64, 1), ([2, 3, 5, 7], 13, 2), ([2047], 1, 1),
                                           ([2, 1021], 1, 1), ([2, 1021], 2, 1), ([2, 1023], 2, 1)])
def test_gdn_integer_to_float_term_table(bases, tmax, r_b):
    """Shapes whose per-CTA product tables RN(recip_t * digit) fit in shared memory (the
    one-FP64-add-per-digit path), odd and even digit counts, bases per randomisation, digits
    at and beyond the base (products outside the table)."""
    rng = np.random.Generator(np.random.SFC64(len(bases) * 100 + tmax + r_b))
    r, n, d = 3, 257, len(bases)
    B = np.array([bases] * r_b, U)
    if r_b > 1:
        B[1:] = B[1:] + 2  # another base per randomisation (2 -> 4, 3 -> 5, ...)
    xdig = np.empty((r, n, d, tmax), U)
    for l in range(r):
        for j in range(d):
            xdig[l, :, j] = rng.integers(0, B[l % r_b, j], (n, tmax), dtype=U)
    xdig[0, 0, 0, 0] = B[0, 0]             # the base itself: just outside the table
    xdig[1, 5, d - 1, tmax - 1] = U(1 << 40)  # far outside
    xdig[2, 7, 0, :] = B[0 if r_b == 1 else 2 % r_b, 0] - 1  # every digit maximal
    gpu, orc = both("gdn_integer_to_float", [U(r), U(n), U(d), U(r_b), U(tmax), B, xdig,
                                             poison((r, n, d), np.float64)], ["x"])["x"]
    assert same_bits(gpu, orc)


def test_gdn_same_base_and_interlace_random():
    rng = np.random.Generator(np.random.SFC64(3))
    r, n, d, mmax, tmax, b = 2, 500, 6, 6, 7, 5
    C = rng.integers(0, b, (r, d, mmax, tmax), dtype=U)
    x = both("gdn_gen_natural_same_base", [U(r), U(n), U(d), U(mmax), U(tmax), U(3), U(b), C,
                                           poison((r, n, d, tmax), U)], ["xdig"])["xdig"]
    assert same_bits(*x)
    alpha = 3
    Ca = both("gdn_interlace", [U(r), U(d // alpha), U(mmax), U(d), U(tmax), U(alpha * tmax), U(alpha), C,
                                poison((r, d // alpha, mmax, alpha * tmax), U)], ["C_alpha"])["C_alpha"]
    assert same_bits(*Ca)
    Cu = both("gdn_undo_interlace", [U(r), U(d), U(mmax), U(d // alpha), U(tmax), U(alpha * tmax), U(alpha),
                                     Ca[0], poison((r, d, mmax, tmax), U)], ["C"])["C"]
    assert same_bits(*Cu) and same_bits(Cu[0], C)


def test_gdn_permutation_out_of_array_digit_is_reported():
    perms = np.zeros((1, 1, 1, 3), U)
    xdig = np.array([[[[7]]]], U)  # 7 >= bmax and beyond the whole perms array
    with pytest.raises(Exception, match="outside its array"):
        q.gdn_digital_permutation(U(1), U(1), U(1), U(1), U(1), U(1), U(1), U(3), perms, xdig,
                                  np.empty((1, 1, 1, 1), U))
    # a digit >= bmax that still lands inside perms reads what the reference reads
    perms = np.arange(12, dtype=U).reshape(1, 2, 2, 3)
    xdig = np.array([[[[4, 0], [1, 0]]]], U)
    args = [U(1), U(1), U(2), U(1), U(1), U(2), U(2), U(3), perms, xdig, np.empty((1, 1, 2, 2), U)]
    gpu, orc = both("gdn_digital_permutation", args, ["xdig_new"])["xdig_new"]
    assert same_bits(gpu, orc)


# ---------------------------------------------------------------- transforms

def bitrev(m):
    i = np.arange(1 << m)
    out = np.zeros_like(i)
    for b in range(m):
        out |= ((i >> b) & 1) << (m - 1 - b)
    return out


@pytest.mark.parametrize("m", [1, 2, 5, 10, 12, 13, 16, 20])
def test_fft_ifft_against_numpy(m):
    rng = np.random.Generator(np.random.SFC64(m))
    n = 1 << m
    d1, d2 = (2, 3) if m <= 12 else (1, 2)
    z = rng.standard_normal((d1, d2, n)) + 1j * rng.standard_normal((d1, d2, n))
    xr, xi = np.ascontiguousarray(z.real), np.ascontiguousarray(z.imag)
    twr, twi = np.empty(n), np.empty(n)
    q.fft_bro_1d_radix2(U(d1), U(d2), U(n // 2), twr, twi, xr, xi)
    want = np.fft.fft(z[:, :, bitrev(m)], norm="ortho")
    got = xr + 1j * xi
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-13
    t = np.arange(n)
    assert np.allclose(twr, np.cos(-2 * np.pi * t / n), atol=1e-15)
    assert np.allclose(twi, np.sin(-2 * np.pi * t / n), atol=1e-15)
    q.ifft_bro_1d_radix2(U(d1), U(d2), U(n // 2), twr, twi, xr, xi)
    back = xr + 1j * xi
    assert np.linalg.norm(back - z) / np.linalg.norm(z) < 1e-13


@pytest.mark.parametrize("m", [1, 3, 13, 14, 18])
def test_fwht_involution_and_oracle(m):
    rng = np.random.Generator(np.random.SFC64(m))
    n = 1 << m
    x = rng.standard_normal((2, 1, n))
    x0 = x.copy()
    orc = x.copy()
    q.fwht_1d_radix2(U(2), U(1), U(n // 2), x)
    if m <= 14:
        oracle.call("fwht_1d_radix2", U(2), U(1), U(n // 2), orc)
        assert np.linalg.norm(x - orc) / np.linalg.norm(orc) < 1e-13
    q.fwht_1d_radix2(U(2), U(1), U(n // 2), x)  # orthonormal WHT is its own inverse
    assert np.linalg.norm(x - x0) / np.linalg.norm(x0) < 1e-13


# ---------------------------------------------------------------- torch path

def test_device_tensors_in_place_no_copies():
    import torch
    rng = np.random.Generator(np.random.SFC64(1))
    r, n, d = 2, 1024, 8
    g = rng.integers(0, 1 << 19, (r, d), dtype=U) * U(2) + U(1)
    gt = torch.from_numpy(g.view(np.int64)).cuda()
    xt = torch.empty((r, n, d), dtype=torch.float64, device="cuda")
    tp, tc = q.lat_gen_gray(U(r), U(n), U(d), U(0), gt, xt)
    assert tc >= 0
    ref = np.empty((r, n, d))
    oracle.call("lat_gen_gray", U(r), U(n), U(d), U(0), g, ref)
    assert same_bits(xt.cpu().numpy(), ref)
    # asynchronous launch
    _tp, tc = q.lat_gen_gray(U(r), U(n), U(d), U(0), gt, xt, wait=False)
    assert tc == -1
    torch.cuda.synchronize()


# the extents that bound the output loops (n_half = 0 and a zero alpha-dimension count are
# undefined in the reference: log2(0), a division by zero)
_EXTENTS = ("r", "n", "d", "d1", "d2")


def _zero_extent_cases():
    """(case id, extent) for the first golden case of every function and each extent it has."""
    seen, out = set(), []
    for cid in _golden.case_ids():
        case = cases[cid]
        if case["name"] in seen:
            continue
        seen.add(case["name"])
        for ext in _EXTENTS:
            if ext in case["scalars"]:
                out.append((cid, ext))
    return out


@pytest.mark.parametrize("cid,ext", _zero_extent_cases(), ids=lambda v: str(v))
def test_zero_extent_writes_nothing(cid, ext):
    """An extent of 0 (the reference's loops do not run): the outputs keep every bit of
    their previous contents on the GPU as in the oracle, and nothing is reported."""
    case = cases[cid]
    names = [a for a, _k in SIGNATURES[case["name"]][0]]
    args_g, args_o = _golden.build_args(case), _golden.build_args(case)
    for args in (args_g, args_o):
        args[names.index(ext)] = U(0)
    if case["name"] in ("dnb2_interlace", "gdn_interlace") and ext == "d":
        # the reference would read its (empty) d-dimension input outside the array: reported
        from qmctoolscl_gb300._ffi import QmcError
        with pytest.raises(QmcError, match="outside its array"):
            run_gpu(case["name"], args_g)
        return
    before = {o: np.array(args_g[names.index(o)], copy=True) for o in case["outputs"]}
    run_gpu(case["name"], args_g)
    oracle.call(case["name"], *args_o)
    for o in case["outputs"]:
        got, orc = args_g[names.index(o)], args_o[names.index(o)]
        if o in _golden.TWIDDLES:  # written at any vector count, to 1e-15 as in the golden cases
            assert np.allclose(got, orc, rtol=0, atol=1e-15), o
            continue
        assert same_bits(got, orc), (o, "differs from the oracle")
        assert same_bits(got, before[o]), (o, "written at a zero extent")
