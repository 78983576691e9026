"""Fused generalized digital net (randomised Halton) against the oracle.

The oracle runs the reference chain one dimension at a time (d = 1, r_b = 1,
tmax_new = tmax_j): gdn_linear_matrix_scramble -> gdn_gen_natural ->
gdn_digital_permutation -> gdn_digital_shift -> gdn_integer_to_float, and the
fused plan must reproduce every float bit for bit.  Inputs come from the
reference's own generators (rand_funcs), drawn per dimension in order.
"""
import math

import numpy as np
import pytest

import oracle
import qmctoolscl_gb300 as q
from qmctoolscl_gb300 import halton

pytestmark = pytest.mark.gpu
U = np.uint64

PRIMES = [p for p in range(2, 542) if all(p % k for k in range(2, int(p ** 0.5) + 1))]


def digits_needed(n_last, b):
    k = 0
    while n_last:
        n_last //= b
        k += 1
    return max(k, 1)


def make_dims(rng, r, bases, n_last, bits=64, lms=True, perm=True, shift=True, tmax_cap=None):
    """Per-dimension inputs in the reference's shapes at d = 1."""
    dims = []
    for b in bases:
        tmax = math.ceil(bits / math.log2(b))
        if tmax_cap:
            tmax = min(tmax, tmax_cap)
        mmax = digits_needed(n_last, b)
        bb = np.array([[b]], U)
        C = q.gdn_get_halton_generating_matrix(1, 1, max(mmax, tmax))[:, :, :mmax, :tmax]
        dim = dict(b=b, tmax=tmax, mmax=mmax, C=np.ascontiguousarray(C))
        if lms:
            dim["S"] = q.gdn_get_linear_scramble_matrix(rng, r, 1, tmax, tmax, 1, bb)
        if perm:
            dim["perms"] = q.gdn_get_digital_permutations(rng, r, 1, tmax, 1, bb)
        if shift:
            dim["shifts"] = q.gdn_get_digital_shifts(rng, r, 1, tmax, 1, bb)
        dims.append(dim)
    return dims


def oracle_chain(r, n, n_start, dims):
    """The reference's functions, one dimension per call, on the oracle."""
    out = np.empty((r, n, len(dims)), np.float64)
    for j, dm in enumerate(dims):
        b, tmax, mmax = dm["b"], dm["tmax"], dm["mmax"]
        bb = np.array([[b]], U)
        C = dm["C"]
        if dm.get("S") is not None:
            C_lms = np.zeros((r, 1, mmax, tmax), U)
            oracle.call("gdn_linear_matrix_scramble", U(r), U(1), U(mmax), U(1), U(1), U(tmax), U(tmax), bb,
                        dm["S"], C, C_lms)
        else:
            C_lms = np.ascontiguousarray(np.broadcast_to(C, (r, 1, mmax, tmax)))
        xdig = np.zeros((r, n, 1, tmax), U)
        oracle.call("gdn_gen_natural", U(r), U(n), U(1), U(1), U(mmax), U(tmax), U(n_start), bb, C_lms, xdig)
        if dm.get("perms") is not None:
            xp = np.zeros_like(xdig)
            oracle.call("gdn_digital_permutation", U(r), U(n), U(1), U(r), U(1), U(tmax), U(tmax), U(b),
                        dm["perms"], xdig, xp)
            xdig = xp
        if dm.get("shifts") is not None:
            xs = np.zeros_like(xdig)
            oracle.call("gdn_digital_shift", U(r), U(n), U(1), U(r), U(1), U(tmax), U(tmax), bb, dm["shifts"],
                        xdig, xs)
            xdig = xs
        x = np.zeros((r, n, 1), np.float64)
        oracle.call("gdn_integer_to_float", U(r), U(n), U(1), U(1), U(tmax), bb, xdig, x)
        out[:, :, j] = x[:, :, 0]
    return out


def run_fused(r, n, n_start, dims):
    x = np.full((r, n, len(dims)), np.nan)
    halton.generalized_net_fused(r, n, n_start, dims, x)
    return x


def same_bits(a, b):
    return np.array_equal(np.asarray(a).view(U), np.asarray(b).view(U))


@pytest.mark.parametrize("n,n_start", [(700, 13), (64, 0), (1, 5), (33, 2 ** 20 - 7)])
def test_halton_full_chain_matches_oracle(n, n_start):
    rng = np.random.Generator(np.random.SFC64(11 + n))
    r = 3
    bases = [PRIMES[k] for k in (0, 1, 2, 3, 4, 10, 25, 50, 75, 97, 98, 99)]
    dims = make_dims(rng, r, bases, n_start + n - 1)
    assert same_bits(run_fused(r, n, n_start, dims), oracle_chain(r, n, n_start, dims))


def test_halton_first_100_primes_matches_oracle():
    """The benchmark's shape (every base of the first 100 primes, digit counts
    ceil(64/log2 b)), on 2 randomisations of 600 points."""
    rng = np.random.Generator(np.random.SFC64(2024))
    r, n, n_start = 2, 600, 1000
    dims = make_dims(rng, r, PRIMES[:100], n_start + n - 1)
    assert same_bits(run_fused(r, n, n_start, dims), oracle_chain(r, n, n_start, dims))


@pytest.mark.parametrize("lms,perm,shift", [(False, False, False), (True, False, False), (False, True, False),
                                            (False, False, True), (True, False, True), (True, True, False)])
def test_halton_partial_chains(lms, perm, shift):
    rng = np.random.Generator(np.random.SFC64(7 + 4 * lms + 2 * perm + shift))
    r, n, n_start = 2, 300, 3
    bases = [2, 3, 5, 7, 11, 97, 541, 1999]
    dims = make_dims(rng, r, bases, n_start + n - 1, lms=lms, perm=perm, shift=shift)
    assert same_bits(run_fused(r, n, n_start, dims), oracle_chain(r, n, n_start, dims))


def test_halton_unscrambled_is_radical_inverse():
    """Without randomisation the first dimension (base 2) is the van der
    Corput sequence: exact dyadic values."""
    r, n = 1, 256
    dims = make_dims(None, r, [2, 3], n - 1, lms=False, perm=False, shift=False)
    x = run_fused(r, n, 0, dims)
    vdc = np.array([int(format(i, "064b")[::-1], 2) / 2.0 ** 64 for i in range(n)])
    assert np.array_equal(x[0, :, 0], vdc)


def test_halton_big_permutation_values_and_deep_digits():
    """Permutation entries at or above b without a shift (the digit-to-float
    step then sees large digits, so no term may be skipped) and 80 digits."""
    rng = np.random.Generator(np.random.SFC64(99))
    r, n, n_start = 2, 200, 0
    dims = make_dims(rng, r, [3, 5, 31], n - 1, bits=140, shift=False, tmax_cap=80)
    for dm in dims:
        dm["perms"] = dm["perms"] + U(1) + rng.integers(0, 5000, dm["perms"].shape, dtype=U)
    assert same_bits(run_fused(r, n, n_start, dims), oracle_chain(r, n, n_start, dims))


def test_halton_matches_plain_drop_in_chain():
    """The fused plan against the plain drop-in functions (GPU, one call per
    step and dimension) on the same inputs."""
    rng = np.random.Generator(np.random.SFC64(5))
    r, n, n_start = 2, 500, 17
    dims = make_dims(rng, r, [2, 13, 233], n_start + n - 1)
    plain = np.empty((r, n, len(dims)))
    for j, dm in enumerate(dims):
        b, tmax, mmax = dm["b"], dm["tmax"], dm["mmax"]
        bb = np.array([[b]], U)
        C_lms = np.zeros((r, 1, mmax, tmax), U)
        q.gdn_linear_matrix_scramble(U(r), U(1), U(mmax), U(1), U(1), U(tmax), U(tmax), bb, dm["S"], dm["C"], C_lms)
        xdig = np.zeros((r, n, 1, tmax), U)
        q.gdn_gen_natural(U(r), U(n), U(1), U(1), U(mmax), U(tmax), U(n_start), bb, C_lms, xdig)
        xp = np.zeros_like(xdig)
        q.gdn_digital_permutation(U(r), U(n), U(1), U(r), U(1), U(tmax), U(tmax), U(b), dm["perms"], xdig, xp)
        xs = np.zeros_like(xdig)
        q.gdn_digital_shift(U(r), U(n), U(1), U(r), U(1), U(tmax), U(tmax), bb, dm["shifts"], xp, xs)
        x = np.zeros((r, n, 1))
        q.gdn_integer_to_float(U(r), U(n), U(1), U(1), U(tmax), bb, xs, x)
        plain[:, :, j] = x[:, :, 0]
    assert same_bits(run_fused(r, n, n_start, dims), plain)


def test_halton_wide_shift_and_permutation_values():
    """Shift and permutation entries far above b (64-bit wrapping sums in the
    reference) give the same bits."""
    rng = np.random.Generator(np.random.SFC64(1))
    r, n = 2, 100
    dims = make_dims(rng, r, [3, 7, 113], n - 1)
    for dm in dims:
        dm["shifts"] = dm["shifts"] + q.random_tbit_uint64s(rng, 64, dm["shifts"].shape)
        dm["perms"] = dm["perms"] + (q.random_tbit_uint64s(rng, 40, dm["perms"].shape) // U(dm["b"])) * U(dm["b"])
    assert same_bits(run_fused(r, n, 0, dims), oracle_chain(r, n, 0, dims))


@pytest.mark.parametrize("share", [0.0, 0.3, 1.0])
def test_halton_fp64_share_same_bits(share):
    """Any split of the adds between the FP64 unit and integer arithmetic
    gives the same bits."""
    import torch
    rng = np.random.Generator(np.random.SFC64(21))
    r, n, n_start = 2, 2000, 77
    dims = make_dims(rng, r, PRIMES[:40], n_start + n - 1)
    want = oracle_chain(r, n, n_start, dims)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a).reshape(-1).view(np.int64)).cuda()  # noqa: E731
    ddims = [dict(b=dm["b"], tmax=dm["tmax"], mmax=dm["mmax"], C=dev(dm["C"]), S=dev(dm["S"]), perms=dev(dm["perms"]),
                  shifts=dev(dm["shifts"])) for dm in dims]
    x = torch.empty(r * n * len(dims), dtype=torch.float64, device="cuda")
    plan = halton.HaltonPlan(r, n, n_start, ddims, x)
    plan.set_fp64_share(share)
    plan.prepare()
    plan.run()
    assert same_bits(x.cpu().numpy().reshape(r, n, -1), want)
    # a second run of the same plan (tables reused)
    x.fill_(0)
    plan.run()
    assert same_bits(x.cpu().numpy().reshape(r, n, -1), want)


def test_halton_matrix_entry_above_32_bits_is_reported():
    """Without a linear matrix scramble, generating-matrix entries must stay
    below 2^32 (the kernel reduces them to 32-bit words)."""
    dims = make_dims(None, 1, [3], 9, lms=False, perm=False, shift=False)
    dims[0]["C"] = dims[0]["C"].copy()
    dims[0]["C"][0, 0, 0, 0] = U(1 << 40)
    with pytest.raises(q._ffi.QmcError, match="2\\^32"):
        run_fused(1, 10, 0, dims)


def test_halton_many_dimensions_one_point_per_lane():
    """150 dimensions (bases up to 863): the output tile no longer fits two
    points per lane, so the kernel runs one; same bits as the oracle."""
    big_primes = [p for p in range(2, 900) if all(p % k for k in range(2, int(p ** 0.5) + 1))][:150]
    rng = np.random.Generator(np.random.SFC64(150))
    r, n, n_start = 1, 97, 31
    dims = make_dims(rng, r, big_primes, n_start + n - 1)
    assert same_bits(run_fused(r, n, n_start, dims), oracle_chain(r, n, n_start, dims))


def _dev_dims(dims):
    import torch
    dev = lambda a: None if a is None else torch.from_numpy(np.ascontiguousarray(a).reshape(-1).view(np.int64)).cuda()  # noqa: E731
    return [dict(b=dm["b"], tmax=dm["tmax"], mmax=dm["mmax"], C=dev(dm["C"]), S=dev(dm.get("S")),
                 perms=dev(dm.get("perms")), shifts=dev(dm.get("shifts"))) for dm in dims]


def test_halton_batch_of_uneven_requests():
    """Requests of different r, n, n_start, dimension count, bases, digit
    counts and randomisation steps in one plan (one preparation launch set,
    one generation launch); each request's points equal its oracle chain.
    Replayed from a CUDA graph, twice, with the same bits."""
    import torch
    rng = np.random.Generator(np.random.SFC64(77))
    specs = [  # r, n, n_start, bases, lms, perm, shift
        (2, 300, 5, [2, 3, 5, 7], True, True, True),
        (1, 1000, 0, PRIMES[:40], True, False, True),
        (3, 65, 2 ** 16 - 3, [541, 13, 2], False, True, False),
        (1, 1, 7, [97], True, True, True),
    ]
    reqs, wants = [], []
    for (r, n, n_start, bases, lms, perm, shift) in specs:
        dims = make_dims(rng, r, bases, n_start + n - 1, lms=lms, perm=perm, shift=shift)
        wants.append(oracle_chain(r, n, n_start, dims))
        reqs.append(dict(r=r, n=n, n_start=n_start, dims=_dev_dims(dims),
                         x=torch.full((r * n * len(bases),), float("nan"), dtype=torch.float64, device="cuda")))
    plan = halton.HaltonBatch(reqs)
    st = torch.cuda.Stream()
    for _ in range(2):
        for q in reqs:
            q["x"].fill_(float("nan"))
        plan.graph_launch(st)
        st.synchronize()
        for q, want, (r, n, _ns, bases, *_rest) in zip(reqs, wants, specs):
            assert same_bits(q["x"].cpu().numpy().reshape(r, n, len(bases)), want)
    plan.close()


def test_halton_batch_tune_keeps_bits(tmp_path, monkeypatch):
    """The tuner picks an FP64 share by timing; every share gives the same bits."""
    import torch
    monkeypatch.setenv("QMCGB_TUNE_CACHE", str(tmp_path / "tune.json"))
    rng = np.random.Generator(np.random.SFC64(78))
    r, n, n_start = 2, 4000, 11
    dims = make_dims(rng, r, PRIMES[:24], n_start + n - 1)
    want = oracle_chain(r, n, n_start, dims)
    x = torch.empty(r * n * len(dims), dtype=torch.float64, device="cuda")
    plan = halton.HaltonPlan(r, n, n_start, _dev_dims(dims), x)
    share, ms = plan.tune(reps=2)
    assert 0.0 <= share <= 1.0 and ms > 0
    plan.prepare()
    plan.run()
    assert same_bits(x.cpu().numpy().reshape(r, n, -1), want)
    assert plan.tune(reps=2)[0] == share  # cached


def test_halton_plans_of_different_sizes_coexist():
    """Plans whose output tiles need different shared-memory sizes (above the
    default 48 KB) are created one after the other, then the larger one runs:
    creating the smaller must not lower the kernel's limit below it."""
    import torch
    rng = np.random.Generator(np.random.SFC64(79))
    plans, wants, xs = [], [], []
    for d in (100, 97):
        r, n = 1, 70
        dims = make_dims(rng, r, PRIMES[:d], n - 1)
        wants.append(oracle_chain(r, n, 0, dims))
        x = torch.empty(r * n * d, dtype=torch.float64, device="cuda")
        xs.append(x)
        plans.append(halton.HaltonPlan(r, n, 0, _dev_dims(dims), x))
    for plan, x, want in zip(plans, xs, wants):
        plan.prepare()
        plan.run()
        assert same_bits(x.cpu().numpy().reshape(1, 70, -1), want)
