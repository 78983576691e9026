"""The randomisation helpers on the GPU (qmctoolscl_gb300.rand_funcs with
device=..., C entry points qmc_lat_get_shifts ... qmc_random_uint64_permutations)
against the same helpers on numpy (the reference's own calls,
qmctoolscl/rand_funcs.py:4-153): arrays equal bit for bit and the Generators
left in equal states, over every bit count, bases that make numpy's Lemire
rule reject often (32- and 64-bit), bases where integers(1, b) draws nothing,
a buffered 32-bit half at the start, replicated bases, and a device-resident
generator running the per-dimension sequence of the randomised Halton inputs."""
import numpy as np
import pytest

import qmctoolscl_gb300 as q
from qmctoolscl_gb300.nus import sfc64_state_words

pytestmark = pytest.mark.gpu
U = np.uint64


def _pair(seed, pre32=0):
    """two Generators in the same state; pre32 draws of 32 bits leave a buffered half"""
    a, b = (np.random.Generator(np.random.SFC64(seed)) for _ in range(2))
    if pre32:
        a.integers(0, 1 << 20, pre32)
        b.integers(0, 1 << 20, pre32)
    return a, b


def _same(host, dev, ga, gb):
    got = dev.cpu().numpy()
    if host.dtype == np.uint64:
        got = got.view(U)
    assert got.shape == host.shape
    assert np.array_equal(got.view(U) if got.dtype == np.float64 else got,
                          host.view(U) if host.dtype == np.float64 else host)
    assert np.array_equal(sfc64_state_words(ga), sfc64_state_words(gb))


@pytest.mark.parametrize("pre32", [0, 1])
def test_lat_get_shifts(pre32):
    ga, gb = _pair(11, pre32)
    _same(q.lat_get_shifts(ga, 7, 13), q.lat_get_shifts(gb, 7, 13, device="cuda"), ga, gb)


@pytest.mark.parametrize("t", [0, 1, 5, 31, 32, 33, 52, 63, 64])
@pytest.mark.parametrize("pre32", [0, 1])
def test_random_tbit_uint64s(t, pre32):
    ga, gb = _pair(100 + t, pre32)
    _same(q.random_tbit_uint64s(ga, t, (3, 37)), q.random_tbit_uint64s(gb, t, (3, 37), device="cuda"), ga, gb)


@pytest.mark.parametrize("tmax_new", [1, 17, 63, 64])
def test_dnb2_get_digital_shifts(tmax_new):
    ga, gb = _pair(200 + tmax_new, 1)
    _same(q.dnb2_get_digital_shifts(ga, 5, 9, tmax_new), q.dnb2_get_digital_shifts(gb, 5, 9, tmax_new, device=0),
          ga, gb)


@pytest.mark.parametrize("tmax,tmax_new", [(1, 1), (20, 20), (32, 40), (33, 33), (63, 64), (64, 64), (64, 70)])
def test_dnb2_get_linear_scramble_matrix(tmax, tmax_new):
    ga, gb = _pair(300 + tmax, 1)
    _same(q.dnb2_get_linear_scramble_matrix(ga, 3, 4, tmax, tmax_new, False),
          q.dnb2_get_linear_scramble_matrix(gb, 3, 4, tmax, tmax_new, False, device="cuda"), ga, gb)


def test_dnb2_linear_scramble_matrix_refuses_what_numpy_refuses():
    ga, gb = _pair(7)
    with pytest.raises(ValueError):
        q.dnb2_get_linear_scramble_matrix(ga, 2, 2, 10, 8, False)
    with pytest.raises(ValueError):
        q.dnb2_get_linear_scramble_matrix(gb, 2, 2, 10, 8, False, device="cuda")


# bases: small primes; 2 (the diagonal's integers(1, 2) draws nothing); 3e9 (32-bit Lemire
# rejects about 30 % of draws); replicated bases (r_b = 2)
GDN_BASES = [np.array([[2, 3, 5]], U), np.array([[541, 2, 7919]], U), np.array([[3000000019, 3, 65536]], U),
             np.array([[3, 5, 7], [11, 13, 2]], U)]


@pytest.mark.parametrize("k", range(len(GDN_BASES)))
@pytest.mark.parametrize("tmax,tmax_new", [(1, 1), (6, 6), (5, 9)])
def test_gdn_get_linear_scramble_matrix(k, tmax, tmax_new):
    bases = GDN_BASES[k]
    r_b, d = bases.shape
    ga, gb = _pair(400 + k, k % 2)
    _same(q.gdn_get_linear_scramble_matrix(ga, 3, d, tmax, tmax_new, r_b, bases),
          q.gdn_get_linear_scramble_matrix(gb, 3, d, tmax, tmax_new, r_b, bases, device="cuda"), ga, gb)


@pytest.mark.parametrize("k", range(len(GDN_BASES)))
def test_gdn_get_digital_shifts(k):
    bases = GDN_BASES[k]
    r_b, d = bases.shape
    ga, gb = _pair(500 + k, 1 - k % 2)
    _same(q.gdn_get_digital_shifts(ga, 4, d, 9, r_b, bases),
          q.gdn_get_digital_shifts(gb, 4, d, 9, r_b, bases, device="cuda"), ga, gb)


def test_gdn_digital_shifts_with_64_bit_lemire_rejections():
    """bases above 2^32 take numpy's 64-bit Lemire rule; 2^63 + 5 rejects about half its draws"""
    bases = np.array([[(1 << 63) + 5, (1 << 40) + 3, 1]], U)
    ga, gb = _pair(550)
    _same(q.gdn_get_digital_shifts(ga, 5, 3, 40, 1, bases),
          q.gdn_get_digital_shifts(gb, 5, 3, 40, 1, bases, device="cuda"), ga, gb)


@pytest.mark.parametrize("bases", [np.array([[2, 3, 5, 541]], U), np.array([[1, 2], [17, 3]], U),
                                   np.array([[65536, 3]], U), np.array([[5, 5, 5]], U), np.array([[33, 34]], U),
                                   np.array([[19], [19]], U)])
@pytest.mark.parametrize("pre32", [0, 1])
def test_gdn_get_digital_permutations(bases, pre32):
    """mixed bases (runs of rows of changing base), one small base for every
    row (the all-start-positions decoder over merged rows), bases either side
    of its limit of 33, with and without a buffered half"""
    r_b, d = bases.shape
    ga, gb = _pair(600 + int(bases.max()) % 97, pre32)
    _same(q.gdn_get_digital_permutations(ga, 2, d, 3, r_b, bases),
          q.gdn_get_digital_permutations(gb, 2, d, 3, r_b, bases, device="cuda"), ga, gb)


@pytest.mark.parametrize("n,b", [(1, 1), (5, 2), (40, 7), (300, 541), (3, 4097), (2000, 19), (70, 33), (70, 34),
                                 (5000, 2)])
@pytest.mark.parametrize("pre32", [0, 1])
def test_random_uint64_permutations(n, b, pre32):
    ga, gb = _pair(700 + b, pre32)
    _same(q.random_uint64_permutations(ga, n, b), q.random_uint64_permutations(gb, n, b, device="cuda"), ga, gb)


def test_device_generator_runs_the_halton_input_sequence():
    """the per-dimension sequence of the randomised Halton workload (scrambling
    matrices, permutations, shifts for each base in turn) from one
    device-resident generator, against numpy, then the state back"""
    import math
    ga, gb = _pair(800)
    dg = q.DeviceGenerator(gb)
    for b in (2, 3, 5, 7, 11, 13, 541):
        tmax = math.ceil(64 / math.log2(b))
        bb = np.array([[b]], U)
        for host_fn, args in ((q.gdn_get_linear_scramble_matrix, (4, 1, tmax, tmax, 1, bb)),
                              (q.gdn_get_digital_permutations, (4, 1, tmax, 1, bb)),
                              (q.gdn_get_digital_shifts, (4, 1, tmax, 1, bb))):
            want = host_fn(ga, *args)
            got = host_fn(dg, *args)
            assert np.array_equal(got.cpu().numpy().view(U), want), (b, host_fn.__name__)
    dg.sync()
    assert np.array_equal(sfc64_state_words(ga), sfc64_state_words(gb))


def test_gpu_form_refusals_before_any_draw():
    g = np.random.Generator(np.random.SFC64(9))
    before = sfc64_state_words(g)
    with pytest.raises(ValueError):
        q.gdn_get_linear_scramble_matrix(g, 1, 1, 3, 3, 1, np.array([[1]], U), device="cuda")
    with pytest.raises(ValueError):
        q.gdn_get_digital_permutations(g, 1, 1, 3, 1, np.array([[70000]], U), device="cuda")
    with pytest.raises(AssertionError):
        q.random_tbit_uint64s(g, 65, 3, device="cuda")
    assert np.array_equal(sfc64_state_words(g), before)
