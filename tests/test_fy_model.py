"""The permutation-stream decoder of fy_stream.cuh, modelled lane for lane on
the CPU (tests/fy_model.py), against numpy's own Generator.permutation: the
same permutations and the same generator state afterwards, for streams that
start with and without a buffered half, bases from 2 to 65536, runs that end
inside a slot and runs that draw nothing."""
import numpy as np
import pytest

from .fy_model import decode, permutation_of
from qmctoolscl_gb300.nus import set_sfc64_state, sfc64_state_words

CASES = [
    [(19, 40)],
    [(2, 100)],
    [(3, 7), (5, 1), (7, 3)],
    [(33, 3), (64, 2), (65, 2)],
    [(541, 2)],
    [(65536, 1)],
    [(11, 0), (1, 5), (13, 4), (0, 2), (2, 1)],
    [(17, 1)] * 12,
    [(1, 3)],
]


@pytest.mark.parametrize("case", range(len(CASES)))
@pytest.mark.parametrize("buffered", [False, True])
@pytest.mark.parametrize("seed", [0, 7])
def test_decoder_matches_numpy(case, buffered, seed):
    runs = CASES[case]
    rng = np.random.Generator(np.random.SFC64(seed))
    if buffered:
        rng.integers(0, 2 ** 16)  # one 32-bit output: the other half waits in numpy's buffer
    words = sfc64_state_words(rng)
    got, after = decode(words, runs)
    for r, (b, nrows) in enumerate(runs):
        for q in range(nrows):
            want = rng.permutation(b) if b >= 1 else np.arange(0)
            if b >= 2:
                assert permutation_of(got[r][q]) == list(want), (r, q)
    assert [int(x) for x in sfc64_state_words(rng)] == after


def test_state_round_trip_continues_the_stream():
    rng = np.random.Generator(np.random.SFC64(3))
    words = sfc64_state_words(rng)
    _rows, after = decode(words, [(23, 5)])
    twin = np.random.Generator(np.random.SFC64(0))
    set_sfc64_state(twin, np.array(after, dtype=np.uint64))
    for _ in range(5):
        rng.permutation(23)
    assert np.array_equal(rng.integers(0, 1 << 62, 50), twin.integers(0, 1 << 62, 50))


def _numpy_rows(rng, runs):
    return [[list(rng.permutation(b)) if b >= 2 else None for _ in range(n)] for b, n in runs]


@pytest.mark.parametrize("case", range(len(CASES)))
@pytest.mark.parametrize("buffered", [False, True])
def test_general_decoder_matches_numpy(case, buffered):
    from .fy_model import decode_runs
    runs = CASES[case]
    rng = np.random.Generator(np.random.SFC64(11))
    if buffered:
        rng.integers(0, 2 ** 16)
    got, after = decode_runs(sfc64_state_words(rng), runs)
    want = _numpy_rows(rng, runs)
    for r, (b, n) in enumerate(runs):
        for qq in range(n):
            if b >= 2:
                assert permutation_of(got[r][qq]) == want[r][qq], (r, qq)
    assert [int(x) for x in sfc64_state_words(rng)] == after


@pytest.mark.parametrize("b,nrows", [(2, 70), (3, 40), (5, 9), (19, 30), (32, 4), (33, 5), (17, 1), (9, 0)])
@pytest.mark.parametrize("buffered", [False, True])
def test_small_base_decoder_matches_numpy(b, nrows, buffered):
    from .fy_model import decode_small
    rng = np.random.Generator(np.random.SFC64(b * 7 + nrows))
    if buffered:
        rng.integers(0, 2 ** 16)
    got, after = decode_small(sfc64_state_words(rng), b, nrows)
    for qq in range(nrows):
        assert permutation_of(got[qq]) == list(rng.permutation(b)), qq
    assert [int(x) for x in sfc64_state_words(rng)] == after
