"""Host-side behaviour of the drop-in API that needs no GPU: argument
conversion, the reference's own checks and exceptions, size validation."""
import ctypes

import numpy as np
import pytest

import qmctoolscl_gb300 as q
from qmctoolscl_gb300 import api

U = np.uint64


def test_lat_gen_natural_power_of_two_check():
    # qmctoolscl/util.py:84-86 raises a plain Exception with this message
    with pytest.raises(Exception, match="either 0 or powers of 2"):
        q.lat_gen_natural(U(1), U(3), U(2), U(0), np.ones((1, 2), U), np.empty((1, 3, 2)))
    with pytest.raises(Exception, match="either 0 or powers of 2"):
        q.lat_gen_natural(U(1), U(4), U(2), U(3), np.ones((1, 2), U), np.empty((1, 4, 2)))


@pytest.mark.parametrize("bad", [np.ones((1, 2), np.int64), np.ones((1, 2), np.float64),
                                 np.ones((1, 4), U)[:, ::2]])
def test_array_type_errors_like_ndpointer(bad):
    with pytest.raises(ctypes.ArgumentError):
        q.lat_gen_gray(U(1), U(3), U(2), U(0), bad, np.empty((1, 3, 2)))


def test_scalar_type_errors():
    with pytest.raises(ctypes.ArgumentError):
        q.lat_gen_gray(1.5, U(3), U(2), U(0), np.ones((1, 2), U), np.empty((1, 3, 2)))


def test_backend_keyword():
    with pytest.raises(AssertionError):
        q.lat_gen_gray(U(1), U(3), U(2), U(0), np.ones((1, 2), U), np.empty((1, 3, 2)), backend="cuda")


def test_short_arrays_rejected_before_any_launch():
    with pytest.raises(ValueError, match="needs"):
        q.lat_gen_gray(U(2), U(3), U(2), U(0), np.ones((1, 2), U), np.empty((2, 3, 2)))
    with pytest.raises(ValueError, match="needs"):
        q.dnb2_gen_natural(U(1), U(8), U(2), U(0), U(3), np.ones((1, 2, 2), U), np.empty((1, 8, 2), U))


def test_positional_count():
    with pytest.raises(TypeError):
        q.lat_gen_gray(U(1), U(3), U(2), np.ones((1, 2), U), np.empty((1, 3, 2)))


def test_need_table_covers_signatures():
    from qmctoolscl_gb300._signatures import SIGNATURES
    for name, (spec, outs) in SIGNATURES.items():
        s = {a: 3 for a, k in spec if k == "u64"}
        need = api.NEED[name](s)
        assert set(need) == {a for a, k in spec if k != "u64"}, name
        assert set(outs) <= set(need)


def test_no_cpu_fallback_without_gpu():
    """Without a CUDA device the call fails loudly instead of computing on the host."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(Exception, match="CUDA|libqmcgb"):
        q.lat_gen_gray(U(1), U(4), U(2), U(0), np.ones((1, 2), U), np.empty((1, 4, 2)))
