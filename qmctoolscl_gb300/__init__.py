"""qmctoolscl_gb300: the QMCToolsCL point-generation and fast-transform hot
path on one NVIDIA GB300 (sm_103a).

Drop-in for ``import qmctoolscl``: the 23 kernel functions (lat_*, dnb2_*,
gdn_*, fft_bro_1d_radix2, ifft_bro_1d_radix2, fwht_1d_radix2) take the same
arguments and return the same (t_perf, t_process) tuple, and the host-side
random-input helpers (lat_get_shifts, dnb2_get_linear_scramble_matrix, ...)
produce the same arrays from the same numpy Generator state.  The kernels
run only on the GPU, through the C ABI of libqmcgb.so (include/qmcgb.h).

Beyond the reference's surface: ``qmctoolscl_gb300.batch`` (fused pipelines,
batched uneven requests in one persistent launch, CUDA-graph replay) and
``qmctoolscl_gb300.tc_fft`` (tensor-core FFT/FWHT).
"""
__version__ = "1.2.1"

from .rand_funcs import *  # noqa: F401,F403
from .nus import NUSNode_dnb2, NUSNode_gdn, dnb2_nested_uniform_scramble, gdn_nested_uniform_scramble  # noqa: F401
from .api import (  # noqa: F401
    lat_gen_linear,
    lat_gen_natural,
    lat_gen_gray,
    lat_shift_mod_1,
    dnb2_gen_natural,
    dnb2_gen_gray,
    dnb2_digital_shift,
    dnb2_integer_to_float,
    dnb2_linear_matrix_scramble,
    dnb2_interlace,
    dnb2_undo_interlace,
    dnb2_gmat_lsb_to_msb,
    gdn_gen_natural,
    gdn_gen_natural_same_base,
    gdn_linear_matrix_scramble,
    gdn_digital_permutation,
    gdn_digital_shift,
    gdn_integer_to_float,
    gdn_interlace,
    gdn_undo_interlace,
    fft_bro_1d_radix2,
    ifft_bro_1d_radix2,
    fwht_1d_radix2,
)
