"""Argument lists of the 23 QMCToolsCL hot-path functions.

Each entry gives the Python-level argument list of one reference function, in
the reference's order, with the three batch-size arguments removed (the
generated Python stubs drop them, pdm_build.py:78, and the C wrapper fills
them with the full extents, qmctoolscl/util.py:107).  The C signatures they
come from are the ``EXPORT void <name>(...)`` headers in
qmctoolscl/c_funcs/<name>.c:3-16.

Kinds:
    "u64"   scalar, passed as np.uint64 / c_uint64
    "u64*"  C-contiguous np.uint64 array
    "f64*"  C-contiguous np.float64 array

``outputs`` names the arrays the function writes.  The transforms work in
place, and the FFT/IFFT also overwrite both twiddle arrays.
"""

U, PU, PF = "u64", "u64*", "f64*"

SIGNATURES = {
    # rank-1 lattices
    "lat_gen_linear": ([("r", U), ("n", U), ("d", U), ("g", PU), ("x", PF)], ("x",)),
    "lat_gen_natural": ([("r", U), ("n", U), ("d", U), ("n_start", U), ("g", PU), ("x", PF)], ("x",)),
    "lat_gen_gray": ([("r", U), ("n", U), ("d", U), ("n_start", U), ("g", PU), ("x", PF)], ("x",)),
    "lat_shift_mod_1": ([("r", U), ("n", U), ("d", U), ("r_x", U), ("x", PF), ("shifts", PF),
                         ("xr", PF)], ("xr",)),
    # digital nets in base 2
    "dnb2_gen_natural": ([("r", U), ("n", U), ("d", U), ("n_start", U), ("mmax", U), ("C", PU),
                          ("xb", PU)], ("xb",)),
    "dnb2_gen_gray": ([("r", U), ("n", U), ("d", U), ("n_start", U), ("mmax", U), ("C", PU),
                       ("xb", PU)], ("xb",)),
    "dnb2_digital_shift": ([("r", U), ("n", U), ("d", U), ("r_x", U), ("lshifts", PU), ("xb", PU),
                            ("shiftsb", PU), ("xrb", PU)], ("xrb",)),
    "dnb2_integer_to_float": ([("r", U), ("n", U), ("d", U), ("tmaxes", PU), ("xb", PU),
                               ("x", PF)], ("x",)),
    "dnb2_linear_matrix_scramble": ([("r", U), ("d", U), ("mmax", U), ("r_C", U), ("tmax_new", U),
                                     ("S", PU), ("C", PU), ("C_lms", PU)], ("C_lms",)),
    "dnb2_interlace": ([("r", U), ("d_alpha", U), ("mmax", U), ("d", U), ("tmax", U),
                        ("tmax_alpha", U), ("alpha", U), ("C", PU), ("C_alpha", PU)], ("C_alpha",)),
    "dnb2_undo_interlace": ([("r", U), ("d", U), ("mmax", U), ("d_alpha", U), ("tmax", U),
                             ("tmax_alpha", U), ("alpha", U), ("C_alpha", PU), ("C", PU)], ("C",)),
    "dnb2_gmat_lsb_to_msb": ([("r", U), ("d", U), ("mmax", U), ("tmaxes", PU), ("C_lsb", PU),
                              ("C_msb", PU)], ("C_msb",)),
    # generalized digital nets
    "gdn_gen_natural": ([("r", U), ("n", U), ("d", U), ("r_b", U), ("mmax", U), ("tmax", U),
                         ("n_start", U), ("bases", PU), ("C", PU), ("xdig", PU)], ("xdig",)),
    "gdn_gen_natural_same_base": ([("r", U), ("n", U), ("d", U), ("mmax", U), ("tmax", U),
                                   ("n_start", U), ("b", U), ("C", PU), ("xdig", PU)], ("xdig",)),
    "gdn_linear_matrix_scramble": ([("r", U), ("d", U), ("mmax", U), ("r_C", U), ("r_b", U),
                                    ("tmax", U), ("tmax_new", U), ("bases", PU), ("S", PU),
                                    ("C", PU), ("C_lms", PU)], ("C_lms",)),
    "gdn_digital_permutation": ([("r", U), ("n", U), ("d", U), ("r_x", U), ("r_b", U), ("tmax", U),
                                 ("tmax_new", U), ("bmax", U), ("perms", PU), ("xdig", PU),
                                 ("xdig_new", PU)], ("xdig_new",)),
    "gdn_digital_shift": ([("r", U), ("n", U), ("d", U), ("r_x", U), ("r_b", U), ("tmax", U),
                           ("tmax_new", U), ("bases", PU), ("shifts", PU), ("xdig", PU),
                           ("xdig_new", PU)], ("xdig_new",)),
    "gdn_integer_to_float": ([("r", U), ("n", U), ("d", U), ("r_b", U), ("tmax", U), ("bases", PU),
                              ("xdig", PU), ("x", PF)], ("x",)),
    "gdn_interlace": ([("r", U), ("d_alpha", U), ("mmax", U), ("d", U), ("tmax", U),
                       ("tmax_alpha", U), ("alpha", U), ("C", PU), ("C_alpha", PU)], ("C_alpha",)),
    "gdn_undo_interlace": ([("r", U), ("d", U), ("mmax", U), ("d_alpha", U), ("tmax", U),
                            ("tmax_alpha", U), ("alpha", U), ("C_alpha", PU), ("C", PU)], ("C",)),
    # fast transforms
    "fft_bro_1d_radix2": ([("d1", U), ("d2", U), ("n_half", U), ("twiddler", PF), ("twiddlei", PF),
                           ("xr", PF), ("xi", PF)], ("twiddler", "twiddlei", "xr", "xi")),
    "ifft_bro_1d_radix2": ([("d1", U), ("d2", U), ("n_half", U), ("twiddler", PF), ("twiddlei", PF),
                            ("xr", PF), ("xi", PF)], ("twiddler", "twiddlei", "xr", "xi")),
    "fwht_1d_radix2": ([("d1", U), ("d2", U), ("n_half", U), ("x", PF)], ("x",)),
}

NAMES = tuple(SIGNATURES)
