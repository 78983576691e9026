"""Golden vectors for halton_qrng (qmctoolscl/c_funcs/halton_qrng.c:3-162)
from the reference's own compiled C (oracle/_ref/c_lib.so, built by
`make -C oracle ref` where the reference checkout is).  Writes
tests/golden/halton_qrng.npz: seeded cases over n, d, n0, generalized and
the dimension indices, each with its inputs and the reference's output.

    python tests/golden/make_halton_qrng.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402

CASES = [  # (n, d, n0, generalized, dimension indices or None for 0..d-1)
    (16, 3, 0, 1, None), (16, 3, 0, 0, None), (37, 5, 4, 1, None), (100, 2, 1, 0, None),
    (64, 8, 1000, 1, [359, 0, 1, 200, 17, 300, 5, 99]), (1, 4, 0, 1, None), (5, 1, 123456, 0, [358]),
    (257, 12, 0, 1, list(range(0, 360, 30))), (33, 6, 2 ** 20, 1, [0, 1, 2, 3, 4, 5]),
]


def main():
    if not oracle.ref_available():
        oracle.build(ref=True)
    rng = np.random.Generator(np.random.SFC64(2024))
    out = {}
    for c, (n, d, n0, gen, dv) in enumerate(CASES):
        dvec = np.array(dv if dv is not None else list(range(d)), dtype=np.int32)
        randu = rng.random(d * 32)
        res = np.full(d * n, np.nan)
        oracle.halton_qrng_ref(n, d, n0, gen, res, randu, dvec)
        out["case%d_args" % c] = np.array([n, d, n0, gen], dtype=np.int64)
        out["case%d_dvec" % c] = dvec
        out["case%d_randu" % c] = randu
        out["case%d_res" % c] = res
    np.savez_compressed(os.path.join(HERE, "halton_qrng.npz"), **out)
    print("wrote %d cases" % len(CASES))


if __name__ == "__main__":
    main()
