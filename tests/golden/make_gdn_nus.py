"""Golden vectors for gdn_nested_uniform_scramble
(qmctoolscl/rand_funcs.py:255-356) from the reference's own Python code,
imported from a QMCToolsCL checkout (--ref, or $QMCTOOLSCL_REF).

    python tests/golden/make_gdn_nus.py [--ref /path/to/QMCToolsCL]

Each case: the scalars (r, n, d, r_x, r_b, tmax, tmax_new), the bases, the
generator states before the first call (six words per SFC64 generator), and
per call on the same root nodes the digits xdig, the output xrdig and the
states after the call.  The first case is the reference's documented example
(docs/index.md, generalized nets, "nested uniform scramble"); the script
checks that the reference prints the documented array for it.  Every case
keeps tmax_new above tmax, where the reference's walk is defined for every
input (with tmax_new = tmax it raises IndexError when a point repeats an
earlier one to its last digit).  Writes tests/golden/gdn_nus.npz.
"""
import argparse
import importlib.util
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from qmctoolscl_gb300.nus import sfc64_state_words  # noqa: E402


def load_ref_rand_funcs(ref):
    spec = importlib.util.spec_from_file_location("ref_rand_funcs", os.path.join(ref, "qmctoolscl", "rand_funcs.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def documented_xrdig(ref):
    with open(os.path.join(ref, "docs", "index.md")) as f:
        doc = f.read()
    sec = doc[doc.index("## Generalized Digital Net"):]
    sec = sec[sec.index("### nested uniform scramble"):]
    sec = sec[sec.index(">>> xrdig"):]
    sec = sec[sec.index("array("):]
    body = sec[:sec.index("dtype=uint64)")]
    return np.array([int(v) for v in re.findall(r"\d+", body)], dtype=np.uint64)


def gens(seed, count, warm):
    out = [np.random.Generator(np.random.SFC64(s)) for s in np.random.SeedSequence(seed).spawn(count)]
    if warm:
        for k, g in enumerate(out):
            for _ in range(k % 3):
                g.integers(0, 2 ** (5 + 7 * k % 50))
    return out


def natural_digits(r_x, n, d, r_b, tmax, bases):
    """xdig of gdn_gen_natural with identity matrices (the base-b digits of i,
    least significant first), by the oracle."""
    C = np.tile(np.eye(tmax, dtype=np.uint64)[None, None, :, :], (r_x, d, 1, 1))
    xdig = np.zeros((r_x, n, d, tmax), dtype=np.uint64)
    oracle.call("gdn_gen_natural", r_x, n, d, r_b, tmax, tmax, 0, np.ascontiguousarray(bases), C, xdig)
    return xdig


def main():
    ap = argparse.ArgumentParser()
    env_ref = os.environ.get("QMCTOOLSCL_REF")
    ap.add_argument("--ref", default=env_ref, required=env_ref is None,
                    help="QMCToolsCL checkout (default: $QMCTOOLSCL_REF)")
    a = ap.parse_args()
    rf = load_ref_rand_funcs(a.ref)
    rng = np.random.Generator(np.random.SFC64(41))
    cases = []
    # 1. the documented example
    b0 = np.array([[2, 3, 5]], dtype=np.uint64)
    cases.append(dict(r=2, n=9, d=3, r_x=1, r_b=1, tmax=3, tmax_new=8, bases=b0, seed=7, warm=False,
                      xdigs=[natural_digits(1, 9, 3, 1, 3, b0)]))

    def rnd_digits(r_x, n, d, r_b, tmax, bases, low=False):
        bmin = bases.min(axis=0)  # per dimension, valid for every replication of the bases
        x = rng.integers(0, 1 << 30, (r_x, n, d, tmax), dtype=np.uint64)
        cap = np.uint64(2) if low else bmin[None, None, :, None]
        return x % np.minimum(cap, bmin[None, None, :, None])

    b = np.array([[2, 3, 7]], dtype=np.uint64)
    cases.append(dict(r=3, n=40, d=3, r_x=3, r_b=1, tmax=6, tmax_new=9, bases=b, seed=1, warm=True,
                      xdigs=[rnd_digits(3, 40, 3, 1, 6, b)]))
    b = np.array([[3, 5], [11, 2]], dtype=np.uint64)
    cases.append(dict(r=4, n=30, d=2, r_x=2, r_b=2, tmax=5, tmax_new=7, bases=b, seed=2, warm=True,
                      xdigs=[rnd_digits(2, 30, 2, 2, 5, b, low=True), rnd_digits(2, 30, 2, 2, 5, b)]))
    b = np.array([[541]], dtype=np.uint64)
    cases.append(dict(r=1, n=12, d=1, r_x=1, r_b=1, tmax=3, tmax_new=4, bases=b, seed=3, warm=True,
                      xdigs=[rnd_digits(1, 12, 1, 1, 3, b)]))
    b = np.array([[2]], dtype=np.uint64)
    cases.append(dict(r=2, n=64, d=1, r_x=1, r_b=1, tmax=6, tmax_new=12, bases=b, seed=4, warm=False,
                      xdigs=[natural_digits(1, 64, 1, 1, 6, b)]))
    b = np.array([[3, 2]], dtype=np.uint64)
    cases.append(dict(r=1, n=0, d=2, r_x=1, r_b=1, tmax=4, tmax_new=6, bases=b, seed=5, warm=True,
                      xdigs=[np.zeros((1, 0, 2, 4), np.uint64), rnd_digits(1, 5, 2, 1, 4, b)[:, :0]]))
    b = np.array([[5, 3, 2]], dtype=np.uint64)
    cases.append(dict(r=2, n=27, d=3, r_x=1, r_b=1, tmax=3, tmax_new=5, bases=b, seed=6, warm=True,
                      xdigs=[natural_digits(1, 27, 3, 1, 3, b), natural_digits(1, 27, 3, 1, 3, b)]))

    out = {}
    for c, cs in enumerate(cases):
        r, n, d = cs["r"], cs["n"], cs["d"]
        g = gens(cs["seed"], r * d, cs["warm"])
        rngs = np.array(g, dtype=object).reshape(r, d)
        roots = np.array([rf.NUSNode_gdn() for _ in range(r * d)]).reshape(r, d)
        out["case%d_args" % c] = np.array([r, n, d, cs["r_x"], cs["r_b"], cs["tmax"], cs["tmax_new"],
                                           len(cs["xdigs"])], np.uint64)
        out["case%d_bases" % c] = cs["bases"]
        out["case%d_state0" % c] = np.stack([sfc64_state_words(x) for x in g])
        for k, xdig in enumerate(cs["xdigs"]):
            xr = np.zeros((r, n, d, cs["tmax_new"]), dtype=np.uint64)
            rf.gdn_nested_uniform_scramble(np.uint64(r), np.uint64(n), np.uint64(d), np.uint64(cs["r_x"]),
                                           np.uint64(cs["r_b"]), np.uint64(cs["tmax"]), np.uint64(cs["tmax_new"]),
                                           rngs, roots, cs["bases"], xdig, xr)
            out["case%d_xdig%d" % (c, k)] = xdig
            out["case%d_xrdig%d" % (c, k)] = xr
            out["case%d_state%d" % (c, k + 1)] = np.stack([sfc64_state_words(x) for x in g])
        if c == 0:
            assert np.array_equal(out["case0_xrdig0"].reshape(-1), documented_xrdig(a.ref)), \
                "reference differs from its documentation"
    np.savez_compressed(os.path.join(HERE, "gdn_nus.npz"), **out)
    print("wrote %d cases" % len(cases))


if __name__ == "__main__":
    main()
