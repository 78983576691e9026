"""Golden vectors for dnb2_nested_uniform_scramble
(qmctoolscl/rand_funcs.py:155-253) from the reference's own Python code,
imported from a QMCToolsCL checkout (--ref, or $QMCTOOLSCL_REF).

    python tests/golden/make_nus.py [--ref /path/to/QMCToolsCL]

Each case holds: the scalars (r, n, d, r_x, tmax, tmax_new), the generator
states before the first call (numpy SFC64 Generators, six words per
generator: a, b, c, w, has_uint32, uinteger), and for each of its calls on
the same root nodes the input points xb, the output xrb and the generator
states after the call.  The first case is the reference's documented example
(docs/index.md, "nested uniform scrambling"); the script checks that the
reference prints the documented array for it.  Writes tests/golden/nus.npz.
"""
import argparse
import importlib.util
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from qmctoolscl_gb300.nus import sfc64_state_words  # noqa: E402


def load_ref_rand_funcs(ref):
    spec = importlib.util.spec_from_file_location("ref_rand_funcs", os.path.join(ref, "qmctoolscl", "rand_funcs.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def documented_xrb(ref):
    """The array the documentation prints after the nested uniform scramble."""
    with open(os.path.join(ref, "docs", "index.md")) as f:
        doc = f.read()
    sec = doc[doc.index("### nested uniform scrambling"):]
    sec = sec[sec.index(">>> xrb\n") + len(">>> xrb\n"):]
    body = sec[:sec.index("dtype=uint64)")]
    nums = [int(v) for v in re.findall(r"\d+", body)]
    return np.array(nums, dtype=np.uint64)


def gens(seed, count, warm):
    """count SFC64 Generators spawned from SeedSequence(seed); with warm, each
    first draws a few bits so that some start with a buffered 32-bit half."""
    out = [np.random.Generator(np.random.SFC64(s)) for s in np.random.SeedSequence(seed).spawn(count)]
    if warm:
        for k, g in enumerate(out):
            for _ in range(k % 3):
                g.integers(0, 2 ** (5 + 7 * k % 50))
    return out


def net_points(r_x, n, d, m, rng):
    """Natural-order base-2 net points from random upper-unit-triangular matrices
    (MSB-first in m bits), as the reference's dnb2_gen_natural computes them."""
    C = np.zeros((d, m), dtype=np.uint64)
    for j in range(d):
        for k in range(m):
            col = 1 << (m - 1 - k)
            for t in range(k):
                if rng.integers(0, 2):
                    col |= 1 << (m - 1 - t)
            C[j, k] = col
    xb = np.zeros((r_x, n, d), dtype=np.uint64)
    for i in range(n):
        for j in range(d):
            v = 0
            for k in range(m):
                if (i >> k) & 1:
                    v ^= int(C[j, k])
            xb[:, i, j] = v
    return xb


def main():
    ap = argparse.ArgumentParser()
    env_ref = os.environ.get("QMCTOOLSCL_REF")
    ap.add_argument("--ref", default=env_ref, required=env_ref is None,
                    help="QMCToolsCL checkout (default: $QMCTOOLSCL_REF)")
    a = ap.parse_args()
    rf = load_ref_rand_funcs(a.ref)
    rng = np.random.Generator(np.random.SFC64(31))
    cases = []

    # 1. the documented example
    C = np.array([[8, 4, 2, 1], [8, 12, 10, 15], [8, 12, 6, 9], [8, 12, 2, 5]], dtype=np.uint64)
    xb = np.zeros((1, 8, 4), dtype=np.uint64)
    for i in range(8):
        for j in range(4):
            v = 0
            for k in range(4):
                if (i >> k) & 1:
                    v ^= int(C[j, k])
            xb[0, i, j] = v
    cases.append(dict(r=2, n=8, d=4, r_x=1, tmax=4, tmax_new=8, seed=7, warm=False, xbs=[xb]))

    # 2. seeded cases: random words, duplicates and shared prefixes, net points,
    #    64-bit keys, one-bit keys, a continuation call on the same root nodes,
    #    a call with no points, words with bits above tmax
    def rnd(r_x, n, d, tmax):
        hi = 1 << tmax
        return rng.integers(0, hi, (r_x, n, d), dtype=np.uint64) if tmax < 64 else \
            rng.integers(0, 2 ** 63, (r_x, n, d), dtype=np.uint64) * np.uint64(2) + rng.integers(0, 2, (r_x, n, d),
                                                                                               dtype=np.uint64)
    cases.append(dict(r=3, n=50, d=2, r_x=3, tmax=20, tmax_new=20, seed=1, warm=True, xbs=[rnd(3, 50, 2, 20)]))
    cases.append(dict(r=2, n=40, d=3, r_x=1, tmax=64, tmax_new=64, seed=2, warm=True, xbs=[rnd(1, 40, 3, 64)]))
    dup = rng.integers(0, 4, (2, 60, 2), dtype=np.uint64) << np.uint64(10)
    cases.append(dict(r=4, n=60, d=2, r_x=2, tmax=12, tmax_new=40, seed=3, warm=True, xbs=[dup]))
    cases.append(dict(r=2, n=64, d=3, r_x=1, tmax=16, tmax_new=64, seed=4, warm=False,
                      xbs=[net_points(1, 64, 3, 6, rng) << np.uint64(10)]))
    cases.append(dict(r=2, n=30, d=2, r_x=2, tmax=1, tmax_new=1, seed=5, warm=True, xbs=[rnd(2, 30, 2, 1)]))
    cases.append(dict(r=2, n=25, d=2, r_x=1, tmax=10, tmax_new=33, seed=6, warm=True,
                      xbs=[rnd(1, 25, 2, 10), rnd(1, 25, 2, 10), rnd(1, 25, 2, 10)]))
    cases.append(dict(r=1, n=0, d=3, r_x=1, tmax=8, tmax_new=32, seed=8, warm=True,
                      xbs=[np.zeros((1, 0, 3), np.uint64)]))
    cases.append(dict(r=2, n=20, d=2, r_x=1, tmax=3, tmax_new=5, seed=9, warm=False,
                      xbs=[rng.integers(0, 64, (1, 20, 2), dtype=np.uint64)]))
    cases.append(dict(r=1, n=200, d=2, r_x=1, tmax=64, tmax_new=64, seed=10, warm=True,
                      xbs=[net_points(1, 200, 2, 8, rng) << np.uint64(56)]))
    cases.append(dict(r=2, n=16, d=1, r_x=2, tmax=63, tmax_new=64, seed=11, warm=True,
                      xbs=[rnd(2, 16, 1, 63), net_points(2, 16, 1, 4, rng) << np.uint64(59)]))
    # tmax above tmax_new: the reference's uint64 shift count wraps and numpy shifts to 0
    cases.append(dict(r=1, n=12, d=2, r_x=1, tmax=20, tmax_new=12, seed=12, warm=True, xbs=[rnd(1, 12, 2, 20)]))
    # no bits at all (tmax_new = 0): every point repeats the root
    cases.append(dict(r=2, n=5, d=1, r_x=1, tmax=0, tmax_new=0, seed=13, warm=True,
                      xbs=[np.zeros((1, 5, 1), np.uint64)]))
    # r = 3 r_x, 32-bit keys drawn as 32-bit halves, a continuation call
    cases.append(dict(r=6, n=40, d=2, r_x=2, tmax=32, tmax_new=32, seed=14, warm=True,
                      xbs=[rnd(2, 40, 2, 32), rnd(2, 40, 2, 32)]))
    # a longer net: 1024 points of 3 dimensions, 64-bit keys
    cases.append(dict(r=1, n=1024, d=3, r_x=1, tmax=64, tmax_new=64, seed=15, warm=True,
                      xbs=[net_points(1, 1024, 3, 10, rng) << np.uint64(54)]))

    out = {}
    for c, cs in enumerate(cases):
        r, n, d, r_x = cs["r"], cs["n"], cs["d"], cs["r_x"]
        g = gens(cs["seed"], r * d, cs["warm"])
        rngs = np.array(g, dtype=object).reshape(r, d)
        roots = np.array([rf.NUSNode_dnb2() for _ in range(r * d)]).reshape(r, d)
        out["case%d_args" % c] = np.array([r, n, d, r_x, cs["tmax"], cs["tmax_new"], len(cs["xbs"])], np.uint64)
        out["case%d_state0" % c] = np.stack([sfc64_state_words(x) for x in g])
        for k, xb in enumerate(cs["xbs"]):
            xrb = np.zeros((r, n, d), dtype=np.uint64)
            rf.dnb2_nested_uniform_scramble(np.uint64(r), np.uint64(n), np.uint64(d), np.uint64(r_x),
                                            np.uint64(cs["tmax"]), np.uint64(cs["tmax_new"]), rngs, roots, xb, xrb)
            out["case%d_xb%d" % (c, k)] = xb
            out["case%d_xrb%d" % (c, k)] = xrb
            out["case%d_state%d" % (c, k + 1)] = np.stack([sfc64_state_words(x) for x in g])
        if c == 0:
            doc = documented_xrb(a.ref)
            assert np.array_equal(out["case0_xrb0"].reshape(-1), doc), "reference differs from its documentation"
    np.savez_compressed(os.path.join(HERE, "nus.npz"), **out)
    print("wrote %d cases" % len(cases))


if __name__ == "__main__":
    main()
