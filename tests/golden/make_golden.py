"""Generate the golden fixtures from the QMCToolsCL reference itself.

Run in a checkout that has the reference sources (--ref, or $QMCTOOLSCL_REF):

    python tests/golden/make_golden.py [--ref /path/to/QMCToolsCL]

It does three things:

1. compiles the reference C backend from its own sources
   (``make -C oracle ref`` -> oracle/_ref/c_lib.so);
2. replays the reference's own doctest suite (docs/index.md, C-backend
   variant, extracted the way prep_docs_doctests.py:4-14 does) against a
   recording shim that routes every hot-path call into that compiled reference
   and records its inputs and outputs.  The replay must pass with zero
   doctest failures, so every recorded output equals the value the reference
   documentation prints;
3. records seeded random cases for all 23 functions (edge cases included)
   from the same compiled reference, with inputs drawn by the reference's own
   rand_funcs.py generators.

Output: tests/golden/golden.npz (arrays) and tests/golden/golden.json
(the case list: function, scalars, array names, where it came from).
The fixtures are what the tests compare the oracle and the GPU kernels with;
the reference checkout is not needed to run the tests.
"""
import argparse
import doctest
import importlib.util
import json
import os
import re
import sys
import types

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, REPO)

import oracle  # noqa: E402
from qmctoolscl_gb300._signatures import SIGNATURES  # noqa: E402

OUT_NPZ = os.path.join(REPO, "tests", "golden", "golden.npz")
OUT_JSON = os.path.join(REPO, "tests", "golden", "golden.json")
TWIDDLES = ("twiddler", "twiddlei")
IN_PLACE = ("xr", "xi", "x")  # transformed in place by the fft/ifft/fwht (the only in/out arrays)
IN_PLACE_FUNCS = ("fft_bro_1d_radix2", "ifft_bro_1d_radix2", "fwht_1d_radix2")


class Recorder:
    def __init__(self):
        self.cases = []
        self.arrays = {}
        self.source = "doc"

    def call(self, name, args):
        spec, outs = SIGNATURES[name]
        assert len(args) == len(spec), (name, len(args))
        cid = len(self.cases)
        scalars, arrays, shapes = {}, [], {}
        for (an, kind), a in zip(spec, args):
            if kind == "u64":
                scalars[an] = int(a)
            else:
                shapes[an] = list(np.shape(a))
                arrays.append(an)
                # output-only buffers (np.empty in the callers, twiddle tables)
                # are never read, so their initial content is not stored
                if an not in outs or (name in IN_PLACE_FUNCS and an in IN_PLACE):
                    self.arrays["%04d/%s" % (cid, an)] = np.array(a, copy=True)
        oracle.call_ref(name, *args)
        names = [s[0] for s in spec]
        for an in outs:
            out = np.array(args[names.index(an)], copy=True)
            if an in TWIDDLES:  # only the first n = 2*n_half entries are written
                out = out.reshape(-1)[:2 * scalars["n_half"]]
            self.arrays["%04d/%s@out" % (cid, an)] = out
        self.cases.append({"id": cid, "name": name, "scalars": scalars, "arrays": arrays,
                           "shapes": shapes, "outputs": list(outs), "source": self.source})


def load_ref_rand_funcs(ref):
    spec = importlib.util.spec_from_file_location("ref_rand_funcs",
                                                  os.path.join(ref, "qmctoolscl", "rand_funcs.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def ref_docstrings(ref):
    """Docstrings the reference's generator builds from the .cl comments
    (pdm_build.py:51-82), so the doctests that print them pass."""
    docs = {}
    kdir = os.path.join(ref, "qmctoolscl", "cl_kernels")
    for fn in sorted(os.listdir(kdir)):
        with open(os.path.join(kdir, fn)) as f:
            code = f.read()
        for block in re.findall(r'(?<=void\s).*?(?=\s?\))', code, re.DOTALL):
            lines = block.replace("(", "").splitlines()
            name, desc, si = lines[0], [], 1
            while lines[si].strip()[:2] == "//":
                desc.append(lines[si].split("// ")[1].strip())
                si += 1
            doc_args = []
            for ln in lines[si:]:
                var_input, var_desc = ln.split(" // ")
                vtype, var = var_input.replace(",", "").split(" ")[-2:]
                ctype = {"ulong": "uint64", "double": "double", "char": "uint8"}[vtype]
                if var[0] != "*":
                    doc_args.append("%s (np.%s): %s" % (var, ctype, var_desc))
                else:
                    doc_args.append("%s (np.ndarray of np.%s): %s" % (var[1:], ctype, var_desc))
            doc_args = doc_args[:3] + doc_args[6:]
            docs[name] = '%s\n\nArgs:\n    %s' % ("\n".join(desc).strip(), "\n    ".join(doc_args))
    return docs


def make_shim(rec, rand_mod, docs):
    shim = types.ModuleType("qmctoolscl")
    for k in dir(rand_mod):
        if not k.startswith("__"):
            setattr(shim, k, getattr(rand_mod, k))
    for name in SIGNATURES:
        def f(*args, _name=name, **kwargs):
            rec.call(_name, list(args))
            return 0.0, 0.0
        f.__name__ = name
        f.__doc__ = docs[name]
        setattr(shim, name, f)
    return shim


def replay_doctests(ref, shim):
    with open(os.path.join(ref, "docs", "index.md")) as f:
        contents = f.read()
    blocks = re.findall(r'(?<=```python).*?(?=\s?```)', contents, re.DOTALL)
    blocks = [b.replace("\n\n\n", "\n<BLANKLINE>\n<BLANKLINE>\n").replace("\n\n", "\n<BLANKLINE>\n")
              for b in blocks]
    text = "\n".join(blocks[:3] + blocks[4:])  # the C-backend variant
    sys.modules["qmctoolscl"] = shim
    # a few transform examples draw from numpy's global generator (unseeded in
    # the docs); seed it so the recorded fixtures are reproducible
    np.random.seed(7)
    parser = doctest.DocTestParser()
    test = parser.get_doctest(text, {}, "qmctoolscl_docs", "index.md", 0)
    runner = doctest.DocTestRunner(optionflags=doctest.ELLIPSIS)
    runner.run(test)
    res = runner.summarize(verbose=False)
    print("reference doctest replay: attempted=%d failed=%d" % (res.attempted, res.failed))
    if res.failed:
        raise SystemExit("doctest replay failed: fixtures would not match the documented values")


def random_cases(rec, rf):
    rec.source = "random"
    rng = np.random.Generator(np.random.SFC64(20240601))
    U = np.uint64

    def odd(shape, bits):
        return (rng.integers(0, 1 << (bits - 1), shape) * 2 + 1).astype(U)

    # lattices
    for (r, n, d, bits) in [(1, 1, 1, 20), (2, 8, 5, 20), (3, 13, 7, 20), (2, 1000, 3, 24),
                            (2, 64, 4, 52), (1, 33, 3, 62)]:
        g = odd((r, d), bits)
        rec.call("lat_gen_linear", [U(r), U(n), U(d), g, np.empty((r, n, d))])
    for (r, n, d, ns, bits) in [(1, 1, 1, 0, 20), (2, 16, 5, 0, 20), (3, 1, 3, 1, 20),
                                (2, 6, 7, 2, 20), (1, 12, 3, 4, 20), (2, 8, 2, 8, 20),
                                (1, 1024, 3, 0, 30), (2, 32, 3, 32, 45), (1, 0, 3, 0, 20)]:
        g = odd((r, d), bits)
        rec.call("lat_gen_natural", [U(r), U(n), U(d), U(ns), g, np.empty((r, n, d))])
    for (r, n, d, ns, bits) in [(1, 1, 1, 0, 20), (2, 16, 5, 0, 20), (3, 17, 3, 3, 20),
                                (2, 37, 7, 100, 20), (1, 9, 2, (1 << 20) - 5, 20),
                                (2, 1000, 3, 0, 33), (1, 64, 3, 5, 50), (1, 0, 2, 0, 20)]:
        g = odd((r, d), bits)
        rec.call("lat_gen_gray", [U(r), U(n), U(d), U(ns), g, np.empty((r, n, d))])
    for (r, r_x, n, d) in [(1, 1, 5, 3), (4, 2, 9, 5), (3, 1, 16, 4), (2, 2, 33, 7)]:
        x = rng.random((r_x, n, d))
        sh = rf.lat_get_shifts(rng, r, d)
        rec.call("lat_shift_mod_1", [U(r), U(n), U(d), U(r_x), x, sh, np.empty((r, n, d))])
    # lattice points on the 2^-k grid, shift sums that hit 1 exactly, and
    # values outside [0,1) (negative and >= 1) that exercise fmod's sign rules
    x = np.array([[[0.75, 0.5, -0.3, -1.0, 1.5, 0.0, 2.0 ** -60, 0.999999999999]]])
    sh = np.array([[0.25, 0.5, 0.1, 0.0, 0.25, 0.0, 1 - 2.0 ** -53, 0.5]])
    rec.call("lat_shift_mod_1", [U(1), U(1), U(8), U(1), x, sh, np.empty((1, 1, 8))])

    # base-2 nets
    def gmats(r, d, mmax, tmax):
        return rng.integers(0, 1 << tmax, (r, d, mmax), dtype=U) if tmax < 64 else \
            rf.random_tbit_uint64s(rng, 64, (r, d, mmax))
    for (r, n, d, ns, mmax) in [(1, 1, 1, 0, 1), (2, 16, 3, 0, 4), (1, 14, 2, 2, 4),
                                (3, 12, 5, 4, 5), (2, 8, 4, 8, 5), (1, 1024, 3, 0, 10),
                                (2, 96, 3, 32, 7), (1, 0, 2, 0, 3)]:
        C = gmats(r, d, mmax, 63)
        rec.call("dnb2_gen_natural", [U(r), U(n), U(d), U(ns), U(mmax), C, np.empty((r, n, d), U)])
    for (r, n, d, ns, mmax) in [(1, 1, 1, 0, 1), (2, 16, 3, 0, 4), (1, 14, 2, 2, 4),
                                (3, 37, 5, 5, 6), (2, 100, 4, 27, 8), (1, 1024, 3, 0, 10),
                                (1, 0, 2, 0, 3)]:
        C = gmats(r, d, mmax, 64)
        rec.call("dnb2_gen_gray", [U(r), U(n), U(d), U(ns), U(mmax), C, np.empty((r, n, d), U)])
    for (r, r_x, n, d) in [(1, 1, 5, 3), (4, 2, 9, 5), (3, 1, 16, 4)]:
        xb = rf.random_tbit_uint64s(rng, 40, (r_x, n, d))
        lsh = rng.integers(0, 24, r_x).astype(U)
        lsh[0] = 0
        sb = rf.dnb2_get_digital_shifts(rng, r, d, 64)
        rec.call("dnb2_digital_shift", [U(r), U(n), U(d), U(r_x), lsh, xb, sb, np.empty((r, n, d), U)])
    xb = rf.random_tbit_uint64s(rng, 64, (1, 4, 3))
    rec.call("dnb2_digital_shift", [U(1), U(4), U(3), U(1), np.array([63], U), xb,
                                    rf.dnb2_get_digital_shifts(rng, 1, 3, 64), np.empty((1, 4, 3), U)])
    for (r, n, d, tm) in [(1, 5, 3, [64]), (3, 7, 2, [63, 32, 70]), (2, 4, 4, [1, 53])]:
        xb = rf.random_tbit_uint64s(rng, 64, (r, n, d))
        xb.flat[0] = 0
        xb.flat[1] = np.uint64((1 << 64) - 1)
        xb.flat[2] = np.uint64((1 << 53) + 1)  # a tie that rounds to even
        xb.flat[3] = np.uint64((1 << 54) + 6)  # a tie that rounds up
        rec.call("dnb2_integer_to_float", [U(r), U(n), U(d), np.array(tm, U), xb, np.empty((r, n, d))])
    for (r, r_C, d, mmax, tmax, tnew) in [(2, 1, 4, 4, 4, 6), (3, 3, 5, 8, 20, 32),
                                          (4, 2, 3, 10, 64, 64), (1, 1, 2, 3, 10, 10)]:
        C = gmats(r_C, d, mmax, tmax)
        S = rf.dnb2_get_linear_scramble_matrix(rng, r, d, tmax, tnew, False)
        rec.call("dnb2_linear_matrix_scramble", [U(r), U(d), U(mmax), U(r_C), U(tnew), S, C,
                                                 np.empty((r, d, mmax), U)])
    for (r, d, mmax, tmax, alpha) in [(2, 4, 4, 6, 2), (1, 6, 5, 10, 3), (3, 8, 3, 32, 2),
                                      (1, 4, 2, 40, 2)]:
        da = d // alpha
        ta = min(alpha * tmax, 64)
        C = gmats(r, d, mmax, tmax)
        Ca = np.empty((r, da, mmax), U)
        rec.call("dnb2_interlace", [U(r), U(da), U(mmax), U(d), U(tmax), U(ta), U(alpha), C, Ca])
        rec.call("dnb2_undo_interlace", [U(r), U(d), U(mmax), U(da), U(tmax), U(ta), U(alpha),
                                         Ca.copy(), np.empty((r, d, mmax), U)])
    for (r, d, mmax, tm) in [(1, 4, 4, [4]), (2, 3, 5, [10, 20]), (3, 2, 6, [64, 63, 40])]:
        C = np.stack([rng.integers(0, 1 << int(min(t, 63)), (d, mmax), dtype=U) for t in tm])
        rec.call("dnb2_gmat_lsb_to_msb", [U(r), U(d), U(mmax), np.array(tm, U), C,
                                          np.empty((r, d, mmax), U)])

    # generalized nets
    for (r, r_b, n, d, ns, bases_row, mmax, tmax) in [
            (1, 1, 9, 3, 0, [2, 3, 5], 4, 4), (2, 2, 12, 2, 5, None, 5, 6),
            (2, 1, 30, 4, 17, [7, 11, 13, 541], 3, 5), (1, 1, 200, 5, 0, [2, 3, 5, 7, 11], 8, 12),
            (1, 1, 0, 2, 0, [2, 3], 2, 2)]:
        if bases_row is None:
            bases = np.array([[2, 3], [5, 7]], U)
        else:
            bases = np.array([bases_row], U)
        C = np.empty((r, d, mmax, tmax), U)
        for l in range(r):
            for j in range(d):
                C[l, j] = rng.integers(0, bases[l % r_b, j], (mmax, tmax), dtype=U)
        rec.call("gdn_gen_natural", [U(r), U(n), U(d), U(r_b), U(mmax), U(tmax), U(ns), bases, C,
                                     np.empty((r, n, d, tmax), U)])
    for (r, n, d, ns, b, mmax, tmax) in [(1, 9, 2, 0, 3, 2, 4), (2, 30, 3, 4, 5, 3, 6),
                                         (1, 50, 2, 11, 7, 3, 3)]:
        C = rng.integers(0, b, (r, d, mmax, tmax), dtype=U)
        rec.call("gdn_gen_natural_same_base", [U(r), U(n), U(d), U(mmax), U(tmax), U(ns), U(b), C,
                                               np.empty((r, n, d, tmax), U)])
    for (r, r_C, r_b, d, mmax, tmax, tnew, brow) in [
            (4, 2, 2, 2, 5, 5, 10, None), (2, 1, 1, 3, 4, 6, 6, [3, 5, 541]),
            (3, 3, 1, 2, 3, 4, 8, [2, 7])]:
        bases = np.array([[2, 3], [5, 7]], U) if brow is None else np.array([brow], U)
        C = np.empty((r_C, d, mmax, tmax), U)
        for l in range(r_C):
            for j in range(d):
                C[l, j] = rng.integers(0, bases[l % r_b, j], (mmax, tmax), dtype=U)
        S = rf.gdn_get_linear_scramble_matrix(rng, r, d, tmax, tnew, r_b, bases)
        rec.call("gdn_linear_matrix_scramble", [U(r), U(d), U(mmax), U(r_C), U(r_b), U(tmax),
                                                U(tnew), bases, S, C, np.empty((r, d, mmax, tnew), U)])
    for (r, r_x, r_b, n, d, tmax, tnew, brow) in [
            (4, 4, 2, 6, 2, 10, 12, None), (2, 1, 1, 7, 3, 4, 4, [3, 5, 541]),
            (3, 3, 1, 5, 2, 3, 6, [2, 7])]:
        bases = np.array([[2, 3], [5, 7]], U) if brow is None else np.array([brow], U)
        xdig = np.empty((r_x, n, d, tmax), U)
        for l in range(r_x):
            for j in range(d):
                xdig[l, :, j] = rng.integers(0, bases[l % r_b, j], (n, tmax), dtype=U)
        sh = rf.gdn_get_digital_shifts(rng, r, d, tnew, r_b, bases)
        rec.call("gdn_digital_shift", [U(r), U(n), U(d), U(r_x), U(r_b), U(tmax), U(tnew), bases, sh,
                                       xdig, np.empty((r, n, d, tnew), U)])
        perms = rf.gdn_get_digital_permutations(rng, r, d, tnew, r_b, bases)
        bmax = U(bases.max())
        rec.call("gdn_digital_permutation", [U(r), U(n), U(d), U(r_x), U(r_b), U(tmax), U(tnew), bmax,
                                             perms, xdig, np.empty((r, n, d, tnew), U)])
    for (r, r_b, n, d, tmax, brow, big) in [(2, 2, 6, 2, 12, None, False),
                                            (1, 1, 9, 4, 64, [2, 3, 5, 541], False),
                                            (2, 1, 4, 3, 8, [3, 10, 541], True)]:
        bases = np.array([[2, 3], [5, 7]], U) if brow is None else np.array([brow], U)
        xdig = np.empty((r, n, d, tmax), U)
        for l in range(r):
            for j in range(d):
                hi = bases[l % r_b, j] if not big else 1 << 40
                xdig[l, :, j] = rng.integers(0, hi, (n, tmax), dtype=U)
        rec.call("gdn_integer_to_float", [U(r), U(n), U(d), U(r_b), U(tmax), bases, xdig,
                                          np.empty((r, n, d))])
    for (r, d, mmax, tmax, alpha) in [(2, 6, 3, 4, 3), (1, 4, 2, 5, 2), (2, 6, 4, 3, 2)]:
        da = d // alpha
        ta = alpha * tmax
        C = rng.integers(0, 5, (r, d, mmax, tmax), dtype=U)
        Ca = np.empty((r, da, mmax, ta), U)
        rec.call("gdn_interlace", [U(r), U(da), U(mmax), U(d), U(tmax), U(ta), U(alpha), C, Ca])
        rec.call("gdn_undo_interlace", [U(r), U(d), U(mmax), U(da), U(tmax), U(ta), U(alpha),
                                        Ca.copy(), np.empty((r, d, mmax, tmax), U)])

    # transforms
    for (d1, d2, nh) in [(1, 1, 1), (1, 1, 4), (2, 3, 8), (1, 2, 64), (3, 1, 512)]:
        n = 2 * nh
        for name in ("fft_bro_1d_radix2", "ifft_bro_1d_radix2"):
            xr = rng.standard_normal((d1, d2, n))
            xi = rng.standard_normal((d1, d2, n))
            rec.call(name, [U(d1), U(d2), U(nh), np.empty(n), np.empty(n), xr, xi])
        rec.call("fwht_1d_radix2", [U(d1), U(d2), U(nh), rng.standard_normal((d1, d2, n))])


def rand_cases(rf):
    """Outputs of the reference's random-input helpers for a fixed sequence
    of calls on one Generator (the helpers' results are defined by numpy's
    streams; the package restates them and must match these)."""
    rng = np.random.Generator(np.random.SFC64(11))
    U = np.uint64
    b2 = np.array([[2, 3], [5, 7]], U)
    b1 = np.array([3, 5, 541], U)
    calls = [
        ("random_tbit_uint64s", (5, (3, 4))), ("random_tbit_uint64s", (64, (2, 5))),
        ("random_tbit_uint64s", (0, (2,))), ("random_uint64_permutations", (3, 7)),
        ("lat_get_shifts", (3, 5)), ("dnb2_get_digital_shifts", (2, 3, 64)),
        ("dnb2_get_digital_shifts", (2, 3, 20)),
        ("dnb2_get_linear_scramble_matrix", (2, 3, 4, 6, False)),
        ("dnb2_get_linear_scramble_matrix", (2, 2, 64, 64, False)),
        ("gdn_get_linear_scramble_matrix", (4, 2, 5, 10, 2, b2)),
        ("gdn_get_linear_scramble_matrix", (2, 3, 4, 4, 1, b1)),
        ("gdn_get_halton_generating_matrix", (2, 3, 4)),
        ("gdn_get_digital_shifts", (4, 2, 12, 2, b2)), ("gdn_get_digital_shifts", (2, 3, 6, 1, b1)),
        ("gdn_get_digital_permutations", (4, 2, 3, 2, b2)), ("gdn_get_digital_permutations", (1, 3, 2, 1, b1)),
    ]
    out = {}
    meta = []
    for idx, (fname, fargs) in enumerate(calls):
        fn = getattr(rf, fname)
        res = fn(*fargs) if fname == "gdn_get_halton_generating_matrix" else fn(rng, *fargs)
        out["%02d" % idx] = np.asarray(res)
        meta.append({"name": fname, "args": [a.tolist() if isinstance(a, np.ndarray) else a for a in fargs],
                     "array_args": [i for i, a in enumerate(fargs) if isinstance(a, np.ndarray)]})
    return out, meta


def main():
    ap = argparse.ArgumentParser()
    env_ref = os.environ.get("QMCTOOLSCL_REF")
    ap.add_argument("--ref", default=env_ref, required=env_ref is None,
                    help="QMCToolsCL checkout (default: $QMCTOOLSCL_REF)")
    a = ap.parse_args()
    oracle.build(ref=True, ref_dir=a.ref)
    rf = load_ref_rand_funcs(a.ref)
    rec = Recorder()
    replay_doctests(a.ref, make_shim(rec, rf, ref_docstrings(a.ref)))
    n_doc = len(rec.cases)
    random_cases(rec, rf)
    rand_out, rand_meta = rand_cases(rf)
    np.savez_compressed(os.path.join(REPO, "tests", "golden", "rand_funcs.npz"), **rand_out)
    with open(os.path.join(REPO, "tests", "golden", "rand_funcs.json"), "w") as f:
        json.dump({"seed": "np.random.Generator(np.random.SFC64(11))", "calls": rand_meta}, f, indent=1)
    np.savez_compressed(OUT_NPZ, **rec.arrays)
    with open(OUT_JSON, "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py",
                   "reference": "QMCToolsCL 1.2.1 C backend, compiled by oracle/Makefile (ref)",
                   "cases": rec.cases}, f, indent=1)
    print("recorded %d doc cases and %d random cases -> %s (%.1f KB)" % (
        n_doc, len(rec.cases) - n_doc, OUT_NPZ, os.path.getsize(OUT_NPZ) / 1024))


if __name__ == "__main__":
    main()
