"""Access to the golden fixtures recorded from the reference C backend
(tests/golden/make_golden.py)."""
import json
import os

import numpy as np

from qmctoolscl_gb300._signatures import SIGNATURES

HERE = os.path.dirname(os.path.abspath(__file__))
_cache = {}

# transforms are compared with a tolerance; everything else bit for bit
TRANSFORMS = ("fft_bro_1d_radix2", "ifft_bro_1d_radix2", "fwht_1d_radix2")
TWIDDLES = ("twiddler", "twiddlei")


def load():
    if not _cache:
        with open(os.path.join(HERE, "golden", "golden.json")) as f:
            _cache["meta"] = json.load(f)
        _cache["npz"] = np.load(os.path.join(HERE, "golden", "golden.npz"))
    return _cache["meta"]["cases"], _cache["npz"]


def case_ids(name=None):
    cases, _ = load()
    return [c["id"] for c in cases if name is None or c["name"] == name]


def build_args(case):
    """Fresh numpy arguments for one recorded call (outputs poisoned)."""
    _, z = load()
    spec, outs = SIGNATURES[case["name"]]
    args = []
    for an, kind in spec:
        if kind == "u64":
            args.append(np.uint64(case["scalars"][an]))
            continue
        shape = tuple(case["shapes"][an])
        dt = np.uint64 if kind == "u64*" else np.float64
        key = "%04d/%s" % (case["id"], an)
        if key in z.files:
            args.append(np.ascontiguousarray(z[key]).reshape(shape).astype(dt, copy=True))
        else:  # write-only buffer: poison it so unwritten entries show
            a = np.empty(shape, dt)
            a.view(np.uint64)[...] = np.uint64(0xFFF8DEADBEEF0001)
            args.append(a)
    return args


def expected(case):
    _, z = load()
    return {an: z["%04d/%s@out" % (case["id"], an)] for an in case["outputs"]}


def check_outputs(case, args, exact=None):
    """Compare outputs with the recorded reference outputs; returns a list of
    mismatch descriptions (empty when everything agrees)."""
    spec, _ = SIGNATURES[case["name"]]
    names = [a for a, _k in spec]
    if exact is None:
        exact = case["name"] not in TRANSFORMS
    bad = []
    for an, want in expected(case).items():
        got = np.asarray(args[names.index(an)])
        if an in TWIDDLES:
            got = got.reshape(-1)[:want.size]
        got = got.reshape(want.shape)
        if exact:
            if got.dtype == np.float64:
                ok = np.array_equal(got.view(np.uint64), want.view(np.uint64))
            else:
                ok = np.array_equal(got, want)
        else:
            ok = np.allclose(got, want, rtol=1e-12, atol=1e-12)
        if not ok:
            bad.append("%s[%d] %s mismatch" % (case["name"], case["id"], an))
    return bad
