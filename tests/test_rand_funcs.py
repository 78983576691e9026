"""The package's random-input helpers return the arrays the reference's
helpers return for the same Generator state (fixtures recorded from
qmctoolscl/rand_funcs.py by tests/golden/make_golden.py)."""
import json
import os

import numpy as np

import qmctoolscl_gb300 as q

HERE = os.path.dirname(os.path.abspath(__file__))


def test_rand_funcs_match_reference_streams():
    with open(os.path.join(HERE, "golden", "rand_funcs.json")) as f:
        meta = json.load(f)
    want = np.load(os.path.join(HERE, "golden", "rand_funcs.npz"))
    rng = np.random.Generator(np.random.SFC64(11))
    for idx, call in enumerate(meta["calls"]):
        args = [np.array(a, dtype=np.uint64) if i in call["array_args"] else a for i, a in enumerate(call["args"])]
        if call["name"] == "dnb2_get_linear_scramble_matrix":
            args[-1] = bool(args[-1])
        fn = getattr(q, call["name"])
        got = fn(*args) if call["name"] == "gdn_get_halton_generating_matrix" else fn(rng, *args)
        exp = want["%02d" % idx]
        assert np.asarray(got).dtype == exp.dtype, call["name"]
        assert np.array_equal(np.asarray(got), exp), call["name"]


def test_print_mats_format(capsys):
    rng = np.random.Generator(np.random.SFC64(7))
    S = q.dnb2_get_linear_scramble_matrix(rng, 1, 1, 4, 4, True)
    out = capsys.readouterr().out.splitlines()
    assert out[0] == "S with shape (r=1, d=1, tmax_new=4)"
    assert out[1] == "l = 0" and out[2] == "    j = 0"
    rows = [ln.strip() for ln in out[3:]]
    assert rows[0] == "1000" and all(len(r_) == 4 for r_ in rows)
    assert [int(r_, 2) for r_ in rows] == [int(v) for v in S[0, 0]]
