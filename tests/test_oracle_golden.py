"""The oracle (our C restatement) against the golden fixtures recorded from
the reference C backend: bit for bit for the integer, lattice and float
conversion functions, to 1e-12 for the transforms."""
import pytest

import oracle
from tests import _golden

cases, _ = _golden.load()


@pytest.mark.parametrize("cid", _golden.case_ids(), ids=lambda c: "%s-%d" % (cases[c]["name"], c))
def test_oracle_matches_reference(cid):
    case = cases[cid]
    args = _golden.build_args(case)
    oracle.call(case["name"], *args)
    assert _golden.check_outputs(case, args) == []


def test_every_function_has_cases():
    from qmctoolscl_gb300._signatures import NAMES
    names = {c["name"] for c in cases}
    assert set(NAMES) <= names
    doc = {c["name"] for c in cases if c["source"] == "doc"}
    assert len(doc) >= 20
