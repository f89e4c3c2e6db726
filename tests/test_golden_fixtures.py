"""The committed fixtures are what tests/golden/make_golden.py derives from
the reference's example programs (checked where ZENO_REFERENCE names a
reference checkout; the fixtures themselves travel with the tests)."""
import json
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden  # noqa: E402


REF = os.environ.get("ZENO_REFERENCE", "")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "examples")), reason="ZENO_REFERENCE not set")
def test_fixtures_match_the_reference_examples():
    with open(os.path.join(HERE, "golden", "examples.json")) as f:
        committed = json.load(f)
    fresh = json.loads(json.dumps(make_golden.build(REF), sort_keys=True))
    assert fresh == committed
