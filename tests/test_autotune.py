"""Autotuner search logic (CPU) — candidate sets, budget, cache, signatures."""

import json

from zeno_gb300 import autotune as at
from zeno_gb300 import backend as zb
from zeno_gb300 import circuit as C


def test_candidates_by_precision_and_tensor_flag():
    c64 = at.candidates(20, 64, zb.FLAG_FAST)
    assert {k for k, _ in c64} == {1, 2, 3}
    c32 = at.candidates(20, 32, zb.FLAG_FAST | zb.FLAG_TENSOR)
    assert {5, 6, 7} <= {k for k, _ in c32}
    assert {h for _, h in c64} == {0, 4, 5, 6, 7}
    assert {h for _, h in at.candidates(10, 64, zb.FLAG_FAST)} == {0}


def test_search_picks_fastest_and_respects_budget():
    times = {(1, 0): 3.0, (2, 0): 1.0, (3, 0): 2.0}
    win, table = at.search(list(times), lambda k, h: times[(k, h)])
    assert win == (2, 0) and len(table) == 3
    seen = []
    win, table = at.search(list(times), lambda k, h: seen.append(k) or times[(k, h)], budget_s=-1.0)
    assert len(table) == 1 and win == (1, 0)


def test_signature_stable_and_sensitive():
    a = C.matching_circuit(10, 3, 7).to_program()
    b = C.matching_circuit(10, 3, 7).to_program()
    c = C.matching_circuit(10, 3, 8).to_program()
    assert at.signature(a) == at.signature(b) != at.signature(c)


def test_cache_file_round_trip(tmp_path, monkeypatch):
    p = C.matching_circuit(8, 2, 1).to_program()
    k = at.key(8, 64, zb.FLAG_FAST, at.signature(p))
    path = tmp_path / "tune.json"
    path.write_text(json.dumps({k: {"fusion": 2, "max_high": 5, "table": []}}))
    monkeypatch.setattr(at, "_cache", {})
    assert at.tune(p, 64, zb.FLAG_FAST, cache_path=str(path))["fusion"] == 2  # no GPU touched
