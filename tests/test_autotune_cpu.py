"""Host logic of the launch-shape autotuner: the per-process choice table and its JSON cache."""
import json

from discoeb_gb300 import _native, autotune


def _dims(exec_mode=0):
    return _native.DebDims(12, 12, 17, 17, 15, 1, 0, 0, exec_mode)


def test_choice_round_trips_through_the_cache_file(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setenv("DISCOEB_GB300_TUNE_CACHE", str(path))
    monkeypatch.setattr(autotune, "_key", lambda d: f"GB300|{d.lmaxg}|{d.nqmax}")
    monkeypatch.setattr(autotune, "_chosen", {})
    monkeypatch.setattr(autotune, "_loaded", False)
    assert autotune.chosen(_dims()) is None
    autotune.remember(_dims(), ("global", 6))
    assert json.loads(path.read_text()) == {"GB300|12|15": ["global", 6]}
    # a fresh process reads it back
    monkeypatch.setattr(autotune, "_chosen", {})
    monkeypatch.setattr(autotune, "_loaded", False)
    assert autotune.chosen(_dims()) == ("global", 6)
    # the lane-per-mode kernel has no launch shape to tune
    assert autotune.chosen(_dims(exec_mode=_native.EXEC_MODES["lane"])) is None


def test_unreadable_cache_is_ignored(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    path.write_text("{not json")
    monkeypatch.setenv("DISCOEB_GB300_TUNE_CACHE", str(path))
    monkeypatch.setattr(autotune, "_key", lambda d: "k")
    monkeypatch.setattr(autotune, "_chosen", {})
    monkeypatch.setattr(autotune, "_loaded", False)
    assert autotune.chosen(_dims()) is None


def test_candidates_cover_both_stage_vector_placements():
    assert {c[0] for c in autotune.CANDIDATES} == {"shared", "global", "all_global"}
    assert all(c[1] >= 0 for c in autotune.CANDIDATES)
