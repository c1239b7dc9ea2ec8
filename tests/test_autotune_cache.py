"""The autotuner's on-disk cache (DGB_TUNE_CACHE) on CPU: picks stored by one
process are read back by the next, and an unreadable file is ignored."""

from dendra_gb300 import autotune


def test_picks_persist_across_processes(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setenv("DGB_TUNE_CACHE", str(path))
    monkeypatch.setattr(autotune, "_cache", None)
    autotune._store("cable_run_split|GPU|f32|(-1, 0, 0)", [-1, 0, 0])
    autotune._store("tridiag_lanes|GPU|401", 16)
    assert path.exists()
    monkeypatch.setattr(autotune, "_cache", None)  # a new process
    cache = autotune._load_cache()
    assert cache["cable_run_split|GPU|f32|(-1, 0, 0)"] == [-1, 0, 0]
    assert cache["tridiag_lanes|GPU|401"] == 16


def test_unreadable_cache_file_is_ignored(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    path.write_text("{not json")
    monkeypatch.setenv("DGB_TUNE_CACHE", str(path))
    monkeypatch.setattr(autotune, "_cache", None)
    assert autotune._load_cache() == {}
