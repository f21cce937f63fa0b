"""Autotuner cache file (host logic, no GPU)."""
import json

from nd_gb300.tuning import AutotuneCache, cache_path, workload_key


def test_cache_round_trip_and_atomic_replace(tmp_path):
    c = AutotuneCache(tmp_path / "sub" / "autotune.json")
    k1 = workload_key("NVIDIA GB300", 5, 3, 3, 1, 4096, 10_400_000, 30_600_000, 1e-6, 1e-6, 0.5)
    k2 = workload_key("NVIDIA GB300", 5, 3, 3, 0, 4096, 10_400_000, 30_600_000, 1e-6, 1e-6, 0.5)
    assert k1 != k2
    assert c.get(k1) is None
    c.put(k1, 256)
    c.put(k2, 128)
    assert AutotuneCache(c.path).get(k1) == 256 and AutotuneCache(c.path).get(k2) == 128
    assert json.loads(c.path.read_text())[k1] == {"threads": 256}
    assert [p.name for p in c.path.parent.iterdir()] == ["autotune.json"]  # no temporary file left


def test_unreadable_or_foreign_file_is_an_empty_cache(tmp_path):
    path = tmp_path / "autotune.json"
    path.write_text("{not json")
    c = AutotuneCache(path)
    assert c.get("k") is None
    c.put("k", 64)
    assert c.get("k") == 64
    path.write_text(json.dumps({"k": {"threads": "many"}, "j": [1]}))
    assert c.get("k") is None and c.get("j") is None


def test_cache_location_follows_the_environment(monkeypatch, tmp_path):
    monkeypatch.setenv("ND_GB300_CACHE_DIR", str(tmp_path))
    assert cache_path() == tmp_path / "autotune.json"
    monkeypatch.delenv("ND_GB300_CACHE_DIR")
    monkeypatch.setenv("XDG_CACHE_HOME", str(tmp_path / "xdg"))
    assert cache_path() == tmp_path / "xdg" / "nd_gb300" / "autotune.json"
