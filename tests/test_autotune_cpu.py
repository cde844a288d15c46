"""Autotuner bookkeeping on the host: workload signatures and the JSON cache."""

from pytreegrav_gb300 import autotune


def test_signature_buckets_by_powers_of_two():
    a = autotune.signature(1_000_000, 1, 2, True, 0.7)
    assert a == autotune.signature(1_100_000, 1, 2, True, 0.7)
    assert a != autotune.signature(4_000_000, 1, 2, True, 0.7)
    assert a != autotune.signature(1_000_000, 4096, 2, True, 0.7)
    assert a != autotune.signature(1_000_000, 1, 2, False, 0.7)


def test_cache_round_trip(tmp_path, monkeypatch):
    monkeypatch.setenv("TG_AUTOTUNE_CACHE", str(tmp_path / "c.json"))
    assert autotune._load_cache() == {}
    autotune._store("k", {"group_size": 16, "warps": 4, "stack": 1024, "ms": 1.0})
    autotune._store("k2", {"group_size": 32, "warps": 8, "stack": 4096, "ms": 2.0})
    c = autotune._load_cache()
    assert c["k"]["group_size"] == 16 and c["k2"]["stack"] == 4096
