"""Host logic of the launch-shape autotuner's cache (no GPU): keys by device,
precision, method, single/ensemble and power-of-two size bucket; atomic JSON
round trip; an unreadable cache is treated as empty."""
import json

import pytest

from anuga_cuda import autotune as AT


@pytest.fixture
def cache(tmp_path, monkeypatch):
    path = tmp_path / "sub" / "autotune.json"
    monkeypatch.setenv("ANUGA_CUDA_TUNE_CACHE", str(path))
    monkeypatch.setattr(AT, "_device_name", lambda: "GB300 test")
    return path


def test_key_buckets_and_fields(cache):
    assert AT._key("mixed", 1000) == "GB300 test|mixed|euler|single|512"
    assert AT._key("mixed", 1024).endswith("|1024")
    assert AT._key("mixed", 1025).endswith("|1024")
    assert AT._key("fp64", 0).endswith("|1")
    assert AT._key("fp64", 4_000_000, "rk2", ensemble=True) == \
        "GB300 test|fp64|rk2|ensemble|2097152"


def test_store_and_lookup_round_trip(cache):
    cfg = {"flux_block": 256, "update_block": 256, "distribute_block": 128,
           "steps_per_graph": 16, "flux_pipelined": 0, "dependent_launch": 1}
    assert AT.cached_config("mixed", 4_000_000) is None
    AT._store(AT._key("mixed", 4_000_000), cfg)
    assert cache.exists() and not (cache.parent / "autotune.json.tmp").exists()
    # the same bucket finds it; another size, precision or method does not
    assert AT.cached_config("mixed", 3_000_000) == cfg
    assert AT.cached_config("mixed", 1_000_000) is None
    assert AT.cached_config("fp64", 4_000_000) is None
    assert AT.cached_config("mixed", 4_000_000, "rk3") is None
    # a second entry keeps the first
    AT._store(AT._key("fp64", 40_000), dict(cfg, flux_block=128))
    data = json.loads(cache.read_text())
    assert len(data) == 2 and AT.cached_config("mixed", 4_000_000) == cfg


def test_unreadable_cache_is_empty(cache):
    cache.parent.mkdir(parents=True)
    cache.write_text("{not json")
    assert AT._load() == {}
    assert AT.cached_config("mixed", 100) is None
    AT._store(AT._key("mixed", 100), {"flux_block": 64})
    assert AT.cached_config("mixed", 100) == {"flux_block": 64}


def test_default_candidates_within_templated_sizes():
    assert set(AT.DEFAULT_CANDIDATES) == {"flux", "update", "distribute"}
    assert set(AT.DEFAULT_CANDIDATES["flux"]) <= {64, 128, 256}
    for k in ("update", "distribute"):
        assert set(AT.DEFAULT_CANDIDATES[k]) <= {128, 256, 512}
