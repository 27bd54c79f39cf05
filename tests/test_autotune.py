"""Host logic of the launch-shape autotuner (dsplat/autotune.py), on the CPU."""

from __future__ import annotations

import json


def test_shape_keys_bucket_to_powers_of_two():
    from dsplat.autotune import _bucket, shape_key

    assert [_bucket(n) for n in (0, 1, 2, 3, 1000, 1024, 1025, 16384)] == [0, 1, 2, 4, 1024, 1024, 2048, 16384]
    assert shape_key("splat", 16000, 2000, 128, 2) == shape_key("splat", 16384, 1500, 128, 2)
    assert shape_key("splat", 16384, 2000, 128, 2) != shape_key("splat", 16385, 2000, 128, 2)
    assert shape_key("orient", 384, 0, 128, 2).startswith("orient|A512|S0|K128|P2|R0|")


def test_choose_takes_the_fastest_and_breaks_ties_by_the_smaller_value():
    from dsplat.autotune import choose

    times = {2: 3.0, 4: 1.5, 6: 1.5, 8: 2.0}
    best, timings = choose(times, lambda value: times[value])
    assert best == 4 and timings == times


def test_cache_round_trip(tmp_path, monkeypatch):
    from dsplat import autotune

    path = tmp_path / "tuning.json"
    monkeypatch.setenv("DSPLAT_TUNING_CACHE", str(path))
    autotune.reset(memory_only=True)
    key = autotune.shape_key("project", 0, 2000, 128, 2, 60)
    assert autotune.lookup(key) is None
    assert autotune.gram_splits(7, key) == 7
    autotune.record(key, 3, {2: 1.25, 3: 1.0, 4: 1.1})
    stored = json.loads(path.read_text())
    assert stored[key]["value"] == 3 and stored[key]["ms"]["3"] == 1.0
    autotune.reset(memory_only=True)  # a new process reads the file again
    assert autotune.lookup(key) == 3
    assert autotune.gram_splits(7, key) == 3
    autotune.reset()
    assert not path.exists() and autotune.lookup(key) is None
