"""The autotuner's shape cache on the host: a stored shape is read back, an
entry in another form reads as absent, an unwritable cache location is not
an error, and the candidate list and size-stratified sample are what the
tuner measures."""

import json
import os

import numpy as np


def test_cache_round_trip_and_bad_entries(tmp_path, monkeypatch):
    from pycwb_gb300 import _lib, autotune
    monkeypatch.setattr(autotune, "CACHE_PATH", str(tmp_path / "sub" / "tile_shapes.json"))
    key = autotune.problem_key(3, 41, 196608, [20, 300, 3000], True)
    assert autotune.cached_shape(key) is None
    shape = _lib.TileShape(256, 1, 0, 2, 3, 1)
    autotune._store(key, shape, {"256,1,0,2,3,1": 1.5})
    assert autotune.cached_shape(key).key() == shape.key()
    assert not [p for p in os.listdir(tmp_path / "sub") if p.endswith(".tmp")]
    # another tuner's entry in another form: absent, not an exception
    data = json.loads((tmp_path / "sub" / "tile_shapes.json").read_text())
    data["other"] = {"shape": ["a"]}
    data["older"] = {"timings_ms": {}}
    (tmp_path / "sub" / "tile_shapes.json").write_text(json.dumps(data))
    assert autotune.cached_shape("other") is None and autotune.cached_shape("older") is None
    assert autotune.cached_shape(key).key() == shape.key()
    # a torn or foreign file reads as an empty cache
    (tmp_path / "sub" / "tile_shapes.json").write_text("{not json")
    assert autotune.cached_shape(key) is None


def test_unwritable_cache_is_not_an_error(tmp_path, monkeypatch):
    from pycwb_gb300 import _lib, autotune
    blocker = tmp_path / "file"
    blocker.write_text("x")                     # a file where the cache directory should be
    monkeypatch.setattr(autotune, "CACHE_PATH", str(blocker / "tile_shapes.json"))
    autotune._store("k", _lib.TileShape(128, 2, 16, 3, 4, -1), {})
    assert autotune.cached_shape("k") is None


def test_candidates_and_sample():
    from pycwb_gb300 import autotune
    c3 = autotune.candidates(3, True)
    assert len(c3) == 32 and {s.min_blocks for s in c3} == {3, 4}
    assert all(s.fast_math == 1 for s in c3)
    c6 = autotune.candidates(6, False)
    assert {s.min_blocks for s in c6} == {2} and all(s.fast_math == -1 for s in c6)
    sizes = np.random.default_rng(0).integers(20, 3000, 500)
    idx = autotune.sample_indices(sizes, 48)
    assert idx.size == 48 and np.all(np.diff(idx) > 0)
    picked = np.sort(sizes[idx])
    assert picked[0] == sizes.min() and picked[-1] == sizes.max()
    assert np.array_equal(autotune.sample_indices(sizes[:10], 48), np.arange(10))
