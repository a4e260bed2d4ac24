"""Autotuner host logic (no GPU): shape classes, cache keys and the JSON
cache's round trip."""
import json

from marching_cube_gb300 import tune


def test_shape_class_rounds_edges_up():
    assert tune.shape_class((512, 512, 512), 0) == "short2-512x512x512"
    assert tune.shape_class((300, 100, 513), 1) == "float2-1024x128x512"
    assert tune.cache_key("GB300", (5, 6, 7), 0) == "GB300|short2-8x8x8"


def test_cache_round_trip(tmp_path):
    path = str(tmp_path / "sub" / "tune.json")
    assert tune.load_cache(path) == {}
    tune.store_cache("a|b", {"config": {"fused": 0, "classify_shape": 3, "gen_fixed_rounds": 2}, "ms": 0.2}, path)
    tune.store_cache("c|d", {"config": {"fused": 1, "classify_shape": 4, "gen_fixed_rounds": 3}, "ms": 0.1}, path)
    d = tune.load_cache(path)
    assert set(d) == {"a|b", "c|d"} and d["a|b"]["config"]["classify_shape"] == 3
    with open(path) as f:
        assert json.load(f) == d
    # a damaged cache file reads as empty and is replaced on the next store
    with open(path, "w") as f:
        f.write("{not json")
    assert tune.load_cache(path) == {}
    tune.store_cache("e|f", {"config": {"fused": 0, "classify_shape": 0, "gen_fixed_rounds": 0}}, path)
    assert set(tune.load_cache(path)) == {"e|f"}
