"""The batched launch's push/pull divisor tuning (autotune.tune_batch /
lookup_batch): host logic only, with a stand-in for the batched run."""
import json
from types import SimpleNamespace

from belewitte_gb300 import autotune


class _Graph:
    """Just what shape_class reads."""

    def __init__(self, n, m, max_deg):
        import torch
        deg = torch.full((n,), m // n, dtype=torch.int64)
        deg[0] = max_deg
        self.fwd_vertices = torch.cat([torch.zeros(1, dtype=torch.int64), deg.cumsum(0)])
        self.vertex_count, self.edge_count = n, int(deg.sum())


def test_tune_batch_keeps_the_fastest_divisor(tmp_path):
    cache = tmp_path / "autotune.json"
    calls = []

    def run(d):
        calls.append(d)
        return SimpleNamespace(device_ms=abs(d - 48) + 1.0)   # fastest at 48

    best = autotune.tune_batch(None, run, "graphs", divisors=[8, 24, 48, 96], repeats=2, cache=cache)
    assert best == (48, 1.0)
    assert sorted(set(calls)) == [8, 24, 48, 96] and len(calls) == 4 * 3   # warm-up + 2 timed each
    data = json.loads(cache.read_text())
    assert data["batch"]["graphs"] == {"bu_div": 48, "ms": 1.0}
    assert autotune.lookup_batch("graphs", cache=cache) == 48


def test_lookup_batch_sources_nearest_shape_class(tmp_path):
    cache = tmp_path / "autotune.json"
    g_big = _Graph(1 << 12, 16 << 12, 4000)
    g_small = _Graph(1 << 8, 4 << 8, 20)
    key_big = autotune.batch_key("sources", g_big)
    assert key_big.startswith("sources/v12-")
    cache.write_text(json.dumps({"batch": {key_big: {"bu_div": 1024, "ms": 1.0}}}))
    assert autotune.lookup_batch("sources", g_big, cache=cache) == 1024
    # no entry for this class: the nearest cached class, when it is close
    g_near = _Graph(1 << 13, 16 << 13, 8000)
    assert autotune.batch_key("sources", g_near) != key_big
    assert autotune.lookup_batch("sources", g_near, cache=cache) == 1024
    # a graph far from every cached class keeps the library default
    assert autotune.class_distance(key_big.split("/")[1], autotune.shape_class(g_small)) > autotune.MAX_CLASS_DISTANCE
    assert autotune.lookup_batch("sources", g_small, cache=cache) == 0
    # other modes and missing caches fall back to the library default (0)
    assert autotune.lookup_batch("graphs", cache=cache) == 0
    assert autotune.lookup_batch("sources", g_big, cache=tmp_path / "none.json") == 0


def test_shipped_cache_is_well_formed():
    if not autotune.CACHE.exists():
        return
    data = json.loads(autotune.CACHE.read_text())
    for key, entry in data.get("batch", {}).items():
        assert key == "graphs" or key.startswith("sources/v")
        assert int(entry["bu_div"]) >= 1 and float(entry["ms"]) > 0
