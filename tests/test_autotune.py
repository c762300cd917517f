"""The per-variant autotuner (autotune.tune / tuned_config / export_tsv):
host logic with a stand-in timer, and the shipped cache's form."""
import json

import pytest

from belewitte_gb300 import autotune
from tests.test_autotune_batch import _Graph


def test_candidates_start_with_the_library_default():
    for algo, name in (("bfs", "edge-list-bulk"), ("bfs", "vertex-pull-warp"), ("pagerank", "pull-segmented"),
                       ("pagerank", "vertex-push-warp"), ("pagerank", "rev-edge-list")):
        cands = list(autotune.candidates(algo, name, 152))
        assert cands[0] == {}
        assert len(cands) == len({json.dumps(c, sort_keys=True) for c in cands})      # no repeats
        for c in cands[1:]:
            if "chunk" in c:                                      # warp variants: the virtual warp
                assert c["block"] % c["warp"] == 0 and c["chunk"] % c["warp"] == 0
            elif "warp" in c:                                     # work-list kernels: the long-row threshold
                assert algo == "pagerank" and c["warp"] <= 512


def test_tune_keeps_the_fastest_and_writes_both_caches(tmp_path, monkeypatch):
    cache = tmp_path / "autotune.json"
    g = _Graph(1 << 12, 16 << 12, 4000)

    def fake_bfs(ctx, graph, name, root, cfg, repeats):        # fastest: block 512, grid 8 x SMs
        return 1.0 + abs(cfg.get("block", 0) - 512) / 100 + abs(cfg.get("grid", 0) - 8 * 152) / 1000

    monkeypatch.setattr(autotune, "_time_bfs", fake_bfs)

    class Ctx:
        sm_count = 152
    out = autotune.tune(Ctx(), g, "bfs", ["edge-list-bulk", "frontier-push"], cache=cache)
    assert out["edge-list-bulk"][0] == {"block": 512, "grid": 8 * 152}
    assert out["frontier-push"][0] == {"block": 256, "grid": 0} or out["frontier-push"][0] == {}
    cls = autotune.shape_class(g)
    data = json.loads(cache.read_text())
    assert data["bfs"]["edge-list-bulk"][cls]["config"] == {"block": 512, "grid": 8 * 152}
    tsv = cache.with_suffix(".tsv").read_text().splitlines()
    assert f"bfs\tedge-list-bulk\t{cls}\t512\t{8 * 152}\t0\t0" in tsv
    # tuned_config: this class, a near class, and a far one (library default)
    assert autotune.tuned_config("bfs", "edge-list-bulk", g, cache=cache) == {"block": 512, "grid": 8 * 152}
    near = _Graph(1 << 13, 16 << 13, 8000)
    assert autotune.tuned_config("bfs", "edge-list-bulk", near, cache=cache) == {"block": 512, "grid": 8 * 152}
    far = _Graph(1 << 8, 2 << 8, 4)
    assert autotune.tuned_config("bfs", "edge-list-bulk", far, cache=cache) == {}
    assert autotune.tuned_config("pagerank", "edge-list", g, cache=cache) == {}


def test_tuned_config_without_forward_offsets_is_the_default(tmp_path):
    class RevOnly:
        vertex_count, edge_count = 100, 1000
    assert autotune.tuned_config("pagerank", "vertex-pull", RevOnly()) == {}


def test_shipped_cache_entries_are_well_formed():
    if not autotune.CACHE.exists():
        pytest.skip("no cache shipped")
    data = json.loads(autotune.CACHE.read_text())
    tsv = autotune.CACHE.with_suffix(".tsv")
    lines = tsv.read_text().splitlines() if tsv.exists() else []
    count = 0
    for algo in ("bfs", "pagerank"):
        for name, classes in data.get(algo, {}).items():
            for cls, entry in classes.items():
                count += 1
                c = entry["config"]
                assert set(c) <= {"block", "grid", "warp", "chunk"}
                row = "\t".join([algo, name, cls] + [str(int(c.get(k, 0))) for k in ("block", "grid", "warp", "chunk")])
                assert row in lines
    assert count == len(lines)
