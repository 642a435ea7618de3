"""Host-side pieces of bench.py that need no GPU: the DRAM traffic figure of the roofline comes
from the committed ncu summary, per sweep tile when the summary holds one per tile."""
import json

import bench


def test_traffic_per_tile(tmp_path, monkeypatch):
    prof = tmp_path / "profiles"
    prof.mkdir()
    (prof / "t.json").write_text(json.dumps({
        "dram_bytes_per_launch": 7,
        "by_tile": {"4": {"dram_bytes_per_launch": 4}, "8": {"dram_bytes_per_launch": 8}}}))
    (prof / "flat.json").write_text(json.dumps({"dram_bytes_per_launch": 5}))
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.ncu_traffic("t.json", 8) == 8
    assert bench.ncu_traffic("t.json", 4) == 4
    assert bench.ncu_traffic("t.json", 2) is None  # no capture of that tile: no figure
    assert bench.ncu_traffic("t.json") == 7
    assert bench.ncu_traffic("flat.json", 8) == 5
    assert bench.ncu_traffic("missing.json", 8) is None


def test_committed_summary_covers_the_bench_tiles():
    # the tiles the autotuner picks at L=256 have a committed traffic figure
    for tile in (4, 8):
        assert bench.ncu_traffic("sweep_l256_traffic.json", tile) > 67108864  # above the algorithmic bytes
