"""The autotuner's stored tables (pe_gb300.autotune): a table written for a GPU model and real type is
read back for that model and type only, unknown models give no settings, and every candidate value
the tuner tries lies in the ranges pe_gpu_set_tuning accepts (include/pe_gpu.h)."""
from pe_gb300 import autotune


def test_table_round_trip(tmp_path, monkeypatch):
    monkeypatch.setattr(autotune, "TABLE_DIR", tmp_path)
    settings = {"sat_heavy_cost": 400000, "side_streams": 2}
    p = autotune.save_table("NVIDIA GB300", 32, settings, {"mode": "coloured"})
    assert p.parent == tmp_path and p.name == "NVIDIA_GB300.json"
    assert autotune.load_table("NVIDIA GB300", 32) == settings
    assert autotune.load_table("NVIDIA GB300", 64) == {}
    assert autotune.load_table("Some Other GPU", 32) == {}


def test_candidates_are_valid_settings():
    ok = {"sat_heavy_cost": lambda v: v >= 1, "side_streams": lambda v: 1 <= v <= 4,
          "small_island_items": lambda v: 0 <= v <= 64, "color_block": lambda v: 32 <= v <= 256 and v % 32 == 0,
          "level_block": lambda v: 32 <= v <= 256 and v % 32 == 0, "big_island_items": lambda v: 64 < v <= (1 << 24),
          "scene_sort_max": lambda v: 0 <= v <= 2048}
    for name, values in autotune.CANDIDATES.items():
        assert all(ok[name](v) for v in values), name
