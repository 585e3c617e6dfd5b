"""The far-tile autotuner's host logic: the choice per size class from measured records, the lookup by mesh size,
and the committed table's shape (tiles the library has, classes in increasing size)."""
import os

from vortexpanel_gpu import autotune


def test_table_picks_the_fastest_tile_per_size():
    recs = [{"ntri": 2000, "precision": "mixed", "tile": 4, "far_ms": 1.0},
            {"ntri": 2000, "precision": "mixed", "tile": 8, "far_ms": 2.0},
            {"ntri": 20000, "precision": "mixed", "tile": 4, "far_ms": 9.0},
            {"ntri": 20000, "precision": "mixed", "tile": 8, "far_ms": 7.0},
            {"ntri": 2000, "precision": "fp64", "tile": 2, "far_ms": 3.0},
            {"ntri": 2000, "precision": "fp64", "tile": 4, "far_ms": 2.5}]
    t = autotune.table(recs)
    assert t["mixed"][0]["tile"] == 4 and t["mixed"][1]["tile"] == 8
    assert 2000 < t["mixed"][0]["max_ntri"] < 20000
    assert autotune.far_tile("mixed", 1500, t) == 4
    assert autotune.far_tile("mixed", 50000, t) == 8
    assert autotune.far_tile("fp64", 100, t) == 4
    assert autotune.far_tile("fp32", 100, t) is None


def test_committed_table():
    if not os.path.exists(autotune.TABLE_FILE):
        return
    t = autotune.load_table()
    for prec, rows in t.items():
        assert prec in autotune.TILES
        ns = [r["max_ntri"] for r in rows]
        assert ns == sorted(ns)
        assert all(r["tile"] in autotune.TILES[prec] for r in rows)
