"""The byte accounting behind the bench line's live bandwidth figures (CPU
only): radix passes follow the key width of the grid, and each class's
achieved rate is its algorithmic bytes over its device time."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _prof(ms, units):
    return {"launches": 1, "ms": ms, "units": units}


def test_sort_passes_follow_the_key_width():
    peak = 1000.0
    # keys take the values 0..C (C = the out-of-grid sentinel), 8 bits a pass
    for cells, passes in [((4, 4, 4), 1), ((16, 8, 2), 2), ((25, 25, 25), 2), ((248, 124, 124), 3),
                          ((512, 256, 256), 4)]:
        out = bench.stream_kernels({"sort": _prof(1.0, 1_000_000)}, {"cell_size": cells}, peak)
        assert out["sort"]["bytes_per_unit"] == 16 * passes + 4 * (passes - 1), cells


def test_achieved_rate_is_bytes_over_time():
    prof = {"hash": _prof(2.0, 10_000_000), "reorder": _prof(4.0, 10_000_000),
            "up_grid": _prof(8.0, 40_000_000), "sweep": _prof(1.0, 1)}
    out = bench.stream_kernels(prof, {"cell_size": (248, 124, 124)}, 6000.0)
    assert set(out) == {"hash", "reorder", "up_grid"}
    assert abs(out["hash"]["achieved_gbs"] - 24 * 10_000_000 / 2e-3 / 1e9) < 0.1
    assert abs(out["reorder"]["frac"] - round(124 * 10_000_000 / 4e-3 / 1e9 / 6000.0, 3)) < 1e-9
    assert out["up_grid"]["bytes_per_unit"] == 24 + 56 + 68


def test_classes_without_launches_are_left_out():
    prof = {"hash": {"launches": 0, "ms": 0.0, "units": 0}}
    assert bench.stream_kernels(prof, {"cell_size": (8, 8, 8)}, 6000.0) == {}
