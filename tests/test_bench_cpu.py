"""bench.py's roofline arithmetic on CPU (no GPU, no library)."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_l2_sector_roofline():
    """The SpMV's sectors (one per gather plus streamed bytes / 32) against the probe's (one per
    gather plus one per eight index reads): 1e8 gathers and 1.28e9 streamed bytes in 0.5 ms
    against a probe of 2.5e11 gathers/s."""
    r = bench.l2_sector_roofline(1e8, 1.28e9, 0.5, 2.5e11)
    assert r["unit"] == "sectors/s"
    assert abs(r["achieved"] - (1e8 + 4e7) / 5e-4) < 1.0
    assert abs(r["peak"] - 2.8125e11) < 1.0
    assert abs(r["frac"] - 2.8e11 / 2.8125e11) < 1e-12
    assert abs(r["floor_ms"] - 1.4e8 / 2.8125e11 * 1e3) < 1e-12
