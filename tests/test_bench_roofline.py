"""bench.py's roofline arithmetic (host logic, no GPU): algorithmic bytes per
kernel class and the dominant-class pick."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


class _Scene:
    def __init__(self, name, w, h, shadow=None):
        self.name, self.width, self.height = name, w, h
        self.info = {"shadow_size": shadow} if shadow else {}


def test_radix_passes_match_the_device_rule():
    # 8 bits of bin index per pass (setup_bin.cu radix_passes)
    assert bench._radix_passes(32, 32, 32) == 0          # one bin: no sort
    assert bench._radix_passes(256 * 32, 32, 32) == 1     # 256 bins
    assert bench._radix_passes(257 * 32, 32, 32) == 2     # 257 bins
    assert bench._radix_passes(2048, 2048, 32) == 2       # 4096 bins
    assert bench._radix_passes(8192, 8192, 32) == 2       # 65536 bins
    assert bench._radix_passes(8192, 8192, 8) == 3        # 262144 bins


def test_kernel_bytes_per_class():
    sc = _Scene("c2", 1920, 1080, shadow=2048)
    counts = {"pairs": 1000, "triangles": 500, "shaded": 300}
    assert bench.kernel_bytes_per_frame("setup", sc, counts, 32) == 500 * 112 + 1000 * 8
    assert bench.kernel_bytes_per_frame("sort", sc, counts, 32) == 1000 * 16 * 2
    bins = 60 * 34 + 64 * 64
    assert bench.kernel_bytes_per_frame("bounds", sc, counts, 32) == bins * 8
    assert bench.kernel_bytes_per_frame("shade", sc, counts, 32) == 300 * 12
    assert bench.kernel_bytes_per_frame("raster", sc, counts, 32) == \
        bench.algorithmic_bytes(sc, counts)["raster_per_frame"]


def test_dominant_roofline_uses_the_top_class_per_launch():
    sc = _Scene("c1", 640, 480)
    counts = {"pairs": 4000, "triangles": 992, "shaded": 70000}
    # 10 profiled frames: raster 10 launches 2.0 ms in all, sort 10 launches 1.0 ms
    prof = {"raster": (10, 2.0), "sort": (10, 1.0), "setup": (10, 0.5), "bounds": (10, 0.1), "shade": (10, 0.2)}
    r = bench.dominant_roofline(prof, 10, sc, counts, 16, {"raster": 1234})
    per_launch = bench.algorithmic_bytes(sc, counts)["raster_per_frame"]
    assert r["kernel"] == "raster" and r["traffic"] == 1234
    assert r["bytes_per_launch"] == round(per_launch)
    assert abs(r["achieved"] - per_launch / 0.2e-3 / 1e9) < 0.01
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-4
    prof["sort"] = (10, 3.0)
    r = bench.dominant_roofline(prof, 10, sc, counts, 16, {"raster": 1234})
    assert r["kernel"] == "sort" and r["traffic"] is None
    assert r["bytes_per_launch"] == 4000 * 16 * 2
