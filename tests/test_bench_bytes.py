"""The benchmark's algorithmic bytes per tile, derived from the tile layout: a W-wide
elevation tile reads its parent's zf and zm over the child window ((n/2 + 5)^2 samples
each, n = W - 5), its W^2 residual, and writes zf, zc, zm (W^2 each) and the two normal
planes ((W - 4)^2 each), all fp32; an ortho tile reads its (W/2 + 2)^2 parent window
and W^2 residual texels and writes W^2 texels, RGBA8.  And the `clocks` record of a
run from nvidia-smi's samples (median clock, throttle reasons seen).  CPU only."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_elevation_and_ortho_bytes_per_tile():
    sys.path.insert(0, ROOT)
    import bench
    for W in (101, 197):
        n = W - 5
        window = (n // 2 + 5) ** 2
        want = 4 * (2 * window + W * W + 3 * W * W + 2 * (W - 4) ** 2)
        assert bench.BYTES_PER_TILE[W] == want, W
    assert bench.BYTES_PER_TILE == {101: 260960, 197: 1000544}
    Wo = bench.ORTHO_W
    assert bench.ORTHO_BYTES_PER_TILE == 4 * ((Wo // 2 + 2) ** 2 + 2 * Wo * Wo) == 347328


def test_clock_record_from_nvidia_smi_lines():
    sys.path.insert(0, ROOT)
    import bench
    lines = ["0, 2070, 2070, 1012.40, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active\n",
             "0, 1965, 2070, 1398.80, 0x0000000000000004, Not Active, Not Active, Not Active, Active\n",
             "0, 2070, 2070, 1100.00, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active\n",
             "garbage line\n", "0, [N/A], 2070, 0, 0x0, Not Active, Not Active, Not Active, Not Active\n"]
    rec = bench.clock_record(lines)
    assert rec == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    assert bench.clock_record(["garbage\n"]) is None
