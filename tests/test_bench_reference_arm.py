"""The benchmark's reference arm (`bench.py --impl reference`) on the CPU: one JSON line
with the reference's metric and unit, `impl: reference`, a `cpu_baseline` describing the
run and an `e2e` object with no host<->device bytes; ranks other than 0 print nothing.
The arm builds its frame from numpy and the oracle alone: the GPU library is never
loaded in its process, and its `config` is the one the GPU arm prints for the same frame."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# runs bench.py's reference arm in this process, then reports the shared objects it mapped
# and the modules it imported
_WRAP = r"""
import json, runpy, sys
sys.argv = ["bench.py"] + sys.argv[1:]
runpy.run_path("bench.py", run_name="__main__")
maps = open("/proc/self/maps").read()
print("MAPS " + json.dumps({"so": sorted({l.split()[-1] for l in maps.splitlines() if l.endswith(".so")}),
                            "modules": sorted(m for m in sys.modules if m.startswith("proland_gb300"))}))
"""


def run(env_extra, requests=256):
    env = dict(os.environ, **env_extra)
    out = subprocess.run([sys.executable, "-c", _WRAP, "--impl", "reference", "--steps", "2",
                          "--warmup", "1", "--requests", str(requests)],
                         cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip()]
    maps = json.loads(lines[-1][5:])
    return lines[:-1], maps


def test_reference_arm_line():
    lines, maps = run({"RANK": "0"})
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["unit"] == "tiles/s" and d["higher_is_better"] is True and d["value"] > 0
    assert d["steps"] == 2 and d["warmup"] == 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["same_results_as_oracle"] is True
    assert "256 tiles" in d["cpu_baseline"]["sample"]          # the whole frame, not a sample of it
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "workload" in d["config"]
    # nothing of the product is loaded
    assert not any("libproland_gb300" in p for p in maps["so"]), maps["so"]
    assert maps["modules"] == []
    assert any("liboracle" in p for p in maps["so"])


def test_reference_arm_config_is_the_gpu_arms():
    """Both arms name the frame with the same `config` (bench.frame_config over the
    same seeded requests; the noise choice is the only input the arms take from
    different code, and the two choices are identical)."""
    sys.path.insert(0, ROOT)
    import bench
    import oracle
    lines, _ = run({"RANK": "0"})
    ref = json.loads(lines[0])["config"]
    classes = bench.make_frame(256, 2024, oracle.noise_select)
    assert ref == bench.frame_config(classes, 1)


def test_reference_arm_other_ranks_print_nothing():
    lines, _ = run({"RANK": "1"})
    assert lines == []
