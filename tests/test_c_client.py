"""The C ABI from plain C: compile tests/c/c_abi_client.c against the header and
the library with gcc (C99, pedantic) and run its host-side checks (no GPU)."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_c_client_runs(product, tmp_path):
    lib_dir = os.path.dirname(product.LIB_PATH)
    exe = str(tmp_path / "c_abi_client")
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(HERE, "c", "c_abi_client.c"), "-o", exe, "-L", lib_dir, "-lproland_gb300",
           "-Wl,-rpath," + lib_dir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([exe, os.path.join(HERE, "golden", "dem_terrain4_mini.dat"),
                          os.path.join(HERE, "golden", "rgb_graph1_mini.dat")], capture_output=True, text=True,
                         timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr
    assert run.stdout.strip().endswith("all ok")
