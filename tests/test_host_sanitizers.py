"""The library's host C++ (storages, caches, producers, sampler, scheduler) under
AddressSanitizer + UndefinedBehaviorSanitizer and under ThreadSanitizer: its .cpp
sources are compiled with the sanitizer, linked with the CUDA objects of the normal
build and the static CUDA runtime, and driven by tests/c/cache_stress.cpp (threads
acquiring, releasing, prefetching and looking up tiles of shared producers on
bookkeeping-only storages, an invalidating thread, a sampling thread).  CPU only;
the run must end cleanly with no sanitizer report.  Under AddressSanitizer the
residual and ortho pyramid readers and the inflate decoder also read damaged and
truncated copies of the test fixtures (tests/c/dat_fuzz.cpp)."""
import concurrent.futures as cf
import glob
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "proland-4.0_gb300")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")

SANITIZERS = {
    "address": (["-fsanitize=address,undefined", "-fno-sanitize-recover=undefined", "-fno-omit-frame-pointer"],
                {"ASAN_OPTIONS": "detect_leaks=0:abort_on_error=0", "UBSAN_OPTIONS": "print_stacktrace=1"}),
    "thread": (["-fsanitize=thread"], {"TSAN_OPTIONS": "halt_on_error=1:second_deadlock_stack=1"}),
}


def _compile(args):
    r = subprocess.run(args, capture_output=True, text=True)
    return r.returncode, " ".join(args), r.stderr[-3000:]


@pytest.mark.parametrize("kind", sorted(SANITIZERS))
def test_cache_protocol_under_sanitizer(product, tmp_path, kind):
    cu_objs = sorted(glob.glob(os.path.join(PKG, "lib", "obj", "*.cu.o")))
    if not cu_objs:
        pytest.skip("the library's CUDA objects are not built")
    static_rt = os.path.join(CUDA, "lib64", "libcudart_static.a")
    if not os.path.exists(static_rt):
        pytest.skip("no static CUDA runtime")
    flags, env_extra = SANITIZERS[kind]
    common = ["-O1", "-g", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
              "-I", os.path.join(CUDA, "include")] + flags
    jobs = []
    objs = []
    drivers = ["cache_stress.cpp"] + (["dat_fuzz.cpp"] if kind == "address" else [])
    lib_objs = []
    for src in sorted(glob.glob(os.path.join(PKG, "csrc", "*.cpp"))) + [os.path.join(HERE, "c", d) for d in drivers]:
        obj = str(tmp_path / (os.path.basename(src) + ".o"))
        (objs if os.path.basename(src) in drivers else lib_objs).append(obj)
        jobs.append(["g++", "-c", src, "-o", obj] + common)
    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        for rc, cmd, err in ex.map(_compile, jobs):
            assert rc == 0, (cmd, err)
    env = dict(os.environ, **env_extra)
    for drv, obj in zip(drivers, objs):
        exe = str(tmp_path / drv[:-4])
        link = ["g++"] + flags + [obj] + lib_objs + cu_objs + [static_rt, "-ldl", "-lpthread", "-lrt", "-o", exe]
        r = subprocess.run(link, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        args = [exe]
        if drv == "dat_fuzz.cpp":
            args += [os.path.join(HERE, "golden", "dem_terrain4_mini.dat"),
                     os.path.join(HERE, "golden", "rgb_graph1_mini.dat"), str(tmp_path / "fuzz.dat"), "1500"]
        run = subprocess.run(args, capture_output=True, text=True, timeout=600, env=env)
        out = run.stdout + run.stderr
        assert run.returncode == 0, (drv, out[-6000:])
        assert ("cache stress ok" if drv == "cache_stress.cpp" else "dat fuzz ok") in run.stdout
        assert "Sanitizer" not in run.stderr and "runtime error" not in run.stderr, (drv, run.stderr[-6000:])
