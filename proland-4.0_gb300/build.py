"""Builds libproland_gb300.so in-tree (proland-4.0_gb300/lib/) for sm_103a.

CUDA sources go through nvcc with one -gencode (compute_103a -> sm_103a); the
host C++ sources through g++ against the CUDA headers; translation units are
compiled in parallel and linked by nvcc with the static CUDA runtime, so the
library loads with or without PyTorch in the process.

build(debug=True) makes libproland_gb300_debug.so from the same sources with
TP_DEBUG defined: device-side bounds checks on the indexes of device job arrays
(a bad job is reported as TP_E_BOUNDS and skipped) and guard regions around every
storage's slots (tp_storage_check_guards).  The package loads it when the
environment variable PROLAND_GB300_DEBUG is 1.
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "lib")
OBJ_DIR = os.path.join(HERE, "lib", "obj")
LIB = os.path.join(LIB_DIR, "libproland_gb300.so")
DEBUG_LIB = os.path.join(LIB_DIR, "libproland_gb300_debug.so")
DEBUG_OBJ_DIR = os.path.join(HERE, "lib", "obj_debug")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(INCLUDE, "*.h"))


def _compile(src, verbose_ptxas=False, debug=False):
    obj = os.path.join(DEBUG_OBJ_DIR if debug else OBJ_DIR, os.path.basename(src) + ".o")
    defs = ["-DTP_DEBUG=1"] if debug else []
    if src.endswith(".cu"):
        cmd = [NVCC, "-c", src, "-o", obj, "-O3", "-std=c++17", "-lineinfo", *ARCH,
               "-Xcompiler", "-fPIC", "-I", INCLUDE, "--expt-relaxed-constexpr", *defs]
        if verbose_ptxas:
            cmd += ["-Xptxas", "-v"]
    else:
        # -ffp-contract=off: host arithmetic (residual pyramids) rounds each operation
        # as written on x86-64 and aarch64 alike
        cmd = ["g++", "-c", src, "-o", obj, "-O2", "-std=c++17", "-fPIC", "-Wall", "-ffp-contract=off",
               "-I", INCLUDE, "-I", os.path.join(CUDA_HOME, "include"), *defs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj, r.stderr


def build(force=False, verbose_ptxas=False, quiet=True, debug=False):
    srcs = _sources()
    lib, obj_dir = (DEBUG_LIB, DEBUG_OBJ_DIR) if debug else (LIB, OBJ_DIR)
    newest = max(os.path.getmtime(p) for p in srcs + _headers() + [__file__])
    if not force and os.path.exists(lib) and os.path.getmtime(lib) >= newest:
        return lib
    os.makedirs(obj_dir, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose_ptxas, debug), srcs))
    if verbose_ptxas or not quiet:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    tmp = lib + ".tmp%d" % os.getpid()
    cmd = [NVCC, "-shared", "-o", tmp, *[o for o, _ in results], *ARCH, "-cudart", "static",
           "-Xlinker", "--no-undefined", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv, quiet=False, debug="--debug" in sys.argv))
