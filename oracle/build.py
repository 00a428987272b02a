"""Builds the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.

The oracle is compiled with -ffp-contract=off so that each float operation is
rounded on its own, in the order the C source writes it; the CUDA product
follows the same order with explicitly rounded intrinsics.  No -march flag: the
same source must give the same bits on x86-64 and aarch64 hosts.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, "oracle.c"), os.path.join(HERE, "learned.c"), os.path.join(HERE, "ortho.c"),
            os.path.join(HERE, "layers.c")]
    hdr = os.path.join(HERE, "oracle.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max([os.path.getmtime(p) for p in srcs] + [os.path.getmtime(hdr)])):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-ffp-contract=off", "-fno-fast-math",
           "-fPIC", "-shared", "-pthread", "-Wall", "-o", tmp, *srcs, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


TUNED_LIB = os.path.join(OUT_DIR, "liboracle_tuned.so")


def build_tuned(force: bool = False) -> str:
    """The same sources at -O3 (floating-point contraction still off), built on the
    machine that runs them: the timed CPU baseline.  No machine-specific flag, so that
    the build gives the same bits on x86-64 and aarch64 hosts."""
    srcs = [os.path.join(HERE, "oracle.c"), os.path.join(HERE, "learned.c"), os.path.join(HERE, "ortho.c"),
            os.path.join(HERE, "layers.c")]
    hdr = os.path.join(HERE, "oracle.h")
    if (not force and os.path.exists(TUNED_LIB)
            and os.path.getmtime(TUNED_LIB) >= max([os.path.getmtime(p) for p in srcs] + [os.path.getmtime(hdr)])):
        return TUNED_LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = TUNED_LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-std=c11", "-D_GNU_SOURCE", "-ffp-contract=off", "-fno-fast-math",
           "-fPIC", "-shared", "-pthread", "-Wall", "-o", tmp, *srcs, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, TUNED_LIB)
    return TUNED_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
