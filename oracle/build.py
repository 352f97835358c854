"""Build recipe for the CPU oracle (test infrastructure only).

Compiles gsim_oracle.c into oracle/_build/libgsim_oracle.so with plain gcc.
-ffp-contract=off keeps every rounding step explicit; the fused multiply-adds of the
canonical arithmetic are written out with fmaf().  No -march flags: the same source
builds on x86_64 and aarch64 and gives the same bits on both.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgsim_oracle.so")
SOURCES = [os.path.join(HERE, "gsim_oracle.c")]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = SOURCES + [os.path.join(HERE, "gsim_oracle.h")]
    if not force and os.path.exists(LIB):
        lib_mtime = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= lib_mtime for d in deps):
            return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-ffp-contract=off", "-fno-fast-math",
           "-fPIC", "-shared", "-pthread", "-Wall", "-Wextra", "-o", LIB + ".tmp"] + SOURCES + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
