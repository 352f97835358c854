"""Build recipe for libgsim.so (the C ABI of include/gsim.h) for sm_103a.

Every translation unit is compiled by nvcc in parallel with one -gencode
(compute_103a -> sm_103a) and linked into gravity-sim_gb300/lib/libgsim.so.  Kernels are
compiled with --fmad=false: every fused multiply-add in them is written out with fmaf(),
so the rounding sequence is the one the CPU restatement reproduces.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libgsim.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=hidden", "-I" + INCLUDE]
CUDA_SOURCES = ["force_fast.cu", "force_exact.cu", "bh.cu", "direct.cu", "sim.cu", "batch.cu", "serve.cu",
                "render.cu", "tune.cu"]
CXX_SOURCES = ["host.cpp"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def build(force: bool = False, verbose: bool = False, ptxas_verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    jobs, objs = [], []
    for src in CUDA_SOURCES + CXX_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + headers):
            if src.endswith(".cu"):
                cmd = [nvcc] + ARCH + NVCC_FLAGS + (["-Xptxas", "-v"] if ptxas_verbose else []) + ["-c", path, "-o", obj]
            else:
                cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-I" + INCLUDE, "-c", path, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, len(jobs)))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or ptxas_verbose or r.returncode:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError("compile failed: " + cmd[-3])
    if jobs or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart_static", "-lpthread", "-ldl", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("link failed")
        os.replace(LIB + ".tmp", LIB)
    cli_src = os.path.join(HERE, "cli", "main.cpp")
    cli = os.path.join(LIBDIR, "gsim-cli")
    if force or _stale(cli, [cli_src, LIB, os.path.join(INCLUDE, "gsim.hpp")]):
        cmd = ["g++", "-O2", "-std=c++17", "-I" + INCLUDE, cli_src, "-o", cli + ".tmp", "-L" + LIBDIR, "-lgsim",
               "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("cli link failed")
        os.replace(cli + ".tmp", cli)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, ptxas_verbose="--ptxas" in sys.argv))
