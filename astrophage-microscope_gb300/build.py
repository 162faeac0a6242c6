"""Build libagb.so (the engine) in-tree: nvcc for sm_103a, translation units
compiled in parallel, linked with the CUDA runtime."""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libagb.so")
HEADLESS = os.path.join(HERE, "headless")       # the command-line scenario runner over the C ABI
SOURCES = ["k_grid.cu", "k_hash.cu", "k_cells.cu", "k_life.cu", "k_tau.cu", "world.cu", "batch.cu", "snapshot.cu", "conv_tc.cu", "nn_ops.cu", "nn_abi.cu", "surrogate.cu", "noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code that restates the reference's FP64 expressions (per-world constants)
# must not be contracted into FMAs by the host compiler (aarch64 gcc would).
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
         "-Xcompiler", "-ffp-contract=off", "--threads", "2"]


def nvcc():
    for p in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if p and (os.path.sep not in p or os.path.exists(p)):
            return p
    return "nvcc"


def _compile(src, extra):
    obj = os.path.join(BUILD, src.replace(".cu", ".o"))
    cmd = [nvcc()] + ARCH + FLAGS + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stdout + r.stderr))
    return obj, r.stdout + r.stderr


def build(verbose=False, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra)), SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log.strip():
                sys.stdout.write(log)
    cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    inc = os.path.join(os.path.dirname(HERE), "include")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-ffp-contract=off", "-I" + inc, os.path.join(CSRC, "headless.cpp"),
           "-o", HEADLESS, "-L" + HERE, "-lagb", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("headless build failed:\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    extra = sys.argv[1:]
    print(build(verbose=True, extra=extra))
