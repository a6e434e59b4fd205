"""Builds librrlbm.so in-tree with nvcc for sm_103a (one -gencode; the
kernels of each population storage type in one translation unit, or two for
the 16/32-bit types whose tile step and batch carry the packed-pair paths;
all compiled in parallel)."""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "rrlbm", "librrlbm.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INCLUDE = os.path.join(os.path.dirname(PKG), "include")
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall", "-I", INCLUDE]
# the longest compiles first
SOURCES = ["rr_inst_f16_tile.cu", "rr_inst_bf16_tile.cu", "rr_inst_f32_tile.cu", "rr_inst_f64.cu",
           "rr_inst_f32.cu", "rr_inst_f16.cu", "rr_inst_bf16.cu", "rr_aux.cu", "rr_api.cu", "rr_batch.cu",
           "rr_noalloc.cu"]
HEADERS = ["rr_lattice.cuh", "rr_node.cuh", "rr_node27.cuh", "rr_kernels.cuh", "rr_les.cuh", "rr_dispatch.h",
           "rr_aux.h", "rr_inst.inc", "rr_internal.h", "rr_stage.cuh", "rr_fdbc.cuh", "rr_pair.cuh"]



def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [
        os.path.join(os.path.dirname(PKG), "include", "rr_api.h")]
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        if force or _stale(o, [s] + hdrs):
            jobs.append([NVCC] + ARCH + FLAGS + ["-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=min(16, max(1, len(jobs)))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed on " + cmd[-3])
    objs = [os.path.join(BUILD, s.replace(".cu", ".o")) for s in SOURCES]
    if force or _stale(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
