"""Build libsiminf_gb300.so in-tree with nvcc for sm_103a.

The library is the C ABI of include/siminf_gb300.h: siminf_kernels.cu (the
particle filter's kernels and the model lookup), siminf_models_a/b/c.cu
(the SSA and event kernels, one instantiation per shipped model),
siminf_capi.cpp (planning
and the exported entry points), siminf_noalloc.cu (the allocation-free
solver entry point and its static scratch), siminf_batch.cu (batches of
uneven models), siminf_server.cpp (the request loop), siminf_reduce.cu (trajectory and
prevalence on the device) and siminf_events.cu (the event table's ordering
on the device), compiled in parallel and linked with nvcc.

    python -m siminf_gb300.build
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libsiminf_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no fused multiply-add, so every double rounds as in the
# reference's C (bit-identical trajectories).
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off"]
SOURCES = ["siminf_kernels.cu", "siminf_models_a.cu", "siminf_models_b.cu", "siminf_models_c.cu",
           "siminf_capi.cpp", "siminf_noalloc.cu", "siminf_batch.cu", "siminf_server.cpp",
           "siminf_reduce.cu", "siminf_events.cu", "siminf_individual.cu", "siminf_schedule.cu"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
             if f.endswith((".cu", ".cuh", ".h", ".cpp"))]
    files.append(os.path.join(HERE, "..", "include", "siminf_gb300.h"))
    return files


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        cmd = [cc] + ARCH + NVFLAGS + ["-I", CSRC, "-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cpp"):
            cmd = [cc] + NVFLAGS + ["-x", "cu", "-I", CSRC, "-c",
                                    os.path.join(CSRC, src), "-o", obj] + ARCH
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
        return obj

    with ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    subprocess.check_call([cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-ldl"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
