"""Build recipe of the engine library `libpfgpu.so` (sm_103a only).

Every CUDA translation unit is compiled by nvcc in parallel with
`-gencode arch=compute_103a,code=sm_103a`, then linked with the host
generator code into one shared library next to this file.

The seeded instance generators (csrc/gen.cpp) are also linked alone into
`libpfgen.so`, a host-only library without CUDA: CPU-side users of the
generators (the reference arm of bench.py, fixture scripts) load that one, so
they never map the engine.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(HERE, "libpfgpu.so")
GEN_LIB = os.path.join(HERE, "libpfgen.so")
BUILD_DIR = os.path.join(HERE, "_build")

CU_SOURCES = ["prims.cu", "ot.cu", "gc.cu", "bcp.cu", "lcve.cu", "elim.cu", "engine.cu", "server.cu", "tune.cu"]
CPP_SOURCES = ["gen.cpp", "dimacs.cpp", "vmap.cpp", "proof.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpfgpu.so")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "pfgpu.h"))
    return files


def _up_to_date() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(GEN_LIB):
        return False
    t = min(os.path.getmtime(LIB), os.path.getmtime(GEN_LIB))
    return all(os.path.getmtime(f) <= t for f in _deps())


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + p.stdout + p.stderr)
    return p.stderr


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    if not force and _up_to_date():
        return LIB
    nvcc = nvcc_path()
    os.makedirs(BUILD_DIR, exist_ok=True)
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        extra = ["-Xptxas", "-v"] if ptxas_info else []
        jobs.append([nvcc, *ARCH, *common, *extra, "-c", os.path.join(CSRC, src), "-o", obj])
        objs.append(obj)
    for src in CPP_SOURCES:
        obj = os.path.join(BUILD_DIR, src.replace(".cpp", ".o"))
        jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-I", INCLUDE, "-c", os.path.join(CSRC, src), "-o", obj])
        objs.append(obj)
    logs = []
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        for log in ex.map(_run, jobs):
            logs.append(log)
    tmp = LIB + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs])
    os.replace(tmp, LIB)
    gen_obj = os.path.join(BUILD_DIR, "gen.o")
    _run(["g++", "-shared", "-o", GEN_LIB + ".tmp", gen_obj])
    os.replace(GEN_LIB + ".tmp", GEN_LIB)
    if verbose or ptxas_info:
        sys.stderr.write("".join(logs))
    return LIB


if __name__ == "__main__":
    print(build(force=True, ptxas_info="-v" in sys.argv))
