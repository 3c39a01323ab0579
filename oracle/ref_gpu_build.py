"""Recipe that compiles the reference's GPU simplifier (TEST INFRASTRUCTURE
ONLY): the source of the golden fixtures under tests/golden/refgpu.

The reference's sources (src/gpu and the vendored dep/moderngpu) are read
from the directory named by PFG_REFERENCE_DIR (default: the reference
checkout this repository was built beside) and staged, unmodified, into
oracle/_ref/src/gpu and oracle/_ref/dep/moderngpu, so that a GPU host
without the checkout builds from the staged copy; oracle/_ref is never
committed. The reference's install.sh / Makefile are not run.

Two things the reference build takes from outside its tree are supplied
here: the cuArena device-pool library (an empty git submodule in the
reference; oracle/refgpu/cuarena/allocator.cuh implements the part the
reference calls) and the generated version header. nvcc compiles every
src/gpu translation unit except main.cpp with the reference's own flags
(install.sh: -O3 -DNDEBUG --std c++20 -rdc=true, --expt-extended-lambda,
--expt-relaxed-constexpr, -DEXTSHMEM for compute capability >= 7) for
sm_103a, plus oracle/refgpu/dump_main.cpp in place of main, into
oracle/_ref/gpu/pfref_gpu.

Usage: python oracle/ref_gpu_build.py stage   (where the checkout exists)
       python oracle/ref_gpu_build.py build   (stage if possible, compile)
"""
import concurrent.futures as cf
import glob
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
STAGE_SRC = os.path.join(OUT, "src", "gpu")
STAGE_DEP = os.path.join(OUT, "dep")
BUILD = os.path.join(OUT, "gpu")
BIN = os.path.join(BUILD, "pfref_gpu")
SHIM = os.path.join(HERE, "refgpu")
DUMP_MAIN = os.path.join(SHIM, "dump_main.cpp")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def compat_includes() -> list:
    """On hosts that are not x86, the include path of the stand-in <cpuid.h>
    (oracle/refcompat): the reference reads the CPU brand string through it."""
    if platform.machine().lower() in ("x86_64", "amd64", "i386", "i686"):
        return []
    return ["-I", os.path.join(HERE, "refcompat")]


def reference_dir() -> str:
    return os.environ.get("PFG_REFERENCE_DIR", os.path.join(os.sep, "root", "reference"))


def _copy_tree(src, dst, exts):
    os.makedirs(dst, exist_ok=True)
    for f in os.listdir(src):
        if f.endswith(exts):
            a, b = os.path.join(src, f), os.path.join(dst, f)
            if not os.path.exists(b) or os.path.getmtime(b) < os.path.getmtime(a):
                shutil.copy2(a, b)


def stage() -> bool:
    """Copy the reference GPU sources into oracle/_ref; False when absent."""
    ref = reference_dir()
    src = os.path.join(ref, "src", "gpu")
    mgpu = os.path.join(ref, "dep", "moderngpu")
    if not os.path.isdir(src):
        return False
    _copy_tree(src, STAGE_SRC, (".cu", ".cuh", ".cpp", ".hpp", ".h"))
    _copy_tree(mgpu, os.path.join(STAGE_DEP, "moderngpu"), (".hxx", ".h", ".hpp"))
    return True


def _version_header(gen):
    os.makedirs(gen, exist_ok=True)
    with open(os.path.join(gen, "version.hpp"), "w") as f:
        # declarations the sources expect from their generated version header
        f.write('#pragma once\nnamespace ParaFROST {\n'
                'const char* version(); const char* signature(); const char* compiler();\n'
                'const char* compilemode(); const char* osystem(); const char* date();\n}\n'
                '#define VERSION "4.1.1"\n#define OSYSTEM "linux"\n#define DATE "oracle"\n'
                '#define COMPILER "g++ + nvcc"\n')


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def build(force: bool = False) -> str:
    stage()
    if not os.path.isdir(STAGE_SRC):
        raise FileNotFoundError("reference GPU sources are neither present nor staged")
    gen = os.path.join(BUILD, "gen")
    objd = os.path.join(BUILD, "obj")
    os.makedirs(objd, exist_ok=True)
    _version_header(gen)
    nvcc = _nvcc()
    flags = ["-m64", *ARCH, "--std", "c++20", "-DNDEBUG", "-O3", "-DEXTSHMEM", "--expt-extended-lambda",
             "--expt-relaxed-constexpr", "-rdc=true", "-I", STAGE_DEP, "-I", SHIM, "-I", gen, "-I", STAGE_SRC,
             "-Xcompiler", "-std=c++20,-O3", "-w", *compat_includes()]
    srcs = sorted(glob.glob(os.path.join(STAGE_SRC, "*.cu")) + glob.glob(os.path.join(STAGE_SRC, "*.cpp")))
    srcs = [s for s in srcs if os.path.basename(s) != "main.cpp"] + [DUMP_MAIN]
    headers = glob.glob(os.path.join(STAGE_SRC, "*.*h")) + [os.path.join(SHIM, "cuarena", "allocator.cuh")]
    newest_header = max(os.path.getmtime(h) for h in headers)

    def cc(src):
        base = os.path.basename(src)
        obj = os.path.join(objd, base + ".o")
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), newest_header):
            p = subprocess.run([nvcc, *flags, "-c", src, "-o", obj], capture_output=True, text=True)
            if p.returncode != 0:
                raise RuntimeError(f"compiling {base} failed:\n{p.stdout}{p.stderr}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(cc, srcs))
    p = subprocess.run([nvcc, "-m64", *ARCH, "-rdc=true", "-o", BIN + ".tmp", *objs], capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"linking pfref_gpu failed:\n{p.stdout}{p.stderr}")
    os.replace(BIN + ".tmp", BIN)
    return BIN


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "build"
    if what == "stage":
        print("staged" if stage() else "reference sources not found")
    else:
        print(build(force="--force" in sys.argv))
