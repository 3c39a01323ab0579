"""Recipe that compiles the reference's CPU solver (TEST AND BASELINE
INFRASTRUCTURE ONLY).

The reference's sources are read from the directory named by the
environment variable PFG_REFERENCE_DIR (default: the reference checkout this
repository was built beside). When that directory is present they are first
staged, unmodified, into oracle/_ref/src/cpu, so that a machine without the
checkout (the GPU hosts) still builds from the staged copy; oracle/_ref is
never committed. The reference's own build system is not run: g++ compiles
the files of src/cpu directly into

  oracle/_ref/parafrost       the reference's CLI (its own main.cpp), used by
                              the CPU tests as a satisfiability oracle;
  oracle/_ref/pfref_cpu_time  oracle/refcpu/time_main.cpp in place of main:
                              times Solver::sigmify on one file, for the
                              reference arm of bench.py and its cpu_baseline.

Only a generated version header is written beside the staged sources.
"""
import concurrent.futures as cf
import glob
import os
import platform
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
STAGE = os.path.join(OUT, "src", "cpu")
BIN = os.path.join(OUT, "parafrost")
TIME_BIN = os.path.join(OUT, "pfref_cpu_time")
TIME_MAIN = os.path.join(HERE, "refcpu", "time_main.cpp")
# Solver::SUB, wrapped at link time to count the clauses entering each round
SUB_SYMBOL = "_ZN9ParaFROST6Solver3SUBEv"


def compat_includes() -> list:
    """On hosts that are not x86, the include path of the stand-in <cpuid.h>
    (oracle/refcompat): the reference reads the CPU brand string through it."""
    if platform.machine().lower() in ("x86_64", "amd64", "i386", "i686"):
        return []
    return ["-I", os.path.join(HERE, "refcompat")]


def reference_dir() -> str:
    return os.environ.get("PFG_REFERENCE_DIR", os.path.join(os.sep, "root", "reference"))


def _src_dir() -> str:
    return os.path.join(reference_dir(), "src", "cpu")


def available() -> bool:
    """True when the reference sources (or their staged copy) are present."""
    return os.path.isdir(_src_dir()) or os.path.isdir(STAGE)


def stage() -> str:
    """Copy src/cpu of the reference checkout into oracle/_ref/src/cpu."""
    src = _src_dir()
    if not os.path.isdir(src):
        if os.path.isdir(STAGE):
            return STAGE
        raise FileNotFoundError(f"reference CPU sources not found at {src}")
    os.makedirs(STAGE, exist_ok=True)
    for f in os.listdir(src):
        if f.endswith((".cpp", ".h", ".hpp")):
            a, b = os.path.join(src, f), os.path.join(STAGE, f)
            if not os.path.exists(b) or os.path.getmtime(b) < os.path.getmtime(a):
                shutil.copy2(a, b)
    return STAGE


def _version_header(gen):
    os.makedirs(gen, exist_ok=True)
    with open(os.path.join(gen, "version.h"), "w") as f:
        # declarations the sources expect from their generated version header
        f.write('#pragma once\nnamespace ParaFROST {\n'
                'const char* version(); const char* signature(); const char* compiler();\n'
                'const char* compilemode(); const char* osystem(); const char* date();\n}\n'
                '#define VERSION "3.2.5"\n#define OSYSTEM "linux"\n#define DATE "oracle"\n'
                '#define COMPILER "g++"\n')


def build(force: bool = False) -> str:
    src_dir = stage()
    srcs = sorted(glob.glob(os.path.join(src_dir, "*.cpp")))
    deps = srcs + [TIME_MAIN, os.path.abspath(__file__)]
    outs = (BIN, TIME_BIN)
    if not force and all(os.path.exists(o) for o in outs) and \
            all(os.path.getmtime(s) <= min(os.path.getmtime(o) for o in outs) for s in deps):
        return BIN
    gen = os.path.join(OUT, "gen")
    objd = os.path.join(OUT, "obj")
    os.makedirs(objd, exist_ok=True)
    _version_header(gen)
    flags = ["-std=c++20", "-O3", "-DNDEBUG", "-I", gen, "-I", src_dir, "-w", *compat_includes()]

    def cc(src):
        obj = os.path.join(objd, os.path.basename(src).replace(".cpp", ".o"))
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < os.path.getmtime(src):
            subprocess.check_call(["g++", *flags, "-c", src, "-o", obj])
        return obj

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(cc, srcs + [TIME_MAIN]))
    time_obj = objs.pop()
    main_obj = [o for o in objs if os.path.basename(o) == "main.o"]
    lib_objs = [o for o in objs if os.path.basename(o) != "main.o"]
    subprocess.check_call(["g++", "-O3", "-o", BIN + ".tmp", *main_obj, *lib_objs, "-lpthread"])
    os.replace(BIN + ".tmp", BIN)
    subprocess.check_call(["g++", "-O3", f"-Wl,--wrap={SUB_SYMBOL}", "-o", TIME_BIN + ".tmp", time_obj, *lib_objs,
                           "-lpthread"])
    os.replace(TIME_BIN + ".tmp", TIME_BIN)
    return BIN


if __name__ == "__main__":
    print(build(force=True))
