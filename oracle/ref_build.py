"""Recipe that compiles the reference's CPU solver (TEST INFRASTRUCTURE ONLY).

Compiles the sources where they lie under /root/reference/src/cpu with g++
(its own few source files; the reference's build system is not run) into
oracle/_ref/parafrost. The binary is used by the CPU tests as a second
satisfiability oracle and, where present, as an informational CPU timing.
Only a generated version header is written; no reference source is copied.
"""
import concurrent.futures as cf
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SRC = "/root/reference/src/cpu"
OUT = os.path.join(HERE, "_ref")
BIN = os.path.join(OUT, "parafrost")


def available() -> bool:
    return os.path.isdir(REF_SRC)


def build(force: bool = False) -> str:
    if not available():
        raise FileNotFoundError("reference sources are not present on this machine")
    srcs = sorted(glob.glob(os.path.join(REF_SRC, "*.cpp")))
    if not force and os.path.exists(BIN) and all(os.path.getmtime(s) <= os.path.getmtime(BIN) for s in srcs):
        return BIN
    gen = os.path.join(OUT, "gen")
    objd = os.path.join(OUT, "obj")
    os.makedirs(gen, exist_ok=True)
    os.makedirs(objd, exist_ok=True)
    with open(os.path.join(gen, "version.h"), "w") as f:
        # declarations the sources expect from their generated version header
        f.write('#pragma once\nnamespace ParaFROST {\n'
                'const char* version(); const char* signature(); const char* compiler();\n'
                'const char* compilemode(); const char* osystem(); const char* date();\n}\n'
                '#define VERSION "3.2.5"\n#define OSYSTEM "linux"\n#define DATE "oracle"\n'
                '#define COMPILER "g++"\n')
    flags = ["-std=c++20", "-O3", "-DNDEBUG", "-I", gen, "-I", REF_SRC, "-w"]

    def cc(src):
        obj = os.path.join(objd, os.path.basename(src).replace(".cpp", ".o"))
        subprocess.check_call(["g++", *flags, "-c", src, "-o", obj])
        return obj

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(cc, srcs))
    subprocess.check_call(["g++", "-O3", "-o", BIN, *objs, "-lpthread"])
    return BIN


if __name__ == "__main__":
    print(build(force=True))
