"""Build recipe for the oracle (test infrastructure only).

Compiles the C restatement `pfo.c` into `oracle/libpfo.so` with the host C
compiler. Nothing in the engine links this library.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libpfo.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "pfo.c")
    deps = [src, os.path.join(HERE, "pfo.h"), os.path.join(HERE, "..", "include", "pfgpu.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["gcc", "-O2", "-std=c99", "-Wall", "-fPIC", "-shared", src, "-o", LIB + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
