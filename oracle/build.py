"""Build recipe for the CPU oracle (test infrastructure only): compiles
oracle.c, oracle_par.c and inflate.c into oracle/_build/liboracle.so. The reference is a
Rust crate and there is no Rust toolchain here or on the GPU hosts, so no
oracle/_ref build exists."""

import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
# The synthetic-input generator is compiled in as well (the same C source the
# package uses), so the CPU reference arm loads no product library.
GEN_SRC = os.path.join(os.path.dirname(HERE), "falx_gb300", "csrc", "gen.c")
SOURCES = [os.path.join(HERE, s) for s in ("oracle.c", "oracle_par.c", "inflate.c")] + [GEN_SRC]
DEPS = SOURCES + [os.path.join(HERE, "oracle.h"), os.path.abspath(__file__)]


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in DEPS):
        return LIB
    tmp = LIB + ".tmp"
    # aarch64: the NEON + PMULL tier of the reference's kernels (explicit
    # architecture extension, not the build host's own -march=native)
    arch = ["-march=armv8-a+crypto"] if platform.machine() == "aarch64" else []
    cmd = ["gcc", "-O3", "-std=gnu11", "-shared", "-fPIC", "-pthread"] + arch + ["-o", tmp] + SOURCES + ["-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
