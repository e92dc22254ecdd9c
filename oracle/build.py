"""Build recipe for the CPU oracle (test infrastructure only): compiles
oracle.c and oracle_par.c into oracle/_build/liboracle.so. The reference is a
Rust crate and there is no Rust toolchain here or on the GPU hosts, so no
oracle/_ref build exists."""

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = [os.path.join(HERE, s) for s in ("oracle.c", "oracle_par.c")]
DEPS = SOURCES + [os.path.join(HERE, "oracle.h")]


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in DEPS):
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["gcc", "-O3", "-std=gnu11", "-shared", "-fPIC", "-pthread", "-o", tmp] + SOURCES + ["-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
