"""In-tree build of the native parts: the CUDA engine (sm_103a) and the
synthetic-input generator. Objects land next to the sources' package and are
git-ignored; they are rebuilt when a source is newer than the library."""

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
GPU_LIB = os.path.join(PKG, "libfalx_gpu.so")
GEN_LIB = os.path.join(PKG, "libfalx_gen.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
GPU_SOURCES = ["falx_gpu.cu", "batch.cu", "batch_nb2.cu", "batch_nb3.cu", "inflate.cu"]
GPU_DEPS = ["scan_core.cuh", "rows.cuh", "decimal.cuh", "swar.cuh", "pow5_table.h", "ndjson.cuh", "mlp.cuh", "tile.cuh",
            "context.h", "batch_kernel.cuh", "columns.cuh", "index_pass.cuh", "inflate_core.h"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def build_gpu(force=False, verbose=False):
    """Compile every translation unit (in parallel) and link the engine."""
    srcs = [os.path.join(CSRC, s) for s in GPU_SOURCES]
    deps = srcs + [os.path.join(CSRC, d) for d in GPU_DEPS] + [os.path.join(ROOT, "include", "falx_gpu.h")]
    if not force and not _stale(GPU_LIB, deps):
        return GPU_LIB
    objdir = os.path.join(PKG, "_build")
    os.makedirs(objdir, exist_ok=True)

    def compile_one(src):
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        cmd = [_nvcc()] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = _run(cmd)
        if verbose:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = GPU_LIB + ".tmp"
    _run([_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs)
    os.replace(tmp, GPU_LIB)
    return GPU_LIB


def build_gen(force=False):
    src = os.path.join(CSRC, "gen.c")
    if not force and not _stale(GEN_LIB, [src]):
        return GEN_LIB
    tmp = GEN_LIB + ".tmp"
    _run(["gcc", "-O2", "-std=c11", "-shared", "-fPIC", "-pthread", "-o", tmp, src])
    os.replace(tmp, GEN_LIB)
    return GEN_LIB


def build_all(force=False):
    """Build every native library (the engine and the generator); the engine
    build is the long pole, so the host libraries build beside it."""
    with ThreadPoolExecutor(2) as ex:
        fg = ex.submit(build_gpu, force)
        fh = ex.submit(build_gen, force)
        return fg.result(), fh.result()


if __name__ == "__main__":
    import sys

    print(build_all(force="--force" in sys.argv))
