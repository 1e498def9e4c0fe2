"""Build librj.so (CUDA kernels + C++ runtime + C ABI) for sm_103a, in-tree.

Usage: python raster-join_gb300/build.py [--force]

The translation units compile in parallel with one -gencode
(compute_103a -> sm_103a) and link into raster-join_gb300/lib/librj.so with
the static CUDA runtime.  A stamp of the sources' modification times skips
work when nothing changed.
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "librj.so")
SOURCES = ["rj_runtime.cu", "rj_point_kernels.cu", "rj_point_exact.cu", "rj_poly_kernels.cu", "rj_noalloc.cu",
           "rj_batch.cu", "rj_batch_kernels.cu", "rj_batch_direct.cu", "rj_tier_kernels.cu",
           "rj_count_kernels.cu", "rj_lean_kernels.cu", "rj_hybrid_lean.cu", "rj_splat_kernels.cu",
           "rj_tier_lean.cu"]
HEADERS = ["rj_device.cuh", "rj_launch.h", "rj_internal.h", "rj_point_map.cuh", "rj_point_core.cuh",
           "rj_batch_common.cuh", "rj_lean.cuh",
           os.path.join("..", "..", "include", "rj.h")]

NVCC_FLAGS = [
    "-std=c++17", "-O3", "-lineinfo",
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
    "-Xcompiler", "-ffp-contract=off",
]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _stamp():
    h = hashlib.sha256()
    for f in SOURCES + HEADERS:
        p = os.path.join(CSRC, f)
        with open(p, "rb") as fh:
            h.update(fh.read())
    h.update(" ".join(NVCC_FLAGS).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


CPP = os.path.join(HERE, "cpp")
CLI = os.path.join(LIBDIR, "rj_cli")


def build_cli(force=False):
    """The command-line driver (cpp/rj_cli.cpp, host C++ only) against librj.so."""
    src = os.path.join(CPP, "rj_cli.cpp")
    hdrs = [os.path.join(CPP, "rasterjoin.hpp"), os.path.join(HERE, "..", "include", "rj.h")]
    newest = max(os.path.getmtime(f) for f in [src, LIB] + hdrs)
    if not force and os.path.exists(CLI) and os.path.getmtime(CLI) >= newest:
        return CLI
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(HERE, "..", "include"), src, "-o", CLI + ".tmp",
           "-L", LIBDIR, "-lrj", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("rj_cli build failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(CLI + ".tmp", CLI)
    return CLI


def build(force=False, verbose=False):
    """Compile and link librj.so (and the CLI); returns the library path."""
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    stamp_file = os.path.join(OBJ, "stamp")
    stamp = _stamp()
    if not force and os.path.exists(LIB) and os.path.exists(stamp_file):
        with open(stamp_file) as fh:
            if fh.read().strip() == stamp:
                build_cli()
                return LIB
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(OBJ, src.replace(".cu", ".o"))
        # per-object stamp: the source, every shared header, the flags, the machine
        h = hashlib.sha256()
        for f in [src] + HEADERS:
            with open(os.path.join(CSRC, f), "rb") as fh:
                h.update(fh.read())
        h.update(" ".join(NVCC_FLAGS).encode())
        h.update(os.uname().machine.encode())
        ostamp = obj + ".stamp"
        if not force and os.path.exists(obj) and os.path.exists(ostamp):
            with open(ostamp) as fh:
                if fh.read().strip() == h.hexdigest():
                    return obj
        cmd = [nvcc] + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        with open(ostamp, "w") as fh:
            fh.write(h.hexdigest())
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    with open(stamp_file, "w") as fh:
        fh.write(stamp)
    build_cli(force=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
