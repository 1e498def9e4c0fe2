"""Build oracle/_ref/libreftri.so: the reference's triangulation sources
(RasterJoin/triangulation/{clip2tri,clipper,poly2tri}) compiled where they lie
in the reference tree, with tri_wrap.cpp as the C entry point.  TEST
INFRASTRUCTURE ONLY (fill-rule cross-check).  Nothing is copied into this
repository; without the reference tree the build is skipped."""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(os.path.dirname(HERE), "_ref")
LIB = os.path.join(OUT_DIR, "libreftri.so")
# the reference tree: RJ_REFERENCE_DIR, else its usual mount point
REF = os.path.join(os.environ.get("RJ_REFERENCE_DIR", "/root/reference"), "RasterJoin", "triangulation")
SOURCES = ["clip2tri/clip2tri.cpp", "clipper/clipper.cpp", "poly2tri/common/shapes.cc",
           "poly2tri/sweep/advancing_front.cc", "poly2tri/sweep/cdt.cc", "poly2tri/sweep/sweep.cc",
           "poly2tri/sweep/sweep_context.cc"]


def build(optional=True):
    if not os.path.isdir(REF):
        if optional:
            return None
        raise RuntimeError("reference triangulation sources not found")
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = [os.path.join(REF, s) for s in SOURCES] + [os.path.join(HERE, "tri_wrap.cpp")]
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(s) for s in srcs):
        return LIB
    objs = []

    def cc(src):
        obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
        r = subprocess.run(["g++", "-std=c++11", "-O2", "-fPIC", "-w", "-I", REF, "-c", src, "-o", obj],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("g++ failed on %s:\n%s" % (src, r.stderr))
        return obj

    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        objs = list(ex.map(cc, srcs))
    r = subprocess.run(["g++", "-shared", "-o", LIB] + objs, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(optional="--required" not in sys.argv))
