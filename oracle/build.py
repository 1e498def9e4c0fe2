"""Build the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.

gcc, OpenMP, -ffp-contract=off so that every fp32 operation is rounded on its
own (the kernels use explicitly rounded intrinsics for the same expressions).
"""
import hashlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liboracle.so")
SRC = os.path.join(HERE, "oracle.c")
FLAGS = ["-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
         "-Wall", "-Wno-unused-function"]


def build(force=False):
    os.makedirs(OUT, exist_ok=True)
    with open(SRC, "rb") as fh:
        stamp = hashlib.sha256(fh.read() + " ".join(FLAGS).encode() + os.uname().machine.encode()).hexdigest()
    sf = os.path.join(OUT, "stamp")
    if not force and os.path.exists(LIB) and os.path.exists(sf) and open(sf).read().strip() == stamp:
        return LIB
    cmd = ["gcc"] + FLAGS + [SRC, "-o", LIB + ".tmp", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    os.replace(LIB + ".tmp", LIB)
    with open(sf, "w") as fh:
        fh.write(stamp)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
