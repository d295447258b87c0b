"""Build the CPU oracle (test infrastructure) as oracle/liboracle.so.

g++ -O3 with -ffp-contract=off (the restatement must not fuse a*b+c) and
OpenMP (the oracle's results do not depend on the thread count).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "slime_oracle.cpp")
LIB = os.path.join(HERE, "liboracle.so")


def build(force=False):
    deps = [SRC, os.path.join(HERE, "..", "include", "slime_math.h"), os.path.join(HERE, "..", "include", "slime.h")]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", SRC, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building the oracle failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
