"""Build libslime_gb300.so in-tree for sm_103a.

Each translation unit is compiled in parallel with nvcc (or g++ for plain C++)
into slime-mold_gb300/_build/, then linked into slime-mold_gb300/lib/.  Host
and device arithmetic is kept unfused (-ffp-contract=off, -fmad=false): the
kernels and the CPU oracle must agree bit for bit.

Usage: python slime-mold_gb300/build.py [--verbose-ptxas] [--force]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libslime_gb300.so")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _deps():
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    inc = os.path.join(HERE, "..", "include")
    paths += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return max(os.path.getmtime(p) for p in paths)


def compile_one(src, verbose_ptxas=False):
    obj = os.path.join(BUILD, src + ".o")
    path = os.path.join(CSRC, src)
    if src.endswith(".cu"):
        cmd = [nvcc_path(), *GENCODE, "-lineinfo", "-O3", "-std=c++17", "-fmad=false",
               "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-c", path, "-o", obj]
        if verbose_ptxas:
            cmd.insert(1, "-Xptxas=-v")
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling {src} failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force=False, verbose_ptxas=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    if not force and not verbose_ptxas and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps():
        return LIB
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: compile_one(s, verbose_ptxas), srcs))
    if verbose_ptxas:
        for _, log in results:
            if log.strip():
                print(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc_path(), "-shared", *GENCODE, "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"linking failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="--verbose-ptxas" in sys.argv))
