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


# The reference's compute and display shaders, translated to C++ and built
# beside the oracle to pin it (tests/test_reference_pin.py).  This recipe
# reads them where the reference's source tree lies: the tree given by the
# `reference` argument, else $SLIME_REFERENCE_ROOT, else the build machine's
# checkout below.  Built only where that tree is present; outputs go to
# oracle/_ref/ only.
REFERENCE_CHECKOUT = "/root/reference"


def reference_shaders(reference=None):
    root = reference or os.environ.get("SLIME_REFERENCE_ROOT") or REFERENCE_CHECKOUT
    return os.path.join(root, "src", "compute.wgsl"), os.path.join(root, "src", "display.wgsl")


REF_WGSL, REF_DISPLAY_WGSL = reference_shaders()
REF_DIR = os.path.join(HERE, "_ref")
REF_LIB = os.path.join(REF_DIR, "libwgslref.so")


def build_reference(force=False, reference=None):
    """Translate and build the reference's shaders from `reference` (a source
    tree), or from the default tree; None where it is absent."""
    REF_WGSL, REF_DISPLAY_WGSL = reference_shaders(reference)
    if not os.path.exists(REF_WGSL):
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    wgsl_dir = os.path.join(HERE, "wgsl")
    deps = [REF_WGSL, REF_DISPLAY_WGSL, os.path.join(wgsl_dir, "translate.py"), os.path.join(wgsl_dir, "prelude.h"),
            os.path.join(wgsl_dir, "harness.cpp"), os.path.join(HERE, "..", "include", "slime_math.h"),
            os.path.abspath(__file__)]
    if not force and os.path.exists(REF_LIB) and os.path.getmtime(REF_LIB) >= max(os.path.getmtime(d) for d in deps):
        return REF_LIB
    for src, inc in ((REF_WGSL, "compute_wgsl.inc"), (REF_DISPLAY_WGSL, "display_wgsl.inc")):
        r = subprocess.run([sys.executable, os.path.join(wgsl_dir, "translate.py"), src, os.path.join(REF_DIR, inc)],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"translating {src} failed:\n{r.stdout}\n{r.stderr}")
    tmp = REF_LIB + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fwrapv", "-fPIC", "-shared",
           os.path.join(wgsl_dir, "harness.cpp"), "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building the translated reference failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, REF_LIB)
    return REF_LIB


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    print(build(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv, reference=args[0] if args else None))
