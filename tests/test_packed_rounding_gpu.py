"""Packed binary32x2 arithmetic rounds each lane as the scalar operation
does for the forms the agent kernels use (single mul2 / add2, chains of
fused multiply-adds).  tests/probes/packed_rounding.cu compares 16.8 M random
lanes per case with the scalar intrinsics; the sequences in which a packed
product feeds a packed sum are reported, not asserted (the kernels keep those
scalar)."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
NAMES = {0: "mul2", 1: "add2", 2: "fma2 chain", 3: "mul2 -> add2 (asm volatile)", 4: "mix (intrinsics)",
         5: "mix (asm volatile)", 6: "three products summed (intrinsics)"}


def test_packed_forms_used_by_the_kernels_round_per_lane(gpu, tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "packed_rounding"
    # the library's own arithmetic flags: no contraction of scalar products and sums
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-fmad=false", "-o", str(exe),
                    os.path.join(HERE, "probes", "packed_rounding.cu")], check=True, timeout=300)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=120).stdout
    counts = {}
    for line in out.splitlines():
        _, k, bad, lanes, fused = line.split()
        counts[int(k)] = (int(bad), int(lanes), int(fused))
    assert sorted(counts) == list(range(7))
    for k, (bad, lanes, fused) in sorted(counts.items()):
        print(f"{NAMES[k]:40s} {bad:9d} of {lanes} lanes differ" + (f", {fused} of them rounded once" if k == 3 else ""))
    for k in (0, 1, 2):
        assert counts[k][0] == 0, f"{NAMES[k]}: {counts[k][0]} lanes differ from the scalar rounding"
