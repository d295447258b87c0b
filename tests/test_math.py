"""The shared binary32 builtins (include/slime_math.h) through the oracle
library: the generated constants, sin/cos accuracy against mpmath, and the
equality of the two Payne-Hanek window forms the reduction dispatches to."""
import os
import re
import sys

import numpy as np
import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_constants_match_generator():
    pytest.importorskip("mpmath")
    sys.path.insert(0, os.path.join(ROOT, "include"))
    import gen_slime_math_constants as gen
    with open(os.path.join(ROOT, "include", "slime_math.h")) as f:
        header = f.read()
    m = re.search(r"/\* BEGIN GENERATED CONSTANTS.*?END GENERATED CONSTANTS \*/", header, re.S)
    assert m is not None
    assert m.group(0) == gen.c_block()


def test_payne_hanek_window_equals_table_exhaustively():
    # every binary32 with 4096 <= |x| < 2^44, both signs (2^29 inputs)
    assert oracle.ph_window_mismatches(139, 170) == 0


def test_payne_hanek_tail_in_32_bit_words_equals_64_bit_statement_exhaustively():
    # every finite binary32 with |x| >= 4096, both signs (1.9e9 inputs)
    assert oracle.ph_finish_mismatches(139, 254) == 0


def _ulp_errors(x):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 200
    s, c = oracle.sincos(x)
    worst = 0.0
    for xi, si, ci in zip(x.tolist(), s.tolist(), c.tolist()):
        xm = mpmath.mpf(xi)
        for got, ref in ((si, mpmath.sin(xm)), (ci, mpmath.cos(xm))):
            ref_f = float(ref)
            ulp = np.spacing(np.float32(abs(ref_f)))
            worst = max(worst, abs(float(mpmath.mpf(got) - ref)) / float(ulp))
    return worst


@pytest.mark.parametrize("lo,hi", [(0.0, 4.0), (4.0, 4096.0), (4096.0, 2.0 ** 28), (2.0 ** 28, 3.0e38)])
def test_sincos_accuracy_against_mpmath(lo, hi):
    rng = np.random.default_rng(int(lo) % 1000 + 7)
    # log-uniform magnitudes, both signs
    mag = np.exp(rng.uniform(np.log(max(lo, 1e-6)), np.log(hi), 3000))
    x = (mag * rng.choice([-1.0, 1.0], mag.size)).astype(np.float32)
    assert _ulp_errors(x) <= 1.5
