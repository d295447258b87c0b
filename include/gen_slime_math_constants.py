"""Generate the constants of include/slime_math.h from first principles.

Every constant is computed here with mpmath at 400 bits and rounded to the
nearest binary32 value, so the header carries no number of unknown origin:

  * SLM_TWO_OVER_PI_WORDS: the binary expansion of 2/pi, 32 bits per word,
    preceded by one all-zero word (bits "before" the binary point), used by the
    Payne-Hanek reduction for large arguments.
  * SLM_PIO2_{1,2,3}: pi/2 split into three binary32 parts for the
    Cody-Waite reduction of small arguments.
  * SLM_S*, SLM_C*: Taylor coefficients (-1)^k / (2k+1)! and (-1)^k / (2k)!.
  * SLM_PH_WIN_INIT: bits 19..146 of the word stream above (bit 0 = the most
    significant bit of the zero word), the only bits of 2/pi the Payne-Hanek
    window reads for 4096 <= |x| < 2^44.

Run `python include/gen_slime_math_constants.py` to print the C block; the
CPU test suite re-runs it and compares against the header.
"""
import struct

import mpmath

mpmath.mp.prec = 400


def f32(v):
    """Round an mpmath number to the nearest binary32 (ties to even)."""
    # Go through exact rational arithmetic, never through a double.
    v = mpmath.mpf(v)
    if v == 0:
        return 0.0
    sign = -1 if v < 0 else 1
    a = abs(v)
    e = int(mpmath.floor(mpmath.log(a, 2)))
    # normalise: a = m * 2^(e-23) with 2^23 <= m < 2^24
    while a >= mpmath.mpf(2) ** (e + 1):
        e += 1
    while a < mpmath.mpf(2) ** e:
        e -= 1
    scaled = a * mpmath.mpf(2) ** (23 - e)
    m = int(mpmath.floor(scaled))
    rem = scaled - m
    if rem > 0.5 or (rem == 0.5 and (m & 1)):
        m += 1
    val = sign * m * (2.0 ** (e - 23))
    assert struct.unpack("<f", struct.pack("<f", val))[0] == val
    return val


def hexf(v):
    return float(v).hex() + "f"


def words_two_over_pi(n_words=9):
    v = 2 / mpmath.pi
    bits = int(mpmath.floor(v * mpmath.mpf(2) ** (32 * n_words)))
    return [0] + [(bits >> (32 * (n_words - 1 - i))) & 0xFFFFFFFF for i in range(n_words)]


def constants():
    pio2 = mpmath.pi / 2
    p1 = f32(pio2)
    p2 = f32(pio2 - p1)
    p3 = f32(pio2 - p1 - p2)
    out = {
        "SLM_TWO_OVER_PI_F": f32(2 / mpmath.pi),
        "SLM_PIO2_1": p1,
        "SLM_PIO2_2": p2,
        "SLM_PIO2_3": p3,
    }
    for k in range(1, 5):
        out[f"SLM_S{k}"] = f32(mpmath.mpf((-1) ** k) / mpmath.factorial(2 * k + 1))
    for k in range(1, 6):
        out[f"SLM_C{k}"] = f32(mpmath.mpf((-1) ** k) / mpmath.factorial(2 * k))
    return out


def c_block():
    lines = ["/* BEGIN GENERATED CONSTANTS (include/gen_slime_math_constants.py) */"]
    for k, v in constants().items():
        lines.append(f"#define {k} ({hexf(v)})")
    w = words_two_over_pi()
    lines.append("#define SLM_TWO_OVER_PI_NWORDS %d" % len(w))
    lines.append("#define SLM_TWO_OVER_PI_INIT { " + ", ".join("0x%08xu" % x for x in w) + " }")
    stream = 0
    for x in w:
        stream = (stream << 32) | x
    nbits = 32 * len(w)
    win = [(stream >> (nbits - (19 + 32 * i) - 32)) & 0xFFFFFFFF for i in range(4)]
    lines.append("#define SLM_PH_WIN_INIT { " + ", ".join("0x%08xu" % x for x in win) + " }")
    lines.append("/* END GENERATED CONSTANTS */")
    return "\n".join(lines)


if __name__ == "__main__":
    print(c_block())
