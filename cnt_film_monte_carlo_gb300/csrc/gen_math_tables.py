"""Generate kmc_math_tables.h: constants of the engine's FP64 log and acos.

The hop kernels draw dwell times -log(u)/Gamma (the reference's scatterer::ff_time,
src/monte_carlo/scatterer.h:74-80) and the neighbour build needs the pair angle
acos(a1 . a2) (scatterer.cpp:51).  The engine evaluates both with functions of its own so
that every build (CUDA device code, host code) produces the same bits:

* log: P. T. P. Tang's table-driven method (ACM TOMS 16(4), 1990).  x = 2^k z with
  z in [a, 2a), a ~ 0.7012, split into 1024 intervals of equal width in the bit
  pattern; interval i has c_i = 1/midpoint (c = 1 exactly on the interval holding 1.0)
  and -log(c_i) as hi (a multiple of 2^-42, so k ln2_hi + hi is exact) + lo;
  log x = (k ln2_hi + hi) + (r + ((k ln2_lo + lo) + r^2 P(r))), r = fma(z, c_i, -1),
  P(r) = -1/2 + r/3 - r^2/4 + r^3/5 (Taylor series of log1p; |r| <= 2^-11).
* acos: pi/2 - asin(c) for |c| <= 1/2, 2 asin(sqrt((1-c)/2)) above and
  pi - 2 asin(sqrt((1+c)/2)) below, asin(x) = x + x z Q(z), z = x^2, Q from the Taylor
  series (2n)!/(4^n (n!)^2 (2n+1)), 24 terms.

Values are mpmath results at 200 bits rounded once to double.
Run: python cnt_film_monte_carlo_gb300/csrc/gen_math_tables.py
"""
import os
import struct

import mpmath

mpmath.mp.prec = 200

BITS = 10
N = 1 << BITS
ONE = 0x3FF0000000000000
STEP = 1 << (52 - BITS)
CENTER = 76 * 8 + 4  # the interval that holds 1.0 in its middle
OFF = ONE - STEP // 2 - CENTER * STEP
N_ASIN = 24


def bits_to_double(b):
    return struct.unpack("<d", struct.pack("<Q", b))[0]


def nearest(x):
    return float(mpmath.mpf(x))


def to_grid(x, e):
    """Nearest multiple of 2**e."""
    s = mpmath.mpf(2) ** e
    return float(mpmath.nint(mpmath.mpf(x) / s) * s)


def main():
    ln2 = mpmath.log(2)
    ln2_hi = to_grid(ln2, -42)
    rows = []
    for i in range(N):
        a = mpmath.mpf(bits_to_double(OFF + i * STEP))
        b = mpmath.mpf(bits_to_double(OFF + (i + 1) * STEP))
        c = 1.0 if i == CENTER else nearest(2 / (a + b))
        neg_log_c = -mpmath.log(mpmath.mpf(c))
        hi = to_grid(neg_log_c, -42)
        rows.append((c, hi, nearest(neg_log_c - mpmath.mpf(hi))))
    consts = {
        "KMC_LN2_HI": ln2_hi,
        "KMC_LN2_LO": nearest(ln2 - mpmath.mpf(ln2_hi)),
        "KMC_PIO2_HI": nearest(mpmath.pi / 2),
        "KMC_PIO2_LO": nearest(mpmath.pi / 2 - mpmath.mpf(nearest(mpmath.pi / 2))),
        "KMC_PI_HI": nearest(mpmath.pi),
        "KMC_PI_LO": nearest(mpmath.pi - mpmath.mpf(nearest(mpmath.pi))),
    }
    log1p = [nearest(mpmath.mpf((-1) ** (j + 1)) / j) for j in range(2, 6)]
    asin = [
        nearest(mpmath.factorial(2 * n) / (mpmath.mpf(4) ** n * mpmath.factorial(n) ** 2 * (2 * n + 1)))
        for n in range(1, N_ASIN + 1)
    ]
    lines = [
        "/* kmc_math_tables.h -- generated by gen_math_tables.py; do not edit.",
        " * Constants of the engine's FP64 log (Tang's table-driven method) and acos (asin Taylor",
        " * series).  Initialiser macros, so host and device code can each instantiate them. */",
        "#pragma once",
        f"#define KMC_LOG_TABLE_BITS {BITS}",
        f"#define KMC_LOG_OFF 0x{OFF:016X}ULL",
    ]
    for k, v in consts.items():
        lines.append(f"#define {k} ({v.hex()})")
    lines.append("#define KMC_LOG1P_INIT {" + ", ".join(c.hex() for c in log1p) + "}")
    lines.append("#define KMC_ASIN_INIT {" + ", ".join(c.hex() for c in asin) + "}")
    lines.append(f"#define KMC_ASIN_TERMS {N_ASIN}")
    lines.append("#define KMC_LOG_TAB_INIT { \\")
    for c, hi, lo in rows:
        lines.append(f"  {{{c.hex()}, {hi.hex()}, {lo.hex()}}}, \\")
    lines.append("}")
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kmc_math_tables.h")
    with open(out, "w") as f:
        f.write("\n".join(lines) + "\n")
    print("wrote", out)


if __name__ == "__main__":
    main()
