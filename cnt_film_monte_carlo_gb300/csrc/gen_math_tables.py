"""Generate kmc_math_tables.h: constants of the engine's log and acos.

The hop kernels draw dwell times -log(u)/Gamma (the reference's scatterer::ff_time,
src/monte_carlo/scatterer.h:74-80) and the neighbour build needs the pair angle
acos(a1 . a2) (scatterer.cpp:51).  The engine evaluates both with functions of its own so
that every build (CUDA device code, host code) produces the same bits:

* log, fixed point (after the table-driven method of P. T. P. Tang, "Table-driven
  implementation of the logarithm function in IEEE floating-point arithmetic", ACM TOMS 16(4),
  1990): x = 2^k z with z in [a, 2a), a ~ 0.7012, z in one of 1024 intervals of equal width in
  the bit pattern (the interval holding 1.0 has it in its middle).  Interval i has a 21-bit
  integer reciprocal C_i = round(2^20 / midpoint) (C = 2^20 on the interval holding 1.0), so
  r = z C_i 2^-20 - 1 = R 2^(ez - 72) exactly, with ez the exponent of z (-1 or 0), |r| < 2^-11
  and |R| < 2^62: R is the low 64 bits of the product Z C_i of the 53-bit significand and C_i.
  log1p(r) = r S(r), S = 1 - r/2 + r^2/3 - r^3/4 + r^4/5 - r^5/6, evaluated from the inside
  with r^3 .. r^5 in Q1.30 (32-bit) and the outer terms in Q1.62 (64-bit high products of
  r 2^64); log x = k ln2 - log(C_i 2^-20) + r S is summed in a signed 128-bit integer with 116
  fraction bits (ln2 rounded to 2^-116, -log(C_i 2^-20) to 2^-95) and rounded once to double
  (nearest, ties to even).  Error below 0.501 ulp.
* acos: pi/2 - asin(c) for |c| <= 1/2, 2 asin(sqrt((1-c)/2)) above and
  pi - 2 asin(sqrt((1+c)/2)) below, asin(x) = x + x z Q(z), z = x^2, Q from the Taylor
  series (2n)!/(4^n (n!)^2 (2n+1)), 24 terms.

Values are mpmath results at 200 bits, rounded once.
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


def main():
    ln2 = mpmath.log(2)
    consts = {
        "KMC_PIO2_HI": nearest(mpmath.pi / 2),
        "KMC_PIO2_LO": nearest(mpmath.pi / 2 - mpmath.mpf(nearest(mpmath.pi / 2))),
        "KMC_PI_HI": nearest(mpmath.pi),
        "KMC_PI_LO": nearest(mpmath.pi - mpmath.mpf(nearest(mpmath.pi))),
    }
    asin = [
        nearest(mpmath.factorial(2 * n) / (mpmath.mpf(4) ** n * mpmath.factorial(n) ** 2 * (2 * n + 1)))
        for n in range(1, N_ASIN + 1)
    ]
    lines = [
        "/* kmc_math_tables.h -- generated by gen_math_tables.py; do not edit.",
        " * Constants of the engine's fixed-point log and of acos (asin Taylor series).",
        " * Initialiser macros, so host and device code can each instantiate them. */",
        "#pragma once",
        f"#define KMC_LOG_TABLE_BITS {BITS}",
        f"#define KMC_LOG_OFF 0x{OFF:016X}ULL",
    ]
    for k, v in consts.items():
        lines.append(f"#define {k} ({v.hex()})")
    lines.append("#define KMC_ASIN_INIT {" + ", ".join(c.hex() for c in asin) + "}")
    lines.append(f"#define KMC_ASIN_TERMS {N_ASIN}")
    Q = 116
    ln2q = int(mpmath.nint(ln2 * mpmath.mpf(2) ** Q))
    lines.append(f"#define KMC_FX_LN2_HI 0x{ln2q >> 64:016X}ULL")
    lines.append(f"#define KMC_FX_LN2_LO 0x{ln2q & ((1 << 64) - 1):016X}ULL")
    two = mpmath.mpf(2)
    s62 = [int(mpmath.nint(v * two ** 62)) for v in (mpmath.mpf(1), mpmath.mpf(-1) / 2, mpmath.mpf(1) / 3)]
    s30 = [int(mpmath.nint(v * two ** 30)) for v in (mpmath.mpf(-1) / 4, mpmath.mpf(1) / 5, mpmath.mpf(-1) / 6)]
    lines.append("/* S(r) = 1 - r/2 + r^2/3 - r^3/4 + r^4/5 - r^5/6: S62 = 1, -1/2, 1/3 in Q1.62; S30 = -1/4, 1/5, -1/6 in Q1.30 */")
    for j, v in enumerate(s62):
        lines.append(f"#define KMC_FX_S62_{j} ({v}LL)")
    for j, v in enumerate(s30):
        lines.append(f"#define KMC_FX_S30_{j + 3} ({v}LL)")
    lines.append("/* per interval: {hi, lo | C_i} with -log(C_i 2^-20) in Q116 (two's complement, a multiple of 2^21,")
    lines.append(" * so its low 21 bits carry the 21-bit reciprocal C_i) */")
    lines.append("#define KMC_FX_TAB_INIT { \\")
    for i in range(N):
        a = mpmath.mpf(bits_to_double(OFF + i * STEP))
        b = mpmath.mpf(bits_to_double(OFF + (i + 1) * STEP))
        C = 1 << 20 if i == CENTER else int(mpmath.nint(two ** 21 / (a + b)))
        assert 0 < C < (1 << 21)
        lc = (int(mpmath.nint(-mpmath.log(mpmath.mpf(C) / two ** 20) * two ** 95)) << 21) & ((1 << 128) - 1)
        lines.append(f"  {{0x{lc >> 64:016X}ull, 0x{(lc & ((1 << 64) - 1)) | C:016X}ull}}, \\")
    lines.append("}")
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kmc_math_tables.h")
    with open(out, "w") as f:
        f.write("\n".join(lines) + "\n")
    print("wrote", out)


if __name__ == "__main__":
    main()
