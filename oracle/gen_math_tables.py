"""Generate oracle/kmc_math_tables.h: constants for the oracle's log and acos.

TEST INFRASTRUCTURE (oracle). The oracle restates the reference's hot path on the
CPU; the reference calls glibc ``std::log`` (src/monte_carlo/scatterer.h:79) and
``std::acos`` (src/monte_carlo/scatterer.cpp:51).  For bit-exact comparison the
oracle, the shim-compiled reference (oracle/_ref) and the CUDA kernels all evaluate
one project-defined log and acos, written from the mathematics:

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
* acos: acos(c) = pi/2 - asin(c) for |c| <= 1/2, 2 asin(sqrt((1-c)/2)) above,
  pi - 2 asin(sqrt((1+c)/2)) below; asin by its Taylor series
  x + sum_n (2n)!/(4^n (n!)^2 (2n+1)) x^(2n+1), 24 terms (|x| <= 1/2).

All constants are computed here with mpmath at 200 bits and rounded once.
Run: python oracle/gen_math_tables.py  (rewrites oracle/kmc_math_tables.h)
"""
import os
import struct

import mpmath

mpmath.mp.prec = 200

LOG_TABLE_BITS = 10
LOG_N = 1 << LOG_TABLE_BITS
ONE_BITS = 0x3FF0000000000000
STEP = 1 << (52 - LOG_TABLE_BITS)
CENTER_INDEX = 76 * 8 + 4  # the interval that holds 1.0 in its middle
LOG_OFF = ONE_BITS - STEP // 2 - CENTER_INDEX * STEP  # bit pattern of a
ASIN_TERMS = 24


def b2d(b):
    return struct.unpack("<d", struct.pack("<Q", b))[0]


def rn(x):
    """Round an mpmath number to the nearest double."""
    return float(mpmath.mpf(x))


def main():
    ln2 = mpmath.log(2)
    pi = mpmath.pi
    pio2_hi = rn(pi / 2)
    pio2_lo = rn(pi / 2 - mpmath.mpf(pio2_hi))
    pi_hi = rn(pi)
    pi_lo = rn(pi - mpmath.mpf(pi_hi))
    asin_c = []
    for n in range(1, ASIN_TERMS + 1):
        a = mpmath.factorial(2 * n) / (mpmath.mpf(4) ** n * mpmath.factorial(n) ** 2 * (2 * n + 1))
        asin_c.append(rn(a))

    out = []
    out.append("/* Generated by oracle/gen_math_tables.py -- do not edit.")
    out.append(" * TEST INFRASTRUCTURE (oracle): constants of the oracle's log and acos.")
    out.append(" * Every value is an mpmath (200-bit) result rounded once to double. */")
    out.append("#ifndef ORC_MATH_TABLES_H")
    out.append("#define ORC_MATH_TABLES_H")
    out.append("#include <stdint.h>")
    out.append(f"#define ORC_LOG_TABLE_BITS {LOG_TABLE_BITS}")
    out.append(f"#define ORC_LOG_OFF 0x{LOG_OFF:016X}ULL")
    out.append(f"static const double ORC_PIO2_HI = {pio2_hi.hex()};")
    out.append(f"static const double ORC_PIO2_LO = {pio2_lo.hex()};")
    out.append(f"static const double ORC_PI_HI = {pi_hi.hex()};")
    out.append(f"static const double ORC_PI_LO = {pi_lo.hex()};")
    out.append(f"/* asin(x) = x + x z Q(z), z = x^2, Q(z) = a[0] + a[1] z + ... + a[{ASIN_TERMS - 1}] z^{ASIN_TERMS - 1} */")
    out.append(f"static const double ORC_ASIN_C[{ASIN_TERMS}] = {{")
    for c in asin_c:
        out.append(f"  {c.hex()},")
    out.append("};")
    # fixed-point log tables
    Q = 116
    ln2q = int(mpmath.nint(ln2 * mpmath.mpf(2) ** Q))
    out.append(f"#define ORC_FX_LN2_HI 0x{ln2q >> 64:016X}ULL")
    out.append(f"#define ORC_FX_LN2_LO 0x{ln2q & ((1 << 64) - 1):016X}ULL")
    two = mpmath.mpf(2)
    s62 = [int(mpmath.nint(v * two ** 62)) for v in (mpmath.mpf(1), mpmath.mpf(-1) / 2, mpmath.mpf(1) / 3)]
    s30 = [int(mpmath.nint(v * two ** 30)) for v in (mpmath.mpf(-1) / 4, mpmath.mpf(1) / 5, mpmath.mpf(-1) / 6)]
    out.append("/* S(r) = 1 - r/2 + r^2/3 - r^3/4 + r^4/5 - r^5/6: s62 = 1, -1/2, 1/3 in Q1.62; s30 = -1/4, 1/5, -1/6 in Q1.30 */")
    out.append("static const int64_t ORC_FX_S62[3] = {" + ", ".join(f"{v}LL" for v in s62) + "};")
    out.append("static const int32_t ORC_FX_S30[3] = {" + ", ".join(f"{v}LL" for v in s30) + "};")
    out.append(f"/* per interval i: {{hi, lo | C_i}} with -log(C_i 2^-20) in Q{Q} (two's complement, a multiple of")
    out.append(" * 2^21, so its low 21 bits carry the 21-bit reciprocal C_i) */")
    out.append(f"static const uint64_t ORC_FX_TAB[{LOG_N}][2] = {{")
    for i in range(LOG_N):
        lo_ = mpmath.mpf(b2d(LOG_OFF + i * STEP))
        hi_ = mpmath.mpf(b2d(LOG_OFF + (i + 1) * STEP))
        C = 1 << 20 if i == CENTER_INDEX else int(mpmath.nint(two ** 21 / (lo_ + hi_)))
        assert 0 < C < (1 << 21)
        lc = (int(mpmath.nint(-mpmath.log(mpmath.mpf(C) / two ** 20) * two ** 95)) << 21) & ((1 << 128) - 1)
        out.append(f"  {{0x{lc >> 64:016X}ULL, 0x{(lc & ((1 << 64) - 1)) | C:016X}ULL}},")
    out.append("};")
    out.append("#endif")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kmc_math_tables.h")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
    print("wrote", path)


if __name__ == "__main__":
    main()
