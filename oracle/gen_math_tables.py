"""Generate oracle/kmc_math_tables.h: constants for the oracle's FP64 log and acos.

TEST INFRASTRUCTURE (oracle). The oracle restates the reference's hot path on the
CPU; the reference calls glibc ``std::log`` (src/monte_carlo/scatterer.h:79) and
``std::acos`` (src/monte_carlo/scatterer.cpp:51).  For bit-exact comparison the
oracle, the shim-compiled reference (oracle/_ref) and the CUDA kernels all evaluate
one project-defined log and acos, written from the mathematics:

* log: table-driven method of P. T. P. Tang, "Table-driven implementation of the
  logarithm function in IEEE floating-point arithmetic", ACM TOMS 16(4), 1990.
  x = 2^k z with z in [a, 2a), a ~ 0.7012; z falls into one of 1024 intervals
  (equal width in the bit pattern), each with a reciprocal c_i of its midpoint, so that
  |r| = |z c_i - 1| <= 2^-11.  log x = k ln2 - log c_i + log1p(r), log1p by its Taylor
  series r - r^2/2 + r^3/3 - r^4/4 + r^5/5 (the first omitted term is below 2^-55 |r|).
  The interval holding 1.0 has c = 1 exactly, so the result keeps full relative
  accuracy near x = 1.
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


def round_to_multiple(x, ulp_exp):
    """Round x to the nearest multiple of 2**ulp_exp (returned as a double)."""
    q = mpmath.nint(mpmath.mpf(x) * mpmath.mpf(2) ** (-ulp_exp))
    return float(q * mpmath.mpf(2) ** ulp_exp)


def log_tables():
    invc, logc_hi, logc_lo = [], [], []
    for i in range(LOG_N):
        lo = mpmath.mpf(b2d(LOG_OFF + i * STEP))
        hi = mpmath.mpf(b2d(LOG_OFF + (i + 1) * STEP))
        if i == CENTER_INDEX:
            c = 1.0
        else:
            c = rn(2 / (lo + hi))
        lc = -mpmath.log(mpmath.mpf(c))  # log(x) = k ln2 + (-log c) + log1p(z c - 1)
        h = round_to_multiple(lc, -42)
        invc.append(c)
        logc_hi.append(h)
        logc_lo.append(rn(lc - mpmath.mpf(h)))
    assert invc[CENTER_INDEX] == 1.0 and logc_hi[CENTER_INDEX] == 0.0 and logc_lo[CENTER_INDEX] == 0.0
    return invc, logc_hi, logc_lo


def main():
    ln2 = mpmath.log(2)
    ln2_hi = round_to_multiple(ln2, -42)
    ln2_lo = rn(ln2 - mpmath.mpf(ln2_hi))
    pi = mpmath.pi
    pio2_hi = rn(pi / 2)
    pio2_lo = rn(pi / 2 - mpmath.mpf(pio2_hi))
    pi_hi = rn(pi)
    pi_lo = rn(pi - mpmath.mpf(pi_hi))
    asin_c = []
    for n in range(1, ASIN_TERMS + 1):
        a = mpmath.factorial(2 * n) / (mpmath.mpf(4) ** n * mpmath.factorial(n) ** 2 * (2 * n + 1))
        asin_c.append(rn(a))
    log1p_c = [rn(mpmath.mpf((-1) ** (j + 1)) / j) for j in range(2, 6)]  # -1/2, 1/3, -1/4, 1/5
    invc, lhi, llo = log_tables()

    out = []
    out.append("/* Generated by oracle/gen_math_tables.py -- do not edit.")
    out.append(" * TEST INFRASTRUCTURE (oracle): constants of the oracle's FP64 log and acos.")
    out.append(" * Every value is an mpmath (200-bit) result rounded once to double. */")
    out.append("#ifndef ORC_MATH_TABLES_H")
    out.append("#define ORC_MATH_TABLES_H")
    out.append("#include <stdint.h>")
    out.append(f"#define ORC_LOG_TABLE_BITS {LOG_TABLE_BITS}")
    out.append(f"#define ORC_LOG_OFF 0x{LOG_OFF:016X}ULL")
    out.append(f"static const double ORC_LN2_HI = {ln2_hi.hex()};")
    out.append(f"static const double ORC_LN2_LO = {ln2_lo.hex()};")
    out.append(f"static const double ORC_PIO2_HI = {pio2_hi.hex()};")
    out.append(f"static const double ORC_PIO2_LO = {pio2_lo.hex()};")
    out.append(f"static const double ORC_PI_HI = {pi_hi.hex()};")
    out.append(f"static const double ORC_PI_LO = {pi_lo.hex()};")
    out.append("/* log1p(r) = r + r^2 * P(r), P(r) = c[0] + c[1] r + c[2] r^2 + c[3] r^3 */")
    out.append("static const double ORC_LOG1P_C[4] = {" + ", ".join(c.hex() for c in log1p_c) + "};")
    out.append(f"/* asin(x) = x + x z Q(z), z = x^2, Q(z) = a[0] + a[1] z + ... + a[{ASIN_TERMS - 1}] z^{ASIN_TERMS - 1} */")
    out.append(f"static const double ORC_ASIN_C[{ASIN_TERMS}] = {{")
    for c in asin_c:
        out.append(f"  {c.hex()},")
    out.append("};")
    out.append("/* per interval i: {1/c_i, hi(-log c_i) (multiple of 2^-42), lo(-log c_i)} */")
    out.append(f"static const double ORC_LOG_TAB[{LOG_N}][3] = {{")
    for i in range(LOG_N):
        out.append(f"  {{{invc[i].hex()}, {lhi[i].hex()}, {llo[i].hex()}}},")
    out.append("};")
    out.append("#endif")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kmc_math_tables.h")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
    print("wrote", path)


if __name__ == "__main__":
    main()
