/* kmc_math.h -- TEST INFRASTRUCTURE (oracle): counter-based RNG and FP64 math of the oracle.
 *
 * Only the tests, the smoke check and the CPU-baseline leg of the benchmark use the oracle;
 * the product never includes this file.
 *
 * 1. Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as
 *    1, 2, 3", SC'11).  It stands in for the reference's global std::rand()
 *    (src/monte_carlo/scatterer.h:76, scatterer.cpp:17, particle.h:51,
 *    monte_carlo.cpp:311,331).  Each exciton owns one stream; draw n of stream s under
 *    seed S is word (n mod 4) of Philox(counter = {n/4 lo, n/4 hi, s lo, s hi},
 *    key = {S lo, S hi}), shifted right by one bit, so a draw lies in [0, 2^31 - 1],
 *    the range of glibc rand() (RAND_MAX = 2^31 - 1).
 * 2. orc_log / orc_acos: the project's log and acos, which replace std::log and std::acos on
 *    every side of the parity comparison.  Method and constants: oracle/gen_math_tables.py.
 *    log is integer (fixed-point) arithmetic with one final rounding; acos is IEEE operations
 *    written out (fma() where fused); both give the same value on any machine built with
 *    -ffp-contract=off.
 */
#ifndef ORC_KMC_MATH_H
#define ORC_KMC_MATH_H

#include <math.h>
#include <stdint.h>
#include <string.h>

#include "kmc_math_tables.h"

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_RAND_MAX 2147483647

static inline void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int round = 0; round < 10; ++round) {
    if (round > 0) {
      k0 += 0x9E3779B9u; /* Weyl key schedule (golden ratio) */
      k1 += 0xBB67AE85u; /* sqrt(3) - 1 */
    }
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

/* One exciton's stream: (seed, stream id) plus a draw counter and a one-block cache. */
typedef struct {
  uint64_t seed;
  uint64_t stream;
  uint64_t n;      /* draws taken so far */
  uint64_t block;  /* Philox block held in buf (UINT64_MAX: none) */
  uint32_t buf[4];
} orc_rng;

static inline void orc_rng_init(orc_rng* g, uint64_t seed, uint64_t stream, uint64_t n) {
  g->seed = seed;
  g->stream = stream;
  g->n = n;
  g->block = UINT64_MAX;
}

/* The reference's rand(): an int in [0, RAND_MAX]. */
static inline int orc_rand(orc_rng* g) {
  uint64_t b = g->n >> 2;
  if (b != g->block) {
    uint32_t ctr[4] = {(uint32_t)b, (uint32_t)(b >> 32), (uint32_t)g->stream, (uint32_t)(g->stream >> 32)};
    uint32_t key[2] = {(uint32_t)g->seed, (uint32_t)(g->seed >> 32)};
    orc_philox4x32_10(ctr, key, g->buf);
    g->block = b;
  }
  uint32_t w = g->buf[g->n & 3];
  g->n++;
  return (int)(w >> 1);
}

static inline uint64_t orc_d2b(double x) {
  uint64_t b;
  memcpy(&b, &x, 8);
  return b;
}
static inline double orc_b2d(uint64_t b) {
  double x;
  memcpy(&x, &b, 8);
  return x;
}

typedef __int128 orc_i128;
typedef unsigned __int128 orc_u128;

static inline int orc_bitlen128(orc_u128 m) {
  uint64_t hi = (uint64_t)(m >> 64), lo = (uint64_t)m;
  if (hi) return 128 - __builtin_clzll(hi);
  return lo ? 64 - __builtin_clzll(lo) : 0;
}

/* T * 2^-116 rounded to the nearest double (ties to even); T != 0, |T| < 2^127. */
static inline double orc_q116_to_double(orc_i128 T) {
  uint64_t sign = 0;
  orc_u128 m;
  if (T < 0) {
    sign = 1ULL << 63;
    m = (orc_u128)(-T);
  } else {
    m = (orc_u128)T;
  }
  int L = orc_bitlen128(m);
  uint64_t mant;
  int e2;
  if (L <= 53) {
    mant = (uint64_t)m << (53 - L);
    e2 = L - 53 - 116;
  } else {
    int sh = L - 53;
    orc_u128 keep = m >> sh;
    orc_u128 rem = m & ((((orc_u128)1) << sh) - 1);
    orc_u128 half = ((orc_u128)1) << (sh - 1);
    mant = (uint64_t)keep;
    if (rem > half || (rem == half && (mant & 1))) {
      mant++;
      if (mant == (1ULL << 53)) {
        mant >>= 1;
        sh++;
      }
    }
    e2 = sh - 116;
  }
  return orc_b2d(sign | ((uint64_t)(e2 + 52 + 1023) << 52) | (mant & ((1ULL << 52) - 1)));
}

/* Natural logarithm, fixed-point table method (constants and method: oracle/gen_math_tables.py).
 * Every step is integer arithmetic except the final rounding, so the value is the same on any
 * machine; error below 0.52 ulp. */
static inline double orc_log(double x) {
  uint64_t ix = orc_d2b(x);
  if (!(x > 0.0)) {
    if (x == 0.0) return -INFINITY;
    return NAN; /* negative or NaN */
  }
  if (ix >= 0x7FF0000000000000ULL) return x; /* +inf */
  int kadj = 0;
  if (ix < 0x0010000000000000ULL) { /* subnormal: scale into the normal range */
    x = x * 0x1p52;
    ix = orc_d2b(x);
    kadj = -52;
  }
  uint64_t tmp = ix - ORC_LOG_OFF;
  int i = (int)((tmp >> (52 - ORC_LOG_TABLE_BITS)) & ((1u << ORC_LOG_TABLE_BITS) - 1));
  int k = (int)((int64_t)tmp >> 52) + kadj;
  uint64_t iz = ix - (tmp & 0xFFF0000000000000ULL);
  int ez = (int)(iz >> 52) - 1023; /* -1 or 0 */
  uint64_t Z = (iz & ((1ULL << 52) - 1)) | (1ULL << 52);
  uint64_t C = ORC_FX_TAB[i][1] & ((1ULL << 21) - 1);
  /* r = z c - 1 = R 2^(ez - 72) exactly; |R| < 2^62, so R is the low word of Z C */
  int64_t R = (int64_t)(Z * C);
  int64_t rq = R >> (8 - ez);            /* r 2^64 */
  int32_t r30 = (int32_t)(rq >> 34);     /* r 2^30 */
  int32_t t4 = ORC_FX_S30[1] + (int32_t)(((int64_t)r30 * ORC_FX_S30[2]) >> 30);
  int32_t t3 = ORC_FX_S30[0] + (int32_t)(((int64_t)r30 * t4) >> 30);
  int64_t t2 = ORC_FX_S62[2] + (int64_t)(((orc_i128)rq * (orc_i128)((int64_t)t3 * 4294967296LL)) >> 64);
  int64_t t1 = ORC_FX_S62[1] + (int64_t)(((orc_i128)rq * t2) >> 64);
  int64_t S = ORC_FX_S62[0] + (int64_t)(((orc_i128)rq * t1) >> 64);
  orc_i128 L1 = ((orc_i128)R * S) >> (18 - ez); /* r S in Q116 */
  orc_i128 ln2 = (orc_i128)((((orc_u128)ORC_FX_LN2_HI) << 64) | ORC_FX_LN2_LO);
  orc_i128 lc = (orc_i128)((((orc_u128)ORC_FX_TAB[i][0]) << 64) | (ORC_FX_TAB[i][1] & ~((1ULL << 21) - 1)));
  orc_i128 T = (orc_i128)k * ln2 + lc + L1;
  if (T == 0) return 0.0;
  return orc_q116_to_double(T);
}

/* asin on |x| <= 1/2 by its Taylor series. */
static inline double orc_asin_small(double x) {
  double z = x * x;
  double p = ORC_ASIN_C[23];
  for (int j = 22; j >= 0; --j) p = fma(p, z, ORC_ASIN_C[j]);
  double t = x * z;
  return fma(t, p, x);
}

/* Inverse cosine on [-1, 1]; NaN outside. */
static inline double orc_acos(double c) {
  if (c != c) return c;
  if (c > 1.0 || c < -1.0) return NAN;
  if (c <= 0.5 && c >= -0.5) return ORC_PIO2_HI - (orc_asin_small(c) - ORC_PIO2_LO);
  if (c > 0.5) {
    double x = sqrt((1.0 - c) * 0.5);
    return 2.0 * orc_asin_small(x);
  }
  double x = sqrt((1.0 + c) * 0.5);
  return ORC_PI_HI - (2.0 * orc_asin_small(x) - ORC_PI_LO);
}

#ifdef __cplusplus
}
#endif

#endif /* ORC_KMC_MATH_H */
