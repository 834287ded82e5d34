// kmc_device.cuh -- device arithmetic shared by the engine's kernels.
//
// Bit-exactness rules (the hop sequence must equal the FP64 reference step by step):
//  * the library is compiled with --fmad=false: no multiply-add is fused unless fma() is
//    written out, exactly as the CPU build uses -ffp-contract=off;
//  * 3-vector dot products and norms use the reference's vector-library order as the engine
//    defines it: two accumulators over even/odd elements starting at 0,
//    ((0 + a0 b0) + a2 b2) + (0 + a1 b1);
//  * log and acos are the engine's own (kmc_math_tables.h); double division and sqrt are IEEE.
#pragma once
#include <cstdint>

#include "kmc_math_tables.h"

namespace kmc {

constexpr uint32_t kRandMax = 2147483647u;  // glibc RAND_MAX, range of the reference's rand()
constexpr double kMinHopDist = 0.4e-9;      // scatterer.cpp:43

// ---------------------------------------------------------------- Philox-4x32-10 (Salmon et al., SC'11)
__host__ __device__ __forceinline__ void philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                       uint32_t k0, uint32_t k1, uint32_t out[4]) {
#pragma unroll
  for (int round = 0; round < 10; ++round) {
    if (round) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
#ifdef __CUDA_ARCH__
    uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
    uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
#else
    uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32), lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
#endif
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

// One exciton's stream: draw n of stream s under seed S is word (n mod 4) of
// Philox(counter = {n/4 lo, n/4 hi, s lo, s hi}, key = {S lo, S hi}) >> 1.
// The four words of the current block are kept in registers and rotated, so no dynamic
// register indexing occurs.
struct Rng {
  uint64_t seed, stream, n;
  uint32_t w0, w1, w2, w3;

  __host__ __device__ __forceinline__ void refill() {
    uint64_t b = n >> 2;
    uint32_t o[4];
    philox4x32_10((uint32_t)b, (uint32_t)(b >> 32), (uint32_t)stream, (uint32_t)(stream >> 32), (uint32_t)seed,
                  (uint32_t)(seed >> 32), o);
    uint32_t k = (uint32_t)(n & 3);
    // rotate so that w0 is word k
    w0 = o[0];
    w1 = o[1];
    w2 = o[2];
    w3 = o[3];
    for (uint32_t i = 0; i < k; ++i) {
      uint32_t t = w0;
      w0 = w1;
      w1 = w2;
      w2 = w3;
      w3 = t;
    }
  }
  __host__ __device__ __forceinline__ void init(uint64_t s_seed, uint64_t s_stream, uint64_t s_n) {
    seed = s_seed;
    stream = s_stream;
    n = s_n;
    refill();
  }
  __host__ __device__ __forceinline__ uint32_t next() {  // value in [0, 2^31 - 1]
    uint32_t v = w0 >> 1;
    ++n;
    if ((n & 3) == 0) {
      refill();
    } else {
      w0 = w1;
      w1 = w2;
      w2 = w3;
    }
    return v;
  }
};

// ---------------------------------------------------------------- u = RN(r / RAND_MAX) without division
// For 1 <= r < D = 2^31 - 1:  r 2^93 / D = N + r/D with N = r (2^62 + 2^31 + 1), because
// 2^93 = D (2^62 + 2^31 + 1) 2^0 ... precisely 2^31 = D + 1 and 2^62 = D (2^31 + 1) + 1.
// N >= 2^62 has 63..93 bits; keeping 53 of them drops d >= 10 bits.  The fraction r/D lies
// strictly in (0, 1) and decides only would-be ties, which therefore cannot occur: the
// result rounds up exactly when the highest dropped bit of N is set.  Exhaustively checked
// against IEEE division for every r on the device.
__device__ __forceinline__ double u_from_rand(uint32_t r) {
  if (r >= kRandMax) return 1.0;
  uint64_t rr = r;
  uint64_t s1 = (rr << 31) + rr;           // r 2^31 + r < 2^62 + 2^31
  uint64_t c = (rr & 3ull) << 62;          // low word of r 2^62
  uint64_t lo = c + s1;
  uint64_t hi = (rr >> 2) + (lo < c ? 1ull : 0ull);
  int L = hi ? 128 - __clzll((long long)hi) : 64 - __clzll((long long)lo);  // bit length of N (>= 63)
  int d = L - 53;                                                              // 10 <= d <= 40
  uint64_t keep = (hi << (64 - d)) | (lo >> d);
  uint64_t up = (lo >> (d - 1)) & 1ull;
  uint64_t mant = keep + up;  // in [2^52, 2^53]
  int e = d - 93;             // value = mant 2^e
  if (mant == (1ull << 53)) {
    mant >>= 1;
    e += 1;
  }
  uint64_t bits = ((uint64_t)(1023 + 52 + e) << 52) | (mant & ((1ull << 52) - 1));
  return __longlong_as_double((long long)bits);
}

// ---------------------------------------------------------------- log (fixed point, integer pipes)
// x = 2^k z (z in [a, 2a), one of 1024 intervals); c = C 2^-20 with a 21-bit reciprocal C, so
// r = z c - 1 = R 2^(ez - 72) is exact and |R| < 2^62 (R is the low word of Z C);
// log1p(r) = r S(r) with S evaluated in Q1.30 (inner terms) and Q1.62 integers;
// k ln2 - log c + r S is summed in a signed 128-bit Q116 integer and rounded once to double
// (nearest, ties to even).  No floating-point instruction is used: the FP64 pipe of sm_103a is
// the scarce resource of the hop kernels.  Error < 0.501 ulp.
struct LogTab {
  uint64_t t[1 << KMC_LOG_TABLE_BITS][2];  // hi, lo | C of -log(C 2^-20) in Q116 (low 21 bits: C)
};

struct I128 {
  uint64_t lo;
  int64_t hi;
};

__device__ __forceinline__ I128 add128(I128 a, I128 b) {
  I128 r;
  r.lo = a.lo + b.lo;
  r.hi = a.hi + b.hi + (r.lo < a.lo ? 1 : 0);
  return r;
}
// arithmetic shift right by 1 <= s <= 63
__device__ __forceinline__ I128 sar128(I128 a, int s) {
  I128 r;
  r.lo = (a.lo >> s) | ((uint64_t)a.hi << (64 - s));
  r.hi = a.hi >> s;
  return r;
}
__device__ __forceinline__ I128 neg128(I128 a) {
  I128 r;
  r.lo = ~a.lo + 1;
  r.hi = ~a.hi + (r.lo == 0 ? 1 : 0);
  return r;
}
__device__ __forceinline__ I128 mul64s(int64_t a, int64_t b) {
  I128 r;
  r.lo = (uint64_t)a * (uint64_t)b;
  r.hi = __mul64hi((long long)a, (long long)b);
  return r;
}
__device__ __forceinline__ int bitlen128(uint64_t hi, uint64_t lo) {
  return hi ? 128 - __clzll((long long)hi) : (lo ? 64 - __clzll((long long)lo) : 0);
}

// T 2^-116 rounded to the nearest double (ties to even); T != 0
__device__ __forceinline__ double q116_to_double(I128 T) {
  uint64_t sign = 0;
  if (T.hi < 0) {
    sign = 1ull << 63;
    T = neg128(T);
  }
  const uint64_t hi = (uint64_t)T.hi, lo = T.lo;
  const int L = bitlen128(hi, lo);
  uint64_t mant;
  int e2;
  if (L <= 53) {
    mant = lo << (53 - L);
    e2 = L - 53 - 116;
  } else {
    int sh = L - 53;  // 1..74
    uint64_t keep = sh < 64 ? ((lo >> sh) | (sh ? hi << (64 - sh) : 0)) : (hi >> (sh - 64));
    int g = sh - 1;  // guard bit position
    uint64_t guard = g < 64 ? (lo >> g) & 1ull : (hi >> (g - 64)) & 1ull;
    bool sticky = g <= 64 ? (g == 64 ? lo != 0 : (lo & ((1ull << g) - 1)) != 0)
                          : (lo != 0 || (hi & ((1ull << (g - 64)) - 1)) != 0);
    mant = keep;
    if (guard && (sticky || (mant & 1ull))) {
      ++mant;
      if (mant == (1ull << 53)) {
        mant >>= 1;
        ++sh;
      }
    }
    e2 = sh - 116;
  }
  return __longlong_as_double((long long)(sign | ((uint64_t)(e2 + 52 + 1023) << 52) | (mant & ((1ull << 52) - 1))));
}

// The same rounding for |T| >= 2^64 (high word non-zero): normalise to 64 bits with the
// dropped bits folded into a sticky bit, then round the 64-bit significand to 53 bits.
__device__ __forceinline__ double q116_to_double_big(I128 T) {
  uint64_t sign = 0;
  if (T.hi < 0) {
    sign = 1ull << 63;
    T = neg128(T);
  }
  const uint64_t hi = (uint64_t)T.hi, lo = T.lo;
  const int s = __clzll((long long)hi);  // 0..63
  const uint64_t m = s ? ((hi << s) | (lo >> (64 - s))) : hi;
  const uint64_t sticky = (s ? (lo << s) : lo) != 0 ? 1ull : 0ull;
  uint64_t mant = m >> 11;  // 53 bits, top bit set
  const uint64_t guard = (m >> 10) & 1ull;
  const uint64_t rest = (m & 0x3FFull) | sticky;
  mant += guard & ((rest != 0 ? 1ull : 0ull) | (mant & 1ull));
  // |T| 2^-116 = mant 2^(11 - s - 116 + 64) = (mant 2^-52) 2^(11 - s); a carry into bit 53 adds one
  // to the exponent field
  return __longlong_as_double((long long)(sign | (((uint64_t)(1033 - s) << 52) + mant)));
}

// -log(c) + r S for a normal x (bit pattern ix); k = the binary exponent part of log x
__device__ __forceinline__ I128 log_fx_core(uint64_t ix, int kadj, const LogTab* tab) {
  const uint64_t tmp = ix - KMC_LOG_OFF;
  const int i = (int)((tmp >> (52 - KMC_LOG_TABLE_BITS)) & ((1u << KMC_LOG_TABLE_BITS) - 1));
  const int k = (int)((int64_t)tmp >> 52) + kadj;
  const uint64_t iz = ix - (tmp & 0xFFF0000000000000ull);
  const int ez = (int)(iz >> 52) - 1023;  // -1 or 0
  const uint64_t Z = (iz & ((1ull << 52) - 1)) | (1ull << 52);
  const uint4 w = *reinterpret_cast<const uint4*>(&tab->t[i][0]);  // one 16-byte load: hi, lo | C
  const uint64_t whi = ((uint64_t)w.y << 32) | w.x;
  const uint64_t wlo = ((uint64_t)w.w << 32) | w.z;
  const uint64_t C = wlo & ((1ull << 21) - 1);
  const int64_t R = (int64_t)(Z * C);        // z c - 1 = R 2^(ez - 72), |R| < 2^62
  const int64_t rq = R >> (8 - ez);          // r 2^64
  const int32_t r30 = (int32_t)(rq >> 34);   // r 2^30
  const int32_t t4 = (int32_t)KMC_FX_S30_4 + (int32_t)(((int64_t)r30 * KMC_FX_S30_5) >> 30);
  const int32_t t3 = (int32_t)KMC_FX_S30_3 + (int32_t)(((int64_t)r30 * t4) >> 30);
  const int64_t t2 = KMC_FX_S62_2 + __mul64hi((long long)rq, (long long)((uint64_t)(int64_t)t3 << 32));
  const int64_t t1 = KMC_FX_S62_1 + __mul64hi((long long)rq, (long long)t2);
  const int64_t S = KMC_FX_S62_0 + __mul64hi((long long)rq, (long long)t1);
  const I128 L1 = sar128(mul64s(R, S), 18 - ez);  // r S in Q116
  // k ln2 in Q116
  const uint64_t ka = (uint64_t)(k < 0 ? -k : k);
  I128 kl;
  kl.lo = ka * KMC_FX_LN2_LO;
  kl.hi = (int64_t)(ka * KMC_FX_LN2_HI + __umul64hi(ka, KMC_FX_LN2_LO));
  if (k < 0) kl = neg128(kl);
  I128 lc;
  lc.lo = wlo & ~((1ull << 21) - 1);
  lc.hi = (int64_t)whi;
  return add128(add128(kl, lc), L1);
}

// log(x) for a normal x > 0 (kadj: exponent correction of a pre-scaled subnormal)
__device__ __forceinline__ double log_fx_normal(uint64_t ix, int kadj, const LogTab* tab) {
  const I128 T = log_fx_core(ix, kadj, tab);
  if (T.hi == 0 && T.lo == 0) return 0.0;
  return q116_to_double(T);
}

__device__ __forceinline__ double kmc_log(double x, const LogTab* __restrict__ tab) {
  uint64_t ix = (uint64_t)__double_as_longlong(x);
  if (!(x > 0.0)) return x == 0.0 ? -__longlong_as_double(0x7FF0000000000000ll) : __longlong_as_double(0x7FF8000000000000ll);
  if (ix >= 0x7FF0000000000000ull) return x;
  int kadj = 0;
  if (ix < 0x0010000000000000ull) {
    x = x * 0x1p52;
    ix = (uint64_t)__double_as_longlong(x);
    kadj = -52;
  }
  return log_fx_normal(ix, kadj, tab);
}

// kmc_log for the dwell-time uniforms u = RN(r / RAND_MAX), 1 <= r <= RAND_MAX: u = 1 gives 0,
// and every other u lies in [2^-31, 1 - 2^-32], where |log u| >= 2^-32 and T >= 2^84 has a
// non-zero high word.
__device__ __forceinline__ double kmc_log_unit(double x, const LogTab* tab) {
  const uint64_t ix = (uint64_t)__double_as_longlong(x);
  if (ix == 0x3FF0000000000000ull) return 0.0;  // x == 1 as an integer test (no FP64 compare)
  return q116_to_double_big(log_fx_core(ix, 0, tab));
}

// log(RN(r / RAND_MAX)) of a dwell-time draw 1 <= r <= RAND_MAX: kmc_log_unit(u_from_rand(r)),
// with u = 1 recognised from r
__device__ __forceinline__ double kmc_dwell_log(uint32_t r, const LogTab* tab) {
  if (r >= kRandMax) return 0.0;
  return q116_to_double_big(log_fx_core((uint64_t)__double_as_longlong(u_from_rand(r)), 0, tab));
}

// ---------------------------------------------------------------- acos (asin Taylor series)
__device__ __forceinline__ double kmc_asin_small(double x) {
  const double a[KMC_ASIN_TERMS] = KMC_ASIN_INIT;
  double z = x * x;
  double p = a[KMC_ASIN_TERMS - 1];
#pragma unroll
  for (int j = KMC_ASIN_TERMS - 2; j >= 0; --j) p = fma(p, z, a[j]);
  double t = x * z;
  return fma(t, p, x);
}

__device__ __forceinline__ double kmc_acos(double c) {
  if (c != c) return c;
  if (c > 1.0 || c < -1.0) return __longlong_as_double(0x7FF8000000000000ll);
  if (c <= 0.5 && c >= -0.5) return KMC_PIO2_HI - (kmc_asin_small(c) - KMC_PIO2_LO);
  if (c > 0.5) {
    double x = sqrt((1.0 - c) * 0.5);
    return 2.0 * kmc_asin_small(x);
  }
  double x = sqrt((1.0 + c) * 0.5);
  return KMC_PI_HI - (2.0 * kmc_asin_small(x) - KMC_PI_LO);
}

// ---------------------------------------------------------------- 3-vectors in the engine's order
__host__ __device__ __forceinline__ double dot3(double a0, double a1, double a2, double b0, double b1, double b2) {
  double acc1 = 0.0, acc2 = 0.0;
  acc1 += a0 * b0;
  acc2 += a1 * b1;
  acc1 += a2 * b2;
  return acc1 + acc2;
}
__host__ __device__ __forceinline__ double norm3(double a0, double a1, double a2) {
  return sqrt(dot3(a0, a1, a2, a0, a1, a2));
}

// index_min(abs(grid - x)): first index of the smallest |grid[i] - x| (scattering_struct.h:41-49)
__device__ __forceinline__ int index_min_abs(const double* __restrict__ g, int n, double x) {
  double best = __longlong_as_double(0x7FF0000000000000ll);
  int idx = 0;
  for (int i = 0; i < n; ++i) {
    double t = fabs(g[i] - x);
    if (t < best) {
      best = t;
      idx = i;
    }
  }
  return idx;
}

// index_min_abs for an ascending grid with (roughly) uniform spacing: the scan is restricted to
// a window around the estimate (x - g[0]) * inv_h and gives the same index as the full scan,
// which is used whenever that cannot be guaranteed.  The computed differences fl(g[i] - x) are
// non-decreasing in i, so |g[i] - x| falls, then rises: its first minimum is the last index left
// of the sign change or the first one right of it.  The window result stands when the sign
// change lies strictly inside the window (or at a grid end) and no tie reaches the window's
// left edge.
__device__ __forceinline__ int index_min_abs_fast(const double* __restrict__ g, int n, double x, double inv_h) {
  if (!(fabs(x) < __longlong_as_double(0x7FF0000000000000ll)) || n < 8) return index_min_abs(g, n, x);
  double e = (x - g[0]) * inv_h;
  int c = e < 0.0 ? 0 : (e > (double)(n - 1) ? n - 1 : (int)(e + 0.5));
  int lo = c - 2 < 0 ? 0 : c - 2, hi = c + 2 > n - 1 ? n - 1 : c + 2;
  double dlo = g[lo] - x, dhi = g[hi] - x;
  if ((lo > 0 && !(dlo < 0.0)) || (hi < n - 1 && !(dhi >= 0.0))) return index_min_abs(g, n, x);
  double best = __longlong_as_double(0x7FF0000000000000ll);
  int idx = lo;
  for (int i = lo; i <= hi; ++i) {
    double t = fabs(g[i] - x);
    if (t < best) {
      best = t;
      idx = i;
    }
  }
  if (idx == lo && lo > 0) return index_min_abs(g, n, x);  // a tie could extend left of the window
  return idx;
}

}  // namespace kmc
