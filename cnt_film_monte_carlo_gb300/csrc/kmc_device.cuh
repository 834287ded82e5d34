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

// ---------------------------------------------------------------- log (Tang's table-driven method)
struct LogTab {
  double t[1 << KMC_LOG_TABLE_BITS][3];
};

// log(z 2^k) from the reduced argument: the common tail of kmc_log and kmc_log_unit.
__device__ __forceinline__ double log_tail(uint64_t ix, uint64_t tmp, double kf, const LogTab* __restrict__ tab) {
  int i = (int)((tmp >> (52 - KMC_LOG_TABLE_BITS)) & ((1u << KMC_LOG_TABLE_BITS) - 1));
  double z = __longlong_as_double((long long)(ix - (tmp & 0xFFF0000000000000ull)));
  double invc = __ldg(&tab->t[i][0]);
  double lhi = __ldg(&tab->t[i][1]);
  double llo = __ldg(&tab->t[i][2]);
  const double c[4] = KMC_LOG1P_INIT;
  double r = fma(z, invc, -1.0);
  double t1 = fma(kf, KMC_LN2_HI, lhi);
  double p = c[3];
  p = fma(p, r, c[2]);
  p = fma(p, r, c[1]);
  p = fma(p, r, c[0]);
  double r2 = r * r;
  double q = r2 * p;
  double s = fma(kf, KMC_LN2_LO, llo) + q;
  return t1 + (r + s);
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
  uint64_t tmp = ix - KMC_LOG_OFF;
  int k = (int)((int64_t)tmp >> 52) + kadj;
  return log_tail(ix, tmp, (double)k, tab);
}

// kmc_log for a normal x in (0, 1] (the dwell-time uniforms): no special cases, and the exponent
// k in [-1022, 0] is turned into a double with integer operations (same exact value as (double)k).
__device__ __forceinline__ double kmc_log_unit(double x, const LogTab* __restrict__ tab) {
  uint64_t ix = (uint64_t)__double_as_longlong(x);
  uint64_t tmp = ix - KMC_LOG_OFF;
  int k = (int)((int64_t)tmp >> 52);
  uint32_t m = (uint32_t)(-k);
  int e = 31 - __clz((int)m);
  uint64_t kb = m ? ((1ull << 63) | ((uint64_t)(1023 + e) << 52) | (((uint64_t)m << (52 - e)) & ((1ull << 52) - 1)))
                  : 0ull;
  return log_tail(ix, tmp, __longlong_as_double((long long)kb), tab);
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

}  // namespace kmc
