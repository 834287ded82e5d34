// kmc_pair.cuh -- pair geometry and rate-table lookup of find_neighbors
// (src/monte_carlo/scatterer.cpp:40-68, scattering_struct.h:38-52), shared by the neighbour-list
// kernels.
#pragma once
#include "kmc_internal.h"

namespace kmc {

// not inlined: six inlined grid lookups made this translation unit take minutes to compile,
// and the neighbour build is not on the hop path
static __device__ __noinline__ double table_rate(const TableDev& t, double th, double zsh, double a1, double a2,
                                             double dist, int64_t pair_off) {
  auto idx = [&](int d, double x) {
    return t.inv_h[d] > 0 ? index_min_abs_fast(t.grid[d], t.n[d], x, t.inv_h[d]) : index_min_abs(t.grid[d], t.n[d], x);
  };
  if (t.kind == 4) {
    int i0 = idx(0, th);
    int i1 = idx(1, zsh);
    int i2 = idx(2, a1);
    int i3 = idx(3, a2);
    return t.rate[(((int64_t)i0 * t.n[1] + i1) * t.n[2] + i2) * t.n[3] + i3];
  }
  int i0 = idx(0, dist);
  int i1 = idx(1, th);
  return t.rate[pair_off + (int64_t)i0 * t.n[1] + i1];
}

// Offset of the (donor, acceptor) table of a KMC_TABLE_2D_SPECIES table (0 for the others).
__device__ __forceinline__ int64_t pair_table(const TableDev& t, int64_t donor, int64_t acceptor) {
  if (t.kind != 3) return 0;
  return ((int64_t)t.species[donor] * t.n[2] + t.species[acceptor]) * ((int64_t)t.n[0] * t.n[1]);
}

// Pair rate of find_neighbors (scatterer.cpp:40-68) for a pair already inside the window;
// pair_off selects the chirality pair's table (pair_table).
__device__ __forceinline__ double pair_rate(const TableDev& t, const double4_32a& p1, const double* a1v, const double4_32a& p2,
                                            const double* a2v, double dR0, double dR1, double dR2, double distance,
                                            int64_t pair_off = 0) {
  double cosT = dot3(a1v[0], a1v[1], a1v[2], a2v[0], a2v[1], a2v[2]);
  double theta, ash1 = 0, ash2 = 0, zsh = 0;
  if (t.kind != 4) {  // 2-D tables: folded angle
    double ac = fabs(cosT);
    theta = ac >= 1.0 ? 0.0 : kmc_acos(ac);
  } else if (cosT == 1) {
    ash1 = 0;
    ash2 = dot3(dR0, dR1, dR2, a1v[0], a1v[1], a1v[2]);
    theta = 0;
    double tt = dot3(dR0, dR1, dR2, a1v[0], a1v[1], a1v[2]);
    zsh = norm3(dR0 - tt * a1v[0], dR1 - tt * a1v[1], dR2 - tt * a1v[2]);
  } else {
    theta = kmc_acos(cosT);
    double y1 = dot3(a1v[0], a1v[1], a1v[2], dR0, dR1, dR2);
    double y2 = dot3(a2v[0], a2v[1], a2v[2], dR0, dR1, dR2);
    double sin2 = 1 - cosT * cosT;
    ash1 = (y1 + y2 * cosT) / sin2;
    ash2 = (y2 + y1 * cosT) / sin2;
    zsh = norm3((ash1 * a1v[0] + p1.x) - (ash2 * a2v[0] + p2.x), (ash1 * a1v[1] + p1.y) - (ash2 * a2v[1] + p2.y),
                (ash1 * a1v[2] + p1.z) - (ash2 * a2v[2] + p2.z));
  }
  return table_rate(t, theta, zsh, ash1, ash2, distance, pair_off);
}

// pair_rate_2d's exact path (the reference's root and arccosine), out of line: it runs for a
// few pairs in 10^4, and inlined it would sit in the row loop of every pair.
static __device__ __noinline__ double pair_rate_2d_exact(const TableDev& t, const double* a1v, const double* a2v,
                                                         double dR0, double dR1, double dR2, double d2, int64_t pair_off,
                                                         const double4_32a& p1, const double4_32a& p2) {
  const double a1c[3] = {a1v[0], a1v[1], a1v[2]}, a2c[3] = {a2v[0], a2v[1], a2v[2]};
  return pair_rate(t, p1, a1c, p2, a2c, dR0, dR1, dR2, sqrt(d2), pair_off);
}

// Rate of a 2-D table (kinds 2, 3) for a pair in the window, from dR and the two axes: the same
// table entry as pair_rate, found without its FP64 square root and arccosine.  The nearest
// distance index follows from d^2 against the squared midpoints of the distance grid, the
// nearest angle index from |cos theta| against the cosines of the midpoints of the angle grid;
// both are seeded by an FP32 estimate and confirmed in FP64 with a margin (1e-12 relative in d^2,
// 1e-13 in |cos theta|) far wider than the rounding of the reference's own path (FP64 sqrt,
// kmc_acos within 2 ulp, index_min's FP64 differences).  A value inside a margin, or an estimate
// the check rejects, takes pair_rate's exact path, so the entry is always the one the reference
// picks.
__device__ __forceinline__ double pair_rate_2d(const TableDev& t, const double* a1v, const double* a2v, double dR0,
                                               double dR1, double dR2, int64_t pair_off, const double4_32a& p1,
                                               const double4_32a& p2) {
  const double d2 = dot3(dR0, dR1, dR2, dR0, dR1, dR2);
  const double cosT = dot3(a1v[0], a1v[1], a1v[2], a2v[0], a2v[1], a2v[2]);
  const double ac = fabs(cosT);
  if (t.d2_above && ac <= 1.0) {
    const int n0 = t.n[0], n1 = t.n[1];
    int c0 = (int)floorf(((float)sqrt((float)d2) - t.g0f[0]) * t.ihf[0] + 0.5f);
    c0 = c0 < 0 ? 0 : (c0 > n0 - 1 ? n0 - 1 : c0);
    int c1 = (int)floorf((acosf((float)ac) - t.g0f[1]) * t.ihf[1] + 0.5f);
    c1 = c1 < 0 ? 0 : (c1 > n1 - 1 ? n1 - 1 : c1);
    const bool ok0 = (c0 == 0 || d2 > t.d2_above[c0 - 1]) && (c0 == n0 - 1 || d2 < t.d2_below[c0]);
    const bool ok1 = (c1 == 0 || ac < t.cos_below[c1 - 1]) && (c1 == n1 - 1 || ac > t.cos_above[c1]);
    if (ok0 && ok1) return t.rate[pair_off + (int64_t)c0 * n1 + c1];
  }
  return pair_rate_2d_exact(t, a1v, a2v, dR0, dR1, dR2, d2, pair_off, p1, p2);
}

}  // namespace kmc
