// kmc_hop_common.cuh -- device pieces shared by the hop kernels: exciton state in registers,
// fly from a materialised position, load/store of the slot arrays, removal and reinjection,
// counters.  Included by kmc_kernels.cu and the two translation units of the mixed kernel.
#pragma once

#include "kmc_internal.h"

namespace kmc {

// Upper bound of link crossings in one free flight: a flight of length v*dt over links of
// positive length ends long before; only zero-length links (coincident sites) could loop.
constexpr int kMaxCrossings = 1 << 22;

struct Exciton {
  int32_t site;
  bool heading, at_site, active;
  double px, py, pz, dx, dy, dz, ff;
  Rng g;
  uint64_t hops, crossings;
  int64_t trace_i;
};

__device__ __forceinline__ double dwell(double inv_total, uint32_t r, const LogTab* tab) {
  // ff_time: -(1/Gamma) log(r / RAND_MAX), r != 0 (scatterer.h:74-80)
  return -inv_total * kmc_log((double)r / (double)kRandMax, tab);
}

__device__ __forceinline__ void trace_push(const HopArgs& a, const Exciton& e, int32_t v) {
  if (e.trace_i >= 0) {
    int64_t c = a.trace_cnt[e.trace_i];
    if (c < a.trace_cap) a.trace[e.trace_i * a.trace_cap + c] = v;
    a.trace_cnt[e.trace_i] = c + 1;
  }
}

// particle::fly (particle.cpp:9-54) in FP64 from a materialised position.
__device__ __forceinline__ void fly_full(const HopArgs& a, Exciton& e, double dtf) {
  if (a.left[e.site] < 0 && a.right[e.site] < 0) return;
  for (int guard = 0;; ++guard) {
    if (guard >= kMaxCrossings) {
      atomicOr(a.err, KMC_ERR_FLIGHT_CODE);
      return;
    }
    int32_t l = a.left[e.site], r = a.right[e.site];
    int32_t next = e.heading ? (r > -1 ? r : l) : (l > -1 ? l : r);
    if (!KMC_DCHECK(a.err, next >= 0 && next < a.n_sites)) return;
    e.heading = (next == r);
    double4_32a t = a.pos4[next];
    double dist = norm3(e.px - t.x, e.py - t.y, e.pz - t.z);
    if (dist / a.v < dtf) {
      e.px = t.x;
      e.py = t.y;
      e.pz = t.z;
      e.site = next;
      dtf -= dist / a.v;
      e.crossings++;
      trace_push(a, e, -1 - next);
    } else {
      double e0 = t.x - e.px, e1 = t.y - e.py, e2 = t.z - e.pz;
      double nn = norm3(e0, e1, e2);
      double den = nn != 0 ? nn : 1.0;
      double u0 = e0 / den, u1 = e1 / den, u2 = e2 / den;
      double k = a.v * dtf;
      e.px = e.px + k * u0;
      e.py = e.py + k * u1;
      e.pz = e.pz + k * u2;
      return;
    }
  }
}

// particle::step (particle.cpp:57-80) in FP64 over the blocked rows: while the dwell time fits in
// the rest of dt, fly, select the next site by the bisection of update_state
// (scatterer.cpp:14-30) over the FP64 cumulative rates, move there, draw the next dwell time;
// then fly the rest.  False when the exciton exceeded the hop cap (the error word is set).
__device__ __forceinline__ bool step_fp64(const HopArgs& a, Exciton& e, double dt) {
  double rem = dt;
  int64_t hs = 0;
  while (e.ff <= rem) {
    rem -= e.ff;
    fly_full(a, e, e.ff);
    int32_t ns = e.site;
    int64_t n = a.rec[e.site].len_flags & kLenMask;  // row length (rows are stored per slot)
    if (n > 0) {
      const int64_t bo = a.blkptr[e.site];
      if (!KMC_DCHECK(a.err, bo >= 0 && bo + ((n + 7) >> 3) <= a.n_blocks)) return false;  // the exciton stops
      const double* cum = a.cump + bo * 8;
      uint32_t r = e.g.next();
      double dice = a.total[e.site] * (double)r / (double)kRandMax;
      unsigned left = (unsigned)-1, right = (unsigned)(n - 1);
      while (left + 1 < right) {
        unsigned mid = (left + right) / 2;
        if (cum[mid] <= dice)
          left = mid;
        else
          right = mid;
      }
      ns = a.blocks[bo + (right >> 3)].col[right & 7];
      if (!KMC_DCHECK(a.err, ns >= 0 && ns < a.n_sites)) return false;
    }
    e.hops++;
    trace_push(a, e, ns);
    if (ns != e.site) {
      e.site = ns;
      double4_32a p = a.pos4[ns];
      e.px = p.x;
      e.py = p.y;
      e.pz = p.z;
    }
    uint32_t r;
    while ((r = e.g.next()) == 0) {
    }
    e.ff = dwell(a.inv_total[e.site], r, a.logtab);
    if (++hs > a.hop_cap) {
      atomicOr(a.err, KMC_ERR_HOP_CAP_CODE);
      return false;
    }
  }
  fly_full(a, e, rem);
  e.ff -= rem;
  return true;
}

__device__ __forceinline__ void load_exciton(const HopArgs& a, int64_t slot, Exciton& e) {
  const int64_t ns = a.n_slots;
  uint32_t fl = a.e_flags[slot];
  e.active = (fl & kExActive) != 0;
  e.heading = (fl & kExHeading) != 0;
  e.at_site = (fl & kExAtSite) != 0;
  e.site = a.e_site[slot];
  if (e.active && !KMC_DCHECK(a.err, e.site >= 0 && e.site < a.n_sites)) e.active = false;  // slot left as it is
  e.px = a.e_pos[slot];
  e.py = a.e_pos[ns + slot];
  e.pz = a.e_pos[2 * ns + slot];
  e.dx = a.e_delta[slot];
  e.dy = a.e_delta[ns + slot];
  e.dz = a.e_delta[2 * ns + slot];
  e.ff = a.e_ff[slot];
  e.hops = 0;
  e.crossings = 0;
}

__device__ __forceinline__ void store_exciton(const HopArgs& a, int64_t slot, const Exciton& e) {
  const int64_t ns = a.n_slots;
  if (!e.active) return;
  (void)KMC_DCHECK(a.err, e.g.n >= a.e_draws[slot]);  // a Philox counter only moves forward (no wrap)
  a.e_flags[slot] = kExActive | (e.heading ? kExHeading : 0u) | (e.at_site ? kExAtSite : 0u);
  a.e_site[slot] = e.site;
  a.e_pos[slot] = e.px;
  a.e_pos[ns + slot] = e.py;
  a.e_pos[2 * ns + slot] = e.pz;
  a.e_delta[slot] = e.dx;
  a.e_delta[ns + slot] = e.dy;
  a.e_delta[2 * ns + slot] = e.dz;
  a.e_ff[slot] = e.ff;
  a.e_draws[slot] = e.g.n;
  a.e_hops[slot] += e.hops;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Removal and reinjection (monte_carlo.cpp:330-336); position must be materialised.
__device__ __forceinline__ void maybe_reinject(const HopArgs& a, const FilmDev& f, Exciton& e) {
  if (f.mode != 0) return;
  bool out = (e.px < f.rmin[0]) | (e.py < f.rmin[1]) | (e.pz < f.rmin[2]) | (f.rmax[0] < e.px) |
             (f.rmax[1] < e.py) | (f.rmax[2] < e.pz);
  if (!out) return;
  uint32_t dice = e.g.next() % (uint32_t)f.n_inj;
  int32_t site = a.inject[f.inj0 + dice];
  if (!KMC_DCHECK(a.err, site >= 0 && site < a.n_sites)) return;
  double4_32a p = a.pos4[site];
  e.px = p.x;
  e.py = p.y;
  e.pz = p.z;
  e.site = site;
  e.at_site = true;
  trace_push(a, e, INT32_MIN);
  trace_push(a, e, site);
}

__device__ __forceinline__ void step_epilogue(const HopArgs& a, const FilmDev& f, int32_t film, Exciton& e,
                                              double ox, double oy, double oz, int64_t s) {
  if (e.active) {
    e.dx += e.px - ox;
    e.dy += e.py - oy;
    e.dz += e.pz - oz;
    maybe_reinject(a, f, e);
  }
  double sx = e.active ? e.dx * e.dx : 0.0;
  double sy = e.active ? e.dy * e.dy : 0.0;
  double sz = e.active ? e.dz * e.dz : 0.0;
  sx = warp_sum(sx);
  sy = warp_sum(sy);
  sz = warp_sum(sz);
  if ((threadIdx.x & 31) == 0 && KMC_DCHECK(a.err, a.step0 + s < a.msd_cap)) {
    const int64_t batch = ((int64_t)(blockIdx.x * (int64_t)blockDim.x + threadIdx.x - f.slot0) >> 5) % a.msd_batches;
    double* m = a.msd + (((int64_t)film * a.msd_cap + a.step0 + s) * a.msd_batches + batch) * 3;
    atomicAdd(m, sx);
    atomicAdd(m + 1, sy);
    atomicAdd(m + 2, sz);
  }
}

__device__ __forceinline__ void flush_counters(const HopArgs& a, const Exciton& e, uint64_t exact) {
  uint64_t h = e.hops, c = e.crossings, x = exact;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    h += __shfl_xor_sync(0xffffffffu, h, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
    x += __shfl_xor_sync(0xffffffffu, x, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&a.counters[0], (unsigned long long)h);
    atomicAdd(&a.counters[1], (unsigned long long)c);
    if (x) atomicAdd(&a.counters[2], (unsigned long long)x);
  }
}

}  // namespace kmc
