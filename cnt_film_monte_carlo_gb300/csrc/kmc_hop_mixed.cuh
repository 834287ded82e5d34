// kmc_hop_mixed.cuh -- the mixed-precision hop kernel, a template over (threads per block,
// resident blocks per SM).  Instantiated in kmc_mixed_small.cu (128-thread blocks) and
// kmc_mixed_large.cu (256-, 768- and 1024-thread blocks) so that the variants compile in
// parallel.
#pragma once

#include "kmc_hop_common.cuh"

namespace kmc {

// Same decisions and FP64 values as k_hop_fp64, fewer FP64 operations and bytes:
//  * cumulative rates are searched as cum/total in FP32; a selection is accepted only when both
//    bracketing entries are clear of the uniform by a relative margin of 2^-20 (far above the
//    FP32 rounding of either side), otherwise it is re-resolved with the FP64 cumulative row;
//  * the dwell uniform RN(r / RAND_MAX) is formed by integer arithmetic (u_from_rand);
//  * link crossings compare the high 32 bits of the exact link time with the flight time
//    (non-negative doubles order like their bit patterns) and read the low bits only on a tie;
//  * the position is kept as "at the current site" between hops: a partial flight followed by a
//    hop is overwritten by the hop (particle.cpp:78-81), so it is only computed when observed.
__device__ __forceinline__ bool link_time_less(uint32_t lt_hi, const double2* lt64, int32_t site, bool right_side,
                                               double dtf, uint64_t& exact) {
  int64_t db = __double_as_longlong(dtf);
  int32_t dhi = (int32_t)(db >> 32);
  if ((int32_t)lt_hi != dhi) return (int32_t)lt_hi < dhi;
  ++exact;
  double2 l = lt64[site];
  double lt = right_side ? l.y : l.x;
  return lt < dtf;
}

// step-end batching: lanes at the end of a step of fewer than kHoldHops hops wait for the warp
constexpr uint32_t kHoldHops = 64;

// Exact ff <= rem for rem >= +0 and ff not a NaN with the sign bit set (device NaNs are
// positive): non-negative doubles order like their bit patterns, and a negative ff (or -0.0)
// is below every non-negative rem in both orders.
__device__ __forceinline__ bool dwell_fits(double ff, double rem) {
  return __double_as_longlong(ff) <= __double_as_longlong(rem);
}

// Step-boundary state of one lane's exciton, kept in shared memory (one slot per thread): only
// the event loop's hot values stay in registers, which lets more warps stay resident.  The
// exciton's Philox key and stream (film seed, index in the film) are re-derived from the slot,
// and the step's starting point and displacement stay in the slot arrays until the step ends,
// leaving more of the SM's shared-memory/L1 array to the L1 cache.
struct ColdState {
  double p[3];   // position (valid when not at the site)
};

// Draw buffer of a lane: a ring of 8 Philox words in shared memory (word k of the lane at
// ring[k * BLOCK + tid], so a warp's accesses hit 32 banks), holding `avail` words from draw index
// n on.  The ring holds whole blocks: block b occupies words 4(b mod 2) .. +3.
struct DrawRing {
  uint32_t* r;  // this lane's word 0
  int stride;   // BLOCK
  __device__ __forceinline__ uint32_t word(uint64_t i) const { return r[(int)(i & 7) * stride]; }
  // Philox block b = d / 4 (d a multiple of 4) into its ring words
  __device__ __forceinline__ void fill(uint64_t d, uint64_t seed, uint64_t stream) const {
    const uint64_t b = d >> 2;
    uint32_t o[4];
    philox4x32_10((uint32_t)b, (uint32_t)(b >> 32), (uint32_t)stream, (uint32_t)(stream >> 32), (uint32_t)seed,
                  (uint32_t)(seed >> 32), o);
    const int k = (int)(d & 4);
#pragma unroll
    for (int j = 0; j < 4; ++j) r[(k + j) * stride] = o[j];
  }
};

// fly(dtf) at the end of a step (particle.cpp:9-54), the position materialised in e.  From a
// site (at_site: e's position is the site's) the link's flight time and unit vector are the
// precomputed lt64 and ulink, which particle::fly's operations give from the site position; a
// flight that starts between sites computes them as fly_full does.
__device__ __forceinline__ void fly_end(const HopArgs& a, Exciton& e, bool at_site, double dtf) {
  if (a.left[e.site] < 0 && a.right[e.site] < 0) return;
  for (int guard = 0;; ++guard) {
    if (guard >= kMaxCrossings) {
      atomicOr(a.err, KMC_ERR_FLIGHT_CODE);
      return;
    }
    const int32_t l = a.left[e.site], r = a.right[e.site];
    const int32_t next = e.heading ? (r > -1 ? r : l) : (l > -1 ? l : r);
    if (!KMC_DCHECK(a.err, next >= 0 && next < a.n_sites)) return;
    const bool to_right = (next == r);
    e.heading = to_right;
    const double4_32a t = a.pos4[next];
    if (at_site) {
      const double2 lt2 = a.lt64[e.site];
      const double lt = to_right ? lt2.y : lt2.x;
      if (lt < dtf) {
        e.px = t.x;
        e.py = t.y;
        e.pz = t.z;
        e.site = next;
        dtf -= lt;
        e.crossings++;
        trace_push(a, e, -1 - next);
        continue;
      }
      const double* u = a.ulink + (int64_t)e.site * 6 + (to_right ? 3 : 0);
      const double k = a.v * dtf;
      e.px = e.px + k * u[0];
      e.py = e.py + k * u[1];
      e.pz = e.pz + k * u[2];
      return;
    }
    const double dist = norm3(e.px - t.x, e.py - t.y, e.pz - t.z);
    if (dist / a.v < dtf) {
      e.px = t.x;
      e.py = t.y;
      e.pz = t.z;
      e.site = next;
      dtf -= dist / a.v;
      e.crossings++;
      trace_push(a, e, -1 - next);
      at_site = true;
      continue;
    }
    const double e0 = t.x - e.px, e1 = t.y - e.py, e2 = t.z - e.pz;
    const double nn = norm3(e0, e1, e2);
    const double den = nn != 0 ? nn : 1.0;
    const double u0 = e0 / den, u1 = e1 / den, u2 = e2 / den;
    const double k = a.v * dtf;
    e.px = e.px + k * u0;
    e.py = e.py + k * u1;
    e.pz = e.pz + k * u2;
    return;
  }
}

__device__ __forceinline__ void cold_trace(const HopArgs& a, int64_t t, int32_t v) {
  int64_t k = a.trace_cnt[t];
  if (k < a.trace_cap) a.trace[t * a.trace_cap + k] = v;
  a.trace_cnt[t] = k + 1;
}

// Persistent work queue: the grid holds as many threads as the GPU keeps resident; each lane
// takes the next exciton slot from a global counter (warp-aggregated atomics), advances it
// through all n_steps steps of the launch on its own, stores it and takes the next one, so no
// lane waits for another lane's exciton.  MSD sums of a single-film run without batches go to
// block-shared bins (added to global memory once per block); otherwise to global memory.
template <int BLOCK, int MINB, bool HOLD>
__global__ void __launch_bounds__(BLOCK, MINB) k_hop_mixed(HopArgs a, int64_t n_steps, unsigned long long* queue,
                                                         int single_film) {
  extern __shared__ double s_mem[];
  LogTab* s_log = reinterpret_cast<LogTab*>(s_mem);  // the log table, read once per hop
  double* s_bins = s_mem + sizeof(LogTab) / sizeof(double);  // [n_steps][3] when single_film
  ColdState* cs0 = reinterpret_cast<ColdState*>(s_bins + (single_film ? (n_steps * 3 + 15) / 16 * 16 : 0));
  ColdState* cs = cs0 + threadIdx.x;
  const DrawRing ring{reinterpret_cast<uint32_t*>(cs0 + BLOCK) + threadIdx.x, BLOCK};
  const int lane = threadIdx.x & 31;
  {
    const uint64_t* src = &a.logtab->t[0][0];
    uint64_t* dst = &s_log->t[0][0];
    for (int i = threadIdx.x; i < (int)(sizeof(LogTab) / 8); i += blockDim.x) dst[i] = __ldg(src + i);
  }
  if (single_film)
    for (int64_t i = threadIdx.x; i < n_steps * 3; i += blockDim.x) s_bins[i] = 0.0;
  __syncthreads();
  const float lo_m = 1.0f - 0x1p-20f, hi_m = 1.0f + 0x1p-20f;
  uint64_t exact = 0, lane_hops = 0, lane_cross = 0;
  // hot state
  int64_t cur = -1;
  int32_t site = -1, film = 0, s = 0;
  uint32_t ehops = 0, ecross = 0, hs = 0;
  bool heading = false, at_site = false, tracing = false;
  double ff = 0, rem = 0;
  uint64_t rn = 0;
  uint32_t avail = 0;  // draws buffered in the ring from rn on
  double inv = 0;
  uint32_t blk = 0, lenf = 0, lth_l = 0, lth_r = 0;
  int32_t lnk_l = -1, lnk_r = -1;
  const SiteRec* recp = nullptr;
  const FilmDev* fp = a.films;
  bool alive = true;
  auto load_rec = [&](int32_t st) {
    recp = a.rec + st;
    const int4* q = reinterpret_cast<const int4*>(recp);
    int4 q0 = __ldg(q), q1 = __ldg(q + 1);
    inv = __hiloint2double(q0.y, q0.x);
    blk = (uint32_t)q0.z;
    lenf = (uint32_t)q0.w;
    lnk_l = q1.x;
    lnk_r = q1.y;
    lth_l = (uint32_t)q1.z;
    lth_r = (uint32_t)q1.w;
#ifdef KMC_CHECK
    // the record's row must lie inside the block arrays and its links inside the sites; a bad
    // row is treated as empty and a bad link as none
    if (!KMC_DCHECK(a.err, fp->blk0 + (int64_t)blk + (int64_t)(((lenf & kLenMask) + 7) >> 3) <= a.n_blocks))
      lenf &= ~kLenMask;
    if (!KMC_DCHECK(a.err, lnk_l < a.n_sites)) lnk_l = -1;
    if (!KMC_DCHECK(a.err, lnk_r < a.n_sites)) lnk_r = -1;
#endif
  };
  for (;;) {
    // all 32 lanes meet here once per event, so every event starts with the warp converged
    if (!__any_sync(0xffffffffu, alive)) break;
    // When any lane of the warp is short of a hop's two draws, every lane with room in its ring
    // adds the next Philox block: the warp runs Philox together about every other hop instead
    // of once per hop for half of its lanes.
    if (__any_sync(0xffffffffu, alive && cur >= 0 && avail < 2)) {
      if (alive && cur >= 0 && avail <= 4) {
        ring.fill(rn + avail, a.films[film].seed, (uint64_t)(cur - a.films[film].slot0));
        avail += 4;
      }
    }
    if (!alive) continue;
    if (cur < 0) {
      // ---- take the next exciton slot
      unsigned m = __activemask();
      int leader = __ffs(m) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(queue, (unsigned long long)__popc(m));
      base = __shfl_sync(m, base, leader);
      cur = (int64_t)base + __popc(m & ((1u << lane) - 1));
      if (cur >= a.n_slots) {
        alive = false;
        continue;
      }
      if (a.order) cur = a.order[cur];
      film = a.warp_film[cur >> 5];
      fp = a.films + film;
      const int64_t ns = a.n_slots;
      uint32_t fl = a.e_flags[cur];
      if (!(fl & kExActive)) {
        cur = -1;
        continue;
      }
      heading = (fl & kExHeading) != 0;
      at_site = (fl & kExAtSite) != 0;
      site = a.e_site[cur];
      if (!KMC_DCHECK(a.err, site >= 0 && site < a.n_sites)) {  // slot left as it is
        cur = -1;
        continue;
      }
      ff = a.e_ff[cur];
      int64_t local = cur - fp->slot0;
      tracing = film == 0 && local < a.n_trace;
      rn = a.e_draws[cur];
      ring.fill(rn & ~3ull, a.films[film].seed, (uint64_t)(cur - a.films[film].slot0));
      avail = 4 - (uint32_t)(rn & 3);
      double px, py, pz;
      if (at_site) {
        double4_32a p = a.pos4[site];
        px = p.x;
        py = p.y;
        pz = p.z;
        // the slot's position array holds the step's starting point until the step ends
        a.e_pos[cur] = px;
        a.e_pos[ns + cur] = py;
        a.e_pos[2 * ns + cur] = pz;
      } else {
        px = a.e_pos[cur];
        py = a.e_pos[ns + cur];
        pz = a.e_pos[2 * ns + cur];
      }
      cs->p[0] = px;
      cs->p[1] = py;
      cs->p[2] = pz;
      rem = a.dt;
      s = 0;
      hs = 0;
      ehops = 0;
      ecross = 0;
      load_rec(site);
    }
    const FilmDev& f = *fp;
    const bool step_end = !dwell_fits(ff, rem);
    if (HOLD) {
      // The end of a step is mostly FP64 work (flight, displacement, MSD), which the FP64 pipe
      // runs at the same cost for one lane as for a warp.  When steps are short (few hops per
      // step: the HOLD instantiation, launched when a.hold_short), a lane at the end of a short
      // step waits until half of the warp's active lanes are at the end of theirs, so that they
      // run it together.  The waiting lanes stay at their step ends and every other lane reaches
      // its own, so the count only grows and the wait ends.  Only the order of work changes,
      // never a result.
      const unsigned act = __activemask();
      const unsigned ends = __ballot_sync(act, step_end);
      if (step_end && hs < kHoldHops && 2 * __popc(ends) < __popc(act)) continue;
    }
    if (!step_end) {
      // ------------------------------------------------ one event of particle::step (particle.cpp:71-84)
      rem -= ff;
      double dtf = ff;
      if (lnk_l >= 0 || lnk_r >= 0) {  // fly(ff)
        for (int guard = 0;; ++guard) {
          if (guard >= kMaxCrossings) {
            atomicOr(a.err, KMC_ERR_FLIGHT_CODE);
            break;
          }
          int32_t next = heading ? (lnk_r > -1 ? lnk_r : lnk_l) : (lnk_l > -1 ? lnk_l : lnk_r);
          bool to_right = (next == lnk_r);
          heading = to_right;
          bool cross;
          double lt;
          if (at_site) {
            cross = link_time_less(to_right ? lth_r : lth_l, a.lt64, site, to_right, dtf, exact);
            if (cross) {
              double2 l = a.lt64[site];
              lt = to_right ? l.y : l.x;
            }
          } else {
            double4_32a t = a.pos4[next];
            double dist = norm3(cs->p[0] - t.x, cs->p[1] - t.y, cs->p[2] - t.z);
            lt = dist / a.v;
            cross = lt < dtf;
          }
          if (cross) {
            site = next;
            at_site = true;
            dtf -= lt;
            ecross++;
            if (tracing) cold_trace(a, cur - a.films[film].slot0, -1 - next);
            load_rec(next);
            continue;
          }
          // the partial flight is observed only when no hop follows (empty neighbour list)
          if ((lenf & kLenMask) == 0) {
            if (at_site) {
              double4_32a p = a.pos4[site];
              cs->p[0] = p.x;
              cs->p[1] = p.y;
              cs->p[2] = p.z;
            }
            double4_32a t = a.pos4[next];
            double e0 = t.x - cs->p[0], e1 = t.y - cs->p[1], e2 = t.z - cs->p[2];
            double nn = norm3(e0, e1, e2);
            double den = nn != 0 ? nn : 1.0;
            double u0 = e0 / den, u1 = e1 / den, u2 = e2 / den;
            double k = a.v * dtf;
            cs->p[0] = cs->p[0] + k * u0;
            cs->p[1] = cs->p[1] + k * u1;
            cs->p[2] = cs->p[2] + k * u2;
            at_site = false;
          }
          break;
        }
      }
      // update_state (scatterer.cpp:9-31)
      uint32_t n = lenf & kLenMask;
      int32_t nsite = site;
      uint32_t rf;  // the dwell-time draw of this hop (drawn after the selection's)
      uint32_t r = 0;
      float4 q0 = make_float4(0.f, 0.f, 0.f, 0.f), q1 = q0;
      if (n > 0) {
        if (avail < 2) {  // first hop after taking an exciton
          ring.fill(rn + avail, a.films[film].seed, (uint64_t)(cur - a.films[film].slot0));
          avail += 4;
        }
        r = ring.word(rn) >> 1;
        rf = ring.word(rn + 1) >> 1;
        rn += 2;
        avail -= 2;
        const float4* cq = reinterpret_cast<const float4*>(recp->coarse);  // first search level
        q0 = __ldg(cq);
        q1 = __ldg(cq + 1);
      } else {
        if (avail == 0) {
          ring.fill(rn, a.films[film].seed, (uint64_t)(cur - a.films[film].slot0));
          avail = 4;
        }
        rf = ring.word(rn) >> 1;
        ++rn;
        --avail;
      }
      while (rf == 0) {  // ff_time rejects r == 0
        if (avail == 0) {
          ring.fill(rn, a.films[film].seed, (uint64_t)(cur - a.films[film].slot0));
          avail = 4;
        }
        rf = ring.word(rn) >> 1;
        ++rn;
        --avail;
      }
      // the dwell time's log does not depend on the row: computed here, it covers the latency of
      // the row loads
      const double dlog = kmc_dwell_log(rf, s_log);
      if (n > 0) {
        const RowBlock* __restrict__ rb = a.blocks + f.blk0 + blk;
        bool resolved = false;
        if (!(lenf & (kRecExact | kRecLong))) {
          // two- or three-level search for the first FP32 value > u (count of values <= u)
          float u = __uint2float_rn(r) * (1.0f / 2147483647.0f);
          float co[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
          int j1 = 0;
#pragma unroll
          for (int i = 0; i < 8; ++i) j1 += (co[i] <= u);
          float prev = co[0];
#pragma unroll
          for (int i = 1; i < 8; ++i)
            if (j1 == i + 1) prev = co[i];  // value before the group: coarse[j1 - 1]
          uint32_t nb = (n + 7) >> 3;
          uint32_t bsel;
          if (nb <= 8) {
            bsel = (uint32_t)j1;
          } else {
            uint32_t G = (nb + 7) >> 3, g0 = (uint32_t)j1 * G;
            const float* __restrict__ bl = a.blast + f.blk0 + blk + g0;
            float v[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) v[i] = ((uint32_t)i < G && g0 + i < nb) ? __ldg(bl + i) : __int_as_float(0x7f800000);
            int j2 = 0;
#pragma unroll
            for (int i = 0; i < 8; ++i) j2 += (v[i] <= u);
#pragma unroll
            for (int i = 0; i < 7; ++i)
              if (j2 == i + 1) prev = v[i];
            bsel = g0 + (uint32_t)j2;
          }
          // u at or above the row's last FP32 value (u == 1.0f: r >= 2^31 - 64) selects no block of the
          // row; such draws are resolved in FP64 below
          if (bsel < nb) {
            const float4* bp = reinterpret_cast<const float4*>(rb + bsel);
            float4 c0 = __ldg(bp), c1 = __ldg(bp + 1);
            int4 k0 = __ldg(reinterpret_cast<const int4*>(bp + 2)), k1 = __ldg(reinterpret_cast<const int4*>(bp + 3));
            float c[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
            int32_t cl[8] = {k0.x, k0.y, k0.z, k0.w, k1.x, k1.y, k1.z, k1.w};
            int kk = 0;
#pragma unroll
            for (int i = 0; i < 8; ++i) kk += (c[i] <= u);
            float ck = c[0], ckm = prev;
            int32_t colk = cl[0];
#pragma unroll
            for (int i = 1; i < 8; ++i)
              if (kk == i) {
                ck = c[i];
                ckm = c[i - 1];
                colk = cl[i];
              }
            uint32_t R = bsel * 8 + (uint32_t)kk;
            if ((R == 0 || ckm < u * lo_m) && (R == n - 1 || ck > u * hi_m)) {
              nsite = colk;
              resolved = true;
            }
          }
        } else if ((lenf & kRecLong) && !(lenf & kRecExact)) {
          // rows beyond 512 entries: the reference bisection on the blocked FP32 values
          float u = __uint2float_rn(r) * (1.0f / 2147483647.0f);
          unsigned left = (unsigned)-1, right = n - 1;
          float cl = 0.f, cr = 0.f;
          while (left + 1 < right) {
            unsigned mid = (left + right) / 2;
            float cv = __ldg(&rb[mid >> 3].c[mid & 7]);
            if (cv <= u) {
              left = mid;
              cl = cv;
            } else {
              right = mid;
              cr = cv;
            }
          }
          if ((left == (unsigned)-1 || cl < u * lo_m) && (right == n - 1 || cr > u * hi_m)) {
            nsite = __ldg(&rb[right >> 3].col[right & 7]);
            resolved = true;
          }
        }
        if (!resolved) {  // exact FP64 selection on the site's FP64 row (update_state, scatterer.cpp:17-30)
          ++exact;
          const double* cum = a.cump + (f.blk0 + blk) * 8;
          double dice = a.total[site] * (double)r / (double)kRandMax;
          unsigned left = (unsigned)-1, right = n - 1;
          while (left + 1 < right) {
            unsigned mid = (left + right) / 2;
            if (cum[mid] <= dice)
              left = mid;
            else
              right = mid;
          }
          nsite = rb[right >> 3].col[right & 7];
        }
      }
      if (!KMC_DCHECK(a.err, nsite >= 0 && nsite < a.n_sites)) nsite = site;
      ehops++;
      if (tracing) cold_trace(a, cur - a.films[film].slot0, nsite);
      if (nsite != site) {
        site = nsite;
        at_site = true;
        load_rec(nsite);
      }
      ff = -inv * dlog;
      if (++hs > a.hop_cap) {  // leave this exciton where it is and report
        atomicOr(a.err, KMC_ERR_HOP_CAP_CODE);
        Exciton e;
        e.active = true;
        e.site = site;
        e.heading = heading;
        e.at_site = at_site;
        e.px = cs->p[0];
        e.py = cs->p[1];
        e.pz = cs->p[2];
        e.dx = a.e_delta[cur];
        e.dy = a.e_delta[a.n_slots + cur];
        e.dz = a.e_delta[2 * a.n_slots + cur];
        e.ff = ff;
        e.g.n = rn;
        e.hops = ehops;
        store_exciton(a, cur, e);
        cur = -1;
      }
    } else {
      // ------------------------------------------------ end of step s: fly(rem), ff -= rem, kubo_step tail
      Exciton e;
      e.active = true;
      e.site = site;
      e.heading = heading;
      if (at_site) {
        double4_32a p = a.pos4[site];
        e.px = p.x;
        e.py = p.y;
        e.pz = p.z;
      } else {
        e.px = cs->p[0];
        e.py = cs->p[1];
        e.pz = cs->p[2];
      }
      e.trace_i = tracing ? cur - f.slot0 : -1;
      e.crossings = 0;
      fly_end(a, e, at_site, rem);
      ecross += (uint32_t)e.crossings;
      ff -= rem;
      // update_delta_pos: delta += pos - old_pos, with the step's start in the slot arrays
      const int64_t nsl = a.n_slots;
      double dx = a.e_delta[cur] + (e.px - a.e_pos[cur]);
      double dy = a.e_delta[nsl + cur] + (e.py - a.e_pos[nsl + cur]);
      double dz = a.e_delta[2 * nsl + cur] + (e.pz - a.e_pos[2 * nsl + cur]);
      e.dx = dx;
      e.dy = dy;
      e.dz = dz;
      e.at_site = false;
      e.g.seed = f.seed;
      e.g.stream = (uint64_t)(cur - f.slot0);
      if (avail == 0) {  // the Rng below holds the rest of the current block
        ring.fill(rn, a.films[film].seed, (uint64_t)(cur - a.films[film].slot0));
        avail = 4;
      }
      e.g.n = rn;
      e.g.w0 = ring.word(rn);
      e.g.w1 = ring.word(rn + 1);
      e.g.w2 = ring.word(rn + 2);
      e.g.w3 = ring.word(rn + 3);
      maybe_reinject(a, f, e);
      if (e.g.n != rn) {  // the reinjection drew: restart the ring at the new draw index
        rn = e.g.n;
        ring.fill(rn & ~3ull, a.films[film].seed, (uint64_t)(cur - a.films[film].slot0));
        avail = 4 - (uint32_t)(rn & 3);
      }
      site = e.site;
      heading = e.heading;
      at_site = e.at_site;
      if (single_film) {
        atomicAdd(&s_bins[s * 3 + 0], dx * dx);
        atomicAdd(&s_bins[s * 3 + 1], dy * dy);
        atomicAdd(&s_bins[s * 3 + 2], dz * dz);
      } else if (KMC_DCHECK(a.err, a.step0 + s < a.msd_cap)) {
        const int64_t batch = ((cur - f.slot0) >> 5) % a.msd_batches;
        double* m = a.msd + (((int64_t)film * a.msd_cap + a.step0 + s) * a.msd_batches + batch) * 3;
        atomicAdd(m, dx * dx);
        atomicAdd(m + 1, dy * dy);
        atomicAdd(m + 2, dz * dz);
      }
      ++s;
      if (s == n_steps) {
        e.ff = ff;
        e.hops = ehops;
        store_exciton(a, cur, e);
        lane_hops += ehops;
        lane_cross += ecross;
        cur = -1;
        continue;
      }
      cs->p[0] = e.px;
      cs->p[1] = e.py;
      cs->p[2] = e.pz;
      a.e_pos[cur] = e.px;  // the next step's start
      a.e_pos[nsl + cur] = e.py;
      a.e_pos[2 * nsl + cur] = e.pz;
      a.e_delta[cur] = dx;
      a.e_delta[nsl + cur] = dy;
      a.e_delta[2 * nsl + cur] = dz;
      rem = a.dt;
      hs = 0;
      load_rec(site);
    }
  }
  if (single_film && KMC_DCHECK(a.err, a.step0 + n_steps <= a.msd_cap)) {
    __syncthreads();
    double* m = a.msd + a.step0 * 3;
    for (int64_t i = threadIdx.x; i < n_steps * 3; i += blockDim.x) atomicAdd(m + i, s_bins[i]);
  }
  Exciton e;
  e.hops = lane_hops;
  e.crossings = lane_cross;
  __syncwarp();
  flush_counters(a, e, exact);
}

template <int BLOCK>
static size_t mixed_smem(int64_t n_steps, int single_film) {
  return sizeof(LogTab) + (single_film ? (size_t)(n_steps * 3 + 15) / 16 * 16 * sizeof(double) : 0) +
         BLOCK * (sizeof(ColdState) + 8 * sizeof(uint32_t));
}

// a.hold_short picks the instantiation that batches the ends of short steps
template <int BLOCK, int MINB>
static cudaError_t launch_mixed_t(const HopArgs& a, int64_t n_steps, int grid_blocks, int single_film,
                                  unsigned long long* queue, cudaStream_t s) {
  const size_t smem = mixed_smem<BLOCK>(n_steps, single_film);
  auto kern = a.hold_short ? k_hop_mixed<BLOCK, MINB, true> : k_hop_mixed<BLOCK, MINB, false>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  int64_t need = (a.n_slots + BLOCK - 1) / BLOCK;
  int64_t nb = need < grid_blocks ? need : grid_blocks;
  cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  if (nb) kern<<<(unsigned)nb, BLOCK, smem, s>>>(a, n_steps, queue, single_film);
  return cudaGetLastError();
}

// resident blocks per SM (both instantiations are built for MINB blocks of BLOCK threads)
template <int BLOCK, int MINB>
static int blocks_per_sm_t(int64_t n_steps, int single_film) {
  int nb = 0;
  const size_t smem = mixed_smem<BLOCK>(n_steps, single_film);
  if (smem > 48 * 1024) {
    cudaFuncSetAttribute(k_hop_mixed<BLOCK, MINB, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_hop_mixed<BLOCK, MINB, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  }
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_hop_mixed<BLOCK, MINB, false>, BLOCK, smem) != cudaSuccess)
    return 1;
  return nb > 0 ? nb : 1;
}


}  // namespace kmc
