// kmc_contacts.cu -- contacts (steady-state flux) mode: the reference's second driver
// (src/main.cpp:85-106 on mc::monte_carlo, src/monte_carlo/monte_carlo.h):
//
//   init        create_particles (monte_carlo.h:274-316): a linear profile of excitons over the
//               y segments, each at a random site of its segment
//   step        the hop kernels with nothing removed (step :343-354 = particle::step per exciton)
//   metrics     save_population_profile (:525-581): excitons per y segment; save_currents
//               (:584-643): net crossings of each segment interface during the step
//   repopulate  repopulate_contacts (:443-491): excitons in the contact-1 slab are removed and
//               contact_pop[0] new ones placed at random contact-1 sites; then the same for the
//               last segment
//   track       track_particle (:786-818): single excitons walked from contact 1 to the last
//               slab, one thread each
//
// The reference keeps a vector of particles; here excitons live in slots.  Slot k draws from
// Philox stream k, and its draw counter carries on when its exciton is removed and a new one is
// placed in the slot.  The n new excitons of a contact take the n lowest empty slots, in order
// (a block count, its exclusive scan and a block rank).  Segment and interface counts are
// integers, so their order of summation does not matter: they equal the reference's counts.
#include "kmc_internal.h"
#include "kmc_hop_common.cuh"

namespace kmc {

constexpr int kCBlock = 256;

int64_t contacts_blocks(int64_t n_slots) { return (n_slots + kCBlock - 1) / kCBlock; }

// Exclusive rank of `flag` among the block's threads; *total = the block's count.  Every thread
// of the block calls it.
__device__ __forceinline__ int block_rank(bool flag, int* total) {
  __shared__ int wsum[kCBlock / 32];
  const unsigned m = __ballot_sync(0xffffffffu, flag);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) wsum[w] = __popc(m);
  __syncthreads();
  int before = 0, tot = 0;
#pragma unroll
  for (int k = 0; k < kCBlock / 32; ++k) {
    const int v = wsum[k];
    before += k < w ? v : 0;
    tot += v;
  }
  __syncthreads();
  *total = tot;
  return before + __popc(m & ((1u << lane) - 1u));
}

// particle(site pos, site, v) at a random site of `list` (the dice of create_particles :306 and
// repopulate :480,486; the constructor's ff_time and heading, particle.h:48-52), drawing from the
// slot's stream from draw n0 on.
__device__ void create_exciton(const ContactArgs& a, int64_t s, uint64_t n0, const int32_t* list, int64_t n_list) {
  Rng g;
  g.init(a.seed, (uint64_t)s, n0);
  const uint32_t dice = g.next() % (uint32_t)n_list;
  const int32_t site = list[dice];
  uint32_t r;
  while ((r = g.next()) == 0) {
  }
  const double ff = dwell(a.inv_total[site], r, a.logtab);
  const uint32_t heading = g.next() % 2;
  const double4_32a p = a.pos4[site];
  const int64_t ns = a.n_slots;
  a.e_site[s] = site;
  a.e_flags[s] = kExActive | kExAtSite | (heading ? kExHeading : 0u);
  a.e_pos[s] = p.x;
  a.e_pos[ns + s] = p.y;
  a.e_pos[2 * ns + s] = p.z;
  for (int c = 0; c < 3; ++c) a.e_delta[c * ns + s] = 0.0;
  a.e_ff[s] = ff;
  a.e_draws[s] = g.n;
}

__device__ __forceinline__ void empty_slot(const ContactArgs& a, int64_t s) {
  a.e_flags[s] = 0;
  a.e_site[s] = -1;
}

__global__ void __launch_bounds__(kCBlock) k_contacts_init(ContactArgs a, const int32_t* __restrict__ seg_sites,
                                                           const int64_t* __restrict__ seg_off,
                                                           const int64_t* __restrict__ part_first, int64_t n_initial) {
  const int64_t s = blockIdx.x * (int64_t)kCBlock + threadIdx.x;
  const int64_t ns = a.n_slots;
  if (s >= ns) return;
  empty_slot(a, s);
  a.e_ff[s] = 0;
  a.e_draws[s] = 0;
  a.e_hops[s] = 0;
  for (int c = 0; c < 3; ++c) a.e_pos[c * ns + s] = a.e_delta[c * ns + s] = 0.0;
  a.y_old[s] = 0.0;
  if (s >= n_initial) return;
  // the segment of exciton s: the last segment whose first exciton is <= s (empty segments
  // share their start with the next one)
  int lo = 0, hi = a.n_seg;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (part_first[mid] <= s)
      lo = mid;
    else
      hi = mid;
  }
  create_exciton(a, s, 0, seg_sites + seg_off[lo], seg_off[lo + 1] - seg_off[lo]);
  a.y_old[s] = a.e_pos[ns + s];
}

// number of interfaces at or below v (the interface positions do not decrease)
__device__ __forceinline__ int interfaces_below(const double* __restrict__ t, int m, double v) {
  int lo = 0, hi = m;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (t[mid] <= v)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

// The step's metrics over the live excitons, then the contact-1 removal and the empty-slot
// count of every block.
//   segment: i = int((y - ymin) / dy) clamped to [0, n_seg)      (monte_carlo.h:569-570)
//   interface k (y_k = ymin + dy (k + 1)): +1 if old < y_k <= y, -1 if y < y_k <= old (:628-636);
//   the interfaces crossed form one index range, added to a difference array.
__global__ void __launch_bounds__(kCBlock) k_contacts_metrics(ContactArgs a) {
  extern __shared__ int csh[];
  int* spop = csh;
  int* sdiff = csh + a.n_seg;
  for (int i = threadIdx.x; i < 2 * a.n_seg; i += kCBlock) csh[i] = 0;
  __syncthreads();
  const int64_t step = *a.step;
  const int64_t s = blockIdx.x * (int64_t)kCBlock + threadIdx.x;
  const int64_t ns = a.n_slots;
  bool live = false;
  if (s < ns && (a.e_flags[s] & kExActive)) {
    const double y = a.e_pos[ns + s], yo = a.y_old[s];
    int i = (int)((y - a.ymin) / a.dy);
    i = i < 0 ? 0 : (i < a.n_seg ? i : a.n_seg - 1);
    atomicAdd(&spop[i], 1);
    if (y == y && yo == yo) {
      const int lo = interfaces_below(a.y_if, a.n_seg - 1, yo), hi = interfaces_below(a.y_if, a.n_seg - 1, y);
      if (hi != lo) {
        const int sg = hi > lo ? 1 : -1;
        atomicAdd(&sdiff[min(lo, hi)], sg);
        atomicAdd(&sdiff[max(lo, hi)], -sg);
      }
    }
    live = !(y >= a.rem_y1[0] && y <= a.rem_y2[0]);  // repopulate :465
    if (!live) empty_slot(a, s);
  }
  int total;
  block_rank(s < ns && !live, &total);
  if (threadIdx.x == 0) {
    a.blk_a[blockIdx.x] = total;
    if (blockIdx.x == 0) a.blk_a[gridDim.x] = 0;
  }
  __syncthreads();
  if (!KMC_DCHECK(a.err, step < a.steps_cap)) return;  // after the block's last barrier
  for (int i = threadIdx.x; i < a.n_seg; i += kCBlock) {
    if (spop[i]) atomicAdd(&a.pop[step * a.n_seg + i], (unsigned long long)spop[i]);
    if (sdiff[i]) atomicAdd(&a.diff[step * a.n_seg + i], (unsigned long long)(long long)sdiff[i]);
  }
}

// Contact c's new excitons into the lowest empty slots (blk = scanned empty counts per block).
// c = 0: then the contact-n removal and the next empty-slot count.  c = 1: then the start
// positions of the next step and the live count.
__global__ void __launch_bounds__(kCBlock) k_contacts_place(ContactArgs a, int c) {
  const int64_t s = blockIdx.x * (int64_t)kCBlock + threadIdx.x;
  const int64_t ns = a.n_slots;
  const int64_t* blk = c == 0 ? a.blk_a : a.blk_b;
  bool live = s < ns && (a.e_flags[s] & kExActive);
  int total;
  const int r = block_rank(s < ns && !live, &total);
  if (s < ns && !live && blk[blockIdx.x] + r < a.c_pop[c]) {
    create_exciton(a, s, a.e_draws[s], a.c_list[c], a.c_n[c]);
    live = true;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && blk[gridDim.x] < a.c_pop[c]) atomicOr(a.err, KMC_ERR_CAPACITY_CODE);
  if (c == 0) {
    if (live) {
      const double y = a.e_pos[ns + s];
      if (y >= a.rem_y1[1] && y <= a.rem_y2[1]) {
        empty_slot(a, s);
        live = false;
      }
    }
    block_rank(s < ns && !live, &total);
    if (threadIdx.x == 0) {
      a.blk_b[blockIdx.x] = total;
      if (blockIdx.x == 0) a.blk_b[gridDim.x] = 0;
    }
  } else {
    if (live) a.y_old[s] = a.e_pos[ns + s];
    block_rank(live, &total);
    if (threadIdx.x == 0 && total && KMC_DCHECK(a.err, *a.step < a.steps_cap))
      atomicAdd(&a.n_live[*a.step], (unsigned long long)total);
  }
}

__global__ void k_contacts_next(int64_t* step) { *step += 1; }

// track_particle (monte_carlo.h:786-818): one exciton placed at a random contact-1 site
// (repopulate into an empty list), stepped until its y reaches the last slab, its position
// recorded after every step.  Track k draws from Philox stream kTrackStream0 + k.
__global__ void k_contacts_track(HopArgs h, ContactArgs a, int64_t first, int32_t n_tracks, int64_t max_steps,
                                 double* __restrict__ path, int64_t* __restrict__ len, int32_t* __restrict__ arrived) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_tracks) return;
  Exciton e{};
  e.active = true;
  e.trace_i = -1;
  e.g.init(a.seed, kTrackStream0 + (uint64_t)(first + k), 0);
  const uint32_t dice = e.g.next() % (uint32_t)a.c_n[0];
  e.site = a.c_list[0][dice];
  uint32_t r;
  while ((r = e.g.next()) == 0) {
  }
  e.ff = dwell(a.inv_total[e.site], r, a.logtab);
  e.heading = (e.g.next() % 2) != 0;
  const double4_32a p = a.pos4[e.site];
  e.px = p.x;
  e.py = p.y;
  e.pz = p.z;
  const double y_end = a.rem_y1[1];  // ymin + (n_seg - 1) dy
  int64_t n = 0;
  double* out = path + (int64_t)k * max_steps * 3;
  while (e.py < y_end && n < max_steps) {
    if (!step_fp64(h, e, h.dt)) break;
    out[3 * n] = e.px;
    out[3 * n + 1] = e.py;
    out[3 * n + 2] = e.pz;
    ++n;
  }
  len[k] = n;
  arrived[k] = e.py < y_end ? 0 : 1;
}

cudaError_t launch_contacts_track(const HopArgs& h, const ContactArgs& a, int64_t first, int32_t n_tracks,
                                  int64_t max_steps, double* path, int64_t* len, int32_t* arrived, cudaStream_t s) {
  if (n_tracks > 0)
    k_contacts_track<<<(unsigned)((n_tracks + 63) / 64), 64, 0, s>>>(h, a, first, n_tracks, max_steps, path, len, arrived);
  return cudaGetLastError();
}

cudaError_t launch_contacts_init(const ContactArgs& a, const int32_t* seg_sites, const int64_t* seg_off,
                                 const int64_t* part_first, int64_t n_initial, cudaStream_t s) {
  const int64_t nb = contacts_blocks(a.n_slots);
  if (nb) k_contacts_init<<<(unsigned)nb, kCBlock, 0, s>>>(a, seg_sites, seg_off, part_first, n_initial);
  return cudaGetLastError();
}

int contacts_kernel_count(int64_t n_slots) { return 4 + 2 * scan_kernel_count(contacts_blocks(n_slots) + 1); }

cudaError_t enqueue_contacts_step(const ContactArgs& a, int64_t* scan_scratch, int64_t scratch_len, cudaStream_t s) {
  const int64_t nb = contacts_blocks(a.n_slots);
  cudaError_t e;
  k_contacts_metrics<<<(unsigned)nb, kCBlock, 2 * a.n_seg * sizeof(int), s>>>(a);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = exclusive_scan_i64(a.blk_a, nb + 1, scan_scratch, scratch_len, s)) != cudaSuccess) return e;
  k_contacts_place<<<(unsigned)nb, kCBlock, 0, s>>>(a, 0);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = exclusive_scan_i64(a.blk_b, nb + 1, scan_scratch, scratch_len, s)) != cudaSuccess) return e;
  k_contacts_place<<<(unsigned)nb, kCBlock, 0, s>>>(a, 1);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  k_contacts_next<<<1, 1, 0, s>>>(a.step);
  return cudaGetLastError();
}

}  // namespace kmc
