// kmc_kernels.cu -- CUDA kernels of the exciton-hopping engine (sm_103a).
//
//   K1  cell binning: cell id per site, counting sort into cells, members in site order
//       (create_scatterer_buckets, src/monte_carlo/monte_carlo.h:368-416)
//   K2  neighbour + rate CSR: per site the 27 cells in x-outer / y / z-inner order, members in
//       site order, distance window, pair geometry, table lookup, FP64 inclusive prefix sum
//       (find_neighbors scatterer.cpp:34-83, get_rate scattering_struct.h:38-52,
//        set_max_rate scatterer.h:89-93)
//   init  exciton creation (kubo_create_particles monte_carlo.cpp:308-316, particle.h:48-52)
//   hop   Green-Kubo steps (kubo_step monte_carlo.cpp:319-342, particle::step particle.cpp:57-80,
//         fly :9-54, update_state scatterer.cpp:9-31, ff_time scatterer.h:74-80), MSD sums
//         (kubo_save_avg_dispalcement_squared monte_carlo.cpp:382-409) by warp shuffles.
// The library is compiled with --fmad=false; see kmc_device.cuh for the arithmetic rules.
#include <cstdio>

#include "kmc_internal.h"
#include "kmc_pair.cuh"

namespace kmc {

#define KMC_ERR_HOP_CAP_CODE 1
#define KMC_ERR_CELL_CODE 2
#define KMC_ERR_FLIGHT_CODE 4
// Upper bound of link crossings in one free flight: a flight of length v*dt over links of
// positive length ends long before; only zero-length links (coincident sites) could loop.
constexpr int kMaxCrossings = 1 << 22;

// ============================================================================ K1: cells
__global__ void k_cell_ids(BuildArgs a) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= a.n_sites) return;
  const FilmDev& f = a.films[a.site_film[s]];
  double4_32a p = a.pos4[s];
  // int ix = (s.pos(0) - xmin) / radius;  (monte_carlo.h:390-392; conversion truncates)
  int ix = (int)((p.x - f.mn[0]) / f.r);
  int iy = (int)((p.y - f.mn[1]) / f.r);
  int iz = (int)((p.z - f.mn[2]) / f.r);
  if (ix < 0 || iy < 0 || iz < 0 || ix >= f.nx || iy >= f.ny || iz >= f.nz) {
    atomicOr(a.err, KMC_ERR_CELL_CODE);
    ix = min(max(ix, 0), f.nx - 1);
    iy = min(max(iy, 0), f.ny - 1);
    iz = min(max(iz, 0), f.nz - 1);
  }
  int64_t c = f.cell0 + ix + (int64_t)iy * f.nx + (int64_t)iz * f.nx * f.ny;
  a.cell_of[s] = c;
  atomicAdd((unsigned long long*)&a.cell_start[c], 1ull);
}

__global__ void k_cell_scatter(BuildArgs a) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= a.n_sites) return;
  int64_t c = a.cell_of[s];
  unsigned long long k = atomicAdd((unsigned long long*)&a.cell_cursor[c], 1ull);
  a.cell_members[a.cell_start[c] + (int64_t)k] = (int32_t)s;
}

// members of a cell back into site order (push_back order of monte_carlo.h:389-395)
__global__ void k_cell_sort(BuildArgs a) {
  int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= a.n_cells) return;
  int64_t b = a.cell_start[c], e = a.cell_start[c + 1];
  for (int64_t i = b + 1; i < e; ++i) {
    int32_t v = a.cell_members[i];
    int64_t j = i - 1;
    while (j >= b && a.cell_members[j] > v) {
      a.cell_members[j + 1] = a.cell_members[j];
      --j;
    }
    a.cell_members[j + 1] = v;
  }
}

cudaError_t launch_cell_ids(const BuildArgs& a, cudaStream_t s) {
  int64_t nb = (a.n_sites + 255) / 256;
  if (nb) k_cell_ids<<<(unsigned)nb, 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch_cell_fill(const BuildArgs& a, cudaStream_t s) {
  int64_t nb = (a.n_sites + 255) / 256;
  if (nb) k_cell_scatter<<<(unsigned)nb, 256, 0, s>>>(a);
  int64_t nc = (a.n_cells + 127) / 128;
  if (nc) k_cell_sort<<<(unsigned)nc, 128, 0, s>>>(a);
  return cudaGetLastError();
}

// ============================================================================ K2: neighbour + rate CSR
// Visit the neighbours of site s in find_neighbors order; fn(j, p2, dR, distance) per neighbour.
template <typename F>
__device__ __forceinline__ void for_each_neighbor(const BuildArgs& a, int64_t s, F fn) {
  const FilmDev& f = a.films[a.site_film[s]];
  double4_32a p1 = a.pos4[s];
  int64_t local = a.cell_of[s] - f.cell0;
  int ix = (int)(local % f.nx);
  int iy = (int)((local / f.nx) % f.ny);
  int iz = (int)(local / ((int64_t)f.nx * f.ny));
  for (int i = ix - 1; i <= ix + 1; ++i) {
    if (i < 0 || i >= f.nx) continue;
    for (int j = iy - 1; j <= iy + 1; ++j) {
      if (j < 0 || j >= f.ny) continue;
      for (int k = iz - 1; k <= iz + 1; ++k) {
        if (k < 0 || k >= f.nz) continue;
        int64_t c = f.cell0 + i + (int64_t)j * f.nx + (int64_t)k * f.nx * f.ny;
        for (int64_t m = a.cell_start[c], e = a.cell_start[c + 1]; m < e; ++m) {
          int32_t q = a.cell_members[m];
          double4_32a p2 = a.pos4[q];
          double dR0 = p1.x - p2.x, dR1 = p1.y - p2.y, dR2 = p1.z - p2.z;
          double distance = norm3(dR0, dR1, dR2);
          if ((distance < a.r_max) && (distance > kMinHopDist)) fn(q, p2, dR0, dR1, dR2, distance);
        }
      }
    }
  }
}

__global__ void k_nbr_count(BuildArgs a) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= a.n_sites) return;
  int64_t n = 0;
  for_each_neighbor(a, s, [&](int32_t, const double4_32a&, double, double, double, double) { ++n; });
  a.counts[s] = n;
  atomicMax(&a.stats[0], (unsigned long long)n);
  if (n == 0) atomicAdd(&a.stats[1], 1ull);
}

__global__ void k_nbr_fill(BuildArgs a) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= a.n_sites) return;
  const FilmDev& f = a.films[a.site_film[s]];
  double4_32a p1 = a.pos4[s];
  double a1v[3] = {a.orient[3 * s], a.orient[3 * s + 1], a.orient[3 * s + 2]};
  const int64_t bo = a.blkptr[s];
  double* cump = a.cump + bo * 8;  // this row's FP64 cumulative rates (8 per block)
  int64_t k = 0;
  double run = 0.0;
  bool negative = false;
  for_each_neighbor(a, s, [&](int32_t q, const double4_32a& p2, double dR0, double dR1, double dR2, double distance) {
    double a2v[3] = {a.orient[3 * (int64_t)q], a.orient[3 * (int64_t)q + 1], a.orient[3 * (int64_t)q + 2]};
    double rate = pair_rate(a.table, p1, a1v, p2, a2v, dR0, dR1, dR2, distance);
    negative |= rate < 0;
    run = (k == 0) ? rate : run + rate;  // in-place inclusive prefix sum, scatterer.cpp:78-80
    cump[k] = run;
    a.blocks[bo + (k >> 3)].col[k & 7] = q;
    ++k;
  });
  double tot = k > 0 ? run : 0.0;
  double inv = 1. / tot;
  a.total[s] = tot;
  a.inv_total[s] = inv;
  bool exact = negative || !(tot > 0.0) || !(tot < __longlong_as_double(0x7FF0000000000000ll));
  if (exact && k > 0) atomicAdd(&a.stats[2], 1ull);
  // FP32 normalised values, padding, second and first search levels
  const float kInf = __int_as_float(0x7f800000);
  const int64_t nb = (k + 7) / 8;
  for (int64_t j = 0; j < nb; ++j) {
    RowBlock& blk = a.blocks[bo + j];
    for (int i = 0; i < 8; ++i) {
      int64_t q = 8 * j + i;
      if (q < k) {
        blk.c[i] = exact ? 0.0f : (float)(cump[q] / tot);
      } else {
        blk.c[i] = kInf;
        blk.col[i] = -1;
        cump[q] = __longlong_as_double(0x7FF0000000000000ll);
      }
    }
    int64_t last = min(8 * j + 7, k - 1);
    a.blast[bo + j] = exact ? 0.0f : (float)(cump[last] / tot);
  }
  SiteRec r;
  r.inv_total = inv;
  r.blk = (uint32_t)(bo - f.blk0);
  r.len_flags = (uint32_t)k | (exact ? kRecExact : 0u) | (nb > 64 ? kRecLong : 0u);
  r.left = a.left[s];
  r.right = a.right[s];
  r.lt_hi_l = 0;
  r.lt_hi_r = 0;
  const int64_t G = nb <= 8 ? 1 : (nb + 7) / 8;
  for (int i = 0; i < 8; ++i) {
    if (i * G < nb && !exact) {
      int64_t last = min(8 * G * (i + 1) - 1, k - 1);
      r.coarse[i] = (float)(cump[last] / tot);
    } else {
      r.coarse[i] = kInf;
    }
  }
  a.rec[s] = r;
}

// blocks per row, from the row pointers: blkptr[s] = ceil(len / 8) (scanned afterwards)
__global__ void k_blk_counts(BuildArgs a) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s > a.n_sites) return;
  a.blkptr[s] = s < a.n_sites ? (a.rowptr[s + 1] - a.rowptr[s] + 7) / 8 : 0;
}

cudaError_t launch_blk_counts(const BuildArgs& a, cudaStream_t s) {
  int64_t nb = (a.n_sites + 1 + 255) / 256;
  k_blk_counts<<<(unsigned)nb, 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_nbr_count(const BuildArgs& a, cudaStream_t s) {
  int64_t nb = (a.n_sites + 127) / 128;
  if (nb) k_nbr_count<<<(unsigned)nb, 128, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch_nbr_fill(const BuildArgs& a, cudaStream_t s) {
  int64_t nb = (a.n_sites + 127) / 128;
  if (nb) k_nbr_fill<<<(unsigned)nb, 128, 0, s>>>(a);
  return cudaGetLastError();
}

// link times dist/v to the left and right tube neighbour, dist = norm(pos - next.pos) as in
// fly (particle.cpp:40-42) evaluated at the site's own position
__global__ void k_link_times(const double4_32a* __restrict__ pos4, const int32_t* __restrict__ left,
                             const int32_t* __restrict__ right, SiteRec* rec, double2* lt64, int64_t n, double v) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  double4_32a p = pos4[s];
  double tl = 0, tr = 0;
  int32_t l = left[s], r = right[s];
  if (l >= 0) {
    double4_32a t = pos4[l];
    tl = norm3(p.x - t.x, p.y - t.y, p.z - t.z) / v;
  }
  if (r >= 0) {
    double4_32a t = pos4[r];
    tr = norm3(p.x - t.x, p.y - t.y, p.z - t.z) / v;
  }
  lt64[s] = make_double2(tl, tr);
  rec[s].lt_hi_l = (uint32_t)((uint64_t)__double_as_longlong(tl) >> 32);
  rec[s].lt_hi_r = (uint32_t)((uint64_t)__double_as_longlong(tr) >> 32);
}

cudaError_t launch_link_times(const double4_32a* pos4, const int32_t* left, const int32_t* right, SiteRec* rec,
                              double2* lt64, int64_t n, double v, cudaStream_t s) {
  int64_t nb = (n + 255) / 256;
  if (nb) k_link_times<<<(unsigned)nb, 256, 0, s>>>(pos4, left, right, rec, lt64, n, v);
  return cudaGetLastError();
}

// ============================================================================ scan (int64, exclusive)
constexpr int kScanBlock = 512;
constexpr int kScanItems = 8;
constexpr int64_t kScanTile = (int64_t)kScanBlock * kScanItems;

__global__ void k_scan_tiles(int64_t* data, int64_t n, int64_t* tile_sums) {
  __shared__ int64_t warp_sums[kScanBlock / 32];
  int64_t base = blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t v[kScanItems];
  int64_t sum = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = (base + i < n) ? data[base + i] : 0;
    sum += v[i];
  }
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int64_t inc = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) warp_sums[w] = inc;
  __syncthreads();
  if (w == 0) {
    int64_t ws = lane < kScanBlock / 32 ? warp_sums[lane] : 0;
    int64_t wi = ws;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < kScanBlock / 32) warp_sums[lane] = wi - ws;
    if (lane == kScanBlock / 32 - 1 && tile_sums) tile_sums[blockIdx.x] = wi;
  }
  __syncthreads();
  int64_t run = warp_sums[w] + inc - sum;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) data[base + i] = run;
    run += v[i];
  }
}

__global__ void k_scan_add(int64_t* data, int64_t n, const int64_t* tile_offsets) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  data[i] += tile_offsets[i / kScanTile];
}

int64_t scan_scratch_len(int64_t n) {
  int64_t len = 0;
  while (n > kScanTile) {
    n = (n + kScanTile - 1) / kScanTile;
    len += n;
  }
  return len + 1;
}

cudaError_t exclusive_scan_i64(int64_t* data, int64_t n, int64_t* scratch, int64_t scratch_len, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  int64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles == 1) {
    k_scan_tiles<<<1, kScanBlock, 0, s>>>(data, n, nullptr);
    return cudaGetLastError();
  }
  if (scratch_len < tiles) return cudaErrorInvalidValue;
  k_scan_tiles<<<(unsigned)tiles, kScanBlock, 0, s>>>(data, n, scratch);
  cudaError_t e = exclusive_scan_i64(scratch, tiles, scratch + tiles, scratch_len - tiles, s);
  if (e != cudaSuccess) return e;
  k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(data, n, scratch);
  return cudaGetLastError();
}

// ============================================================================ excitons
__device__ __forceinline__ double dwell(double inv_total, uint32_t r, const LogTab* tab) {
  // ff_time: -(1/Gamma) log(r / RAND_MAX), r != 0 (scatterer.h:74-80)
  return -inv_total * kmc_log((double)r / (double)kRandMax, tab);
}

__global__ void k_init_excitons(HopArgs a) {
  int64_t slot = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (slot >= a.n_slots) return;
  const FilmDev& f = a.films[a.warp_film[slot >> 5]];
  int64_t local = slot - f.slot0;
  const int64_t ns = a.n_slots;
  if (local < 0 || local >= f.n_exc) {
    a.e_site[slot] = -1;
    a.e_flags[slot] = 0;
    a.e_ff[slot] = 0;
    a.e_draws[slot] = 0;
    a.e_hops[slot] = 0;
    for (int c = 0; c < 3; ++c) a.e_pos[c * ns + slot] = a.e_delta[c * ns + slot] = 0;
    return;
  }
  Rng g;
  g.init(f.seed, (uint64_t)local, 0);
  // kubo_create_particles: dice = rand() % n_inject (monte_carlo.cpp:311)
  uint32_t dice = g.next() % (uint32_t)f.n_inj;
  int32_t site = (f.mode == 1) ? (int32_t)(f.site0 + dice) : a.inject[f.inj0 + dice];
  // particle(pos, s, v): ff_time() then heading = rand() % 2 (particle.h:48-52)
  uint32_t r;
  while ((r = g.next()) == 0) {
  }
  double ff = dwell(a.inv_total[site], r, a.logtab);
  uint32_t heading = g.next() % 2;
  double4_32a p = a.pos4[site];
  a.e_site[slot] = site;
  a.e_flags[slot] = kExActive | kExAtSite | (heading ? kExHeading : 0u);
  a.e_pos[0 * ns + slot] = p.x;
  a.e_pos[1 * ns + slot] = p.y;
  a.e_pos[2 * ns + slot] = p.z;
  for (int c = 0; c < 3; ++c) a.e_delta[c * ns + slot] = 0;
  a.e_ff[slot] = ff;
  a.e_draws[slot] = g.n;
  a.e_hops[slot] = 0;
}

cudaError_t launch_init_excitons(const HopArgs& a, cudaStream_t s) {
  int64_t nb = (a.n_slots + 255) / 256;
  if (nb) k_init_excitons<<<(unsigned)nb, 256, 0, s>>>(a);
  return cudaGetLastError();
}

// ============================================================================ hop kernels: shared pieces
struct Exciton {
  int32_t site;
  bool heading, at_site, active;
  double px, py, pz, dx, dy, dz, ff;
  Rng g;
  uint64_t hops, crossings;
  int64_t trace_i;
};

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

__device__ __forceinline__ void load_exciton(const HopArgs& a, int64_t slot, Exciton& e) {
  const int64_t ns = a.n_slots;
  uint32_t fl = a.e_flags[slot];
  e.active = (fl & kExActive) != 0;
  e.heading = (fl & kExHeading) != 0;
  e.at_site = (fl & kExAtSite) != 0;
  e.site = a.e_site[slot];
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
  if ((threadIdx.x & 31) == 0) {
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

// ============================================================================ plain FP64 hop kernel
__global__ void __launch_bounds__(256) k_hop_fp64(HopArgs a, int64_t n_steps) {
  int64_t slot = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (slot >= a.n_slots) return;  // n_slots is a multiple of 32: whole warps leave
  int32_t film = a.warp_film[slot >> 5];
  const FilmDev& f = a.films[film];
  Exciton e;
  load_exciton(a, slot, e);
  int64_t local = slot - f.slot0;
  e.trace_i = (film == 0 && local < a.n_trace) ? local : -1;
  if (e.active) e.g.init(f.seed, (uint64_t)local, a.e_draws[slot]);
  bool dead = false;
  for (int64_t s = 0; s < n_steps; ++s) {
    double ox = e.px, oy = e.py, oz = e.pz;
    if (e.active && !dead) {
      double rem = a.dt;
      int64_t hs = 0;
      while (e.ff <= rem) {  // particle::step, particle.cpp:71-84
        rem -= e.ff;
        fly_full(a, e, e.ff);
        int32_t ns = e.site;
        int64_t n = a.rowptr[e.site + 1] - a.rowptr[e.site];
        if (n > 0) {  // update_state, scatterer.cpp:14-30
          const int64_t bo = a.blkptr[e.site];
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
          dead = true;
          break;
        }
      }
      if (!dead) {
        fly_full(a, e, rem);
        e.ff -= rem;
      }
    }
    step_epilogue(a, f, film, e, ox, oy, oz, s);
  }
  e.at_site = false;
  store_exciton(a, slot, e);
  flush_counters(a, e, 0);
}

cudaError_t launch_hop_fp64(const HopArgs& a, int64_t n_steps, int block, cudaStream_t s) {
  int64_t nb = (a.n_slots + block - 1) / block;
  if (nb) k_hop_fp64<<<(unsigned)nb, block, 0, s>>>(a, n_steps);
  return cudaGetLastError();
}

// ============================================================================ mixed-precision hop kernel
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

// Exact ff <= rem for rem >= +0 and ff not a NaN with the sign bit set (device NaNs are
// positive): non-negative doubles order like their bit patterns, and a negative ff (or -0.0)
// is below every non-negative rem in both orders.
__device__ __forceinline__ bool dwell_fits(double ff, double rem) {
  return __double_as_longlong(ff) <= __double_as_longlong(rem);
}

// Step-boundary state of one lane's exciton, kept in shared memory (one slot per thread): only
// the event loop's hot values stay in registers, which lets more warps stay resident.
struct ColdState {
  double p[3];   // position (valid when not at the site)
  double o[3];   // position at the start of the step
  double d[3];   // Green-Kubo displacement
  uint64_t seed, stream;
  int64_t trace_i;
};

__device__ __forceinline__ void cold_refill(uint64_t n, const ColdState* c, uint32_t& w0, uint32_t& w1, uint32_t& w2,
                                            uint32_t& w3) {
  uint64_t b = n >> 2;
  uint32_t o[4];
  philox4x32_10((uint32_t)b, (uint32_t)(b >> 32), (uint32_t)c->stream, (uint32_t)(c->stream >> 32), (uint32_t)c->seed,
                (uint32_t)(c->seed >> 32), o);
  w0 = o[0];
  w1 = o[1];
  w2 = o[2];
  w3 = o[3];
  for (uint32_t i = 0; i < (uint32_t)(n & 3); ++i) {
    uint32_t t = w0;
    w0 = w1;
    w1 = w2;
    w2 = w3;
    w3 = t;
  }
}

// one draw of the exciton's stream (same sequence as Rng::next)
__device__ __forceinline__ uint32_t cold_next(uint64_t& n, const ColdState* c, uint32_t& w0, uint32_t& w1, uint32_t& w2,
                                              uint32_t& w3) {
  uint32_t v = w0 >> 1;
  ++n;
  if ((n & 3) == 0) {
    cold_refill(n, c, w0, w1, w2, w3);
  } else {
    w0 = w1;
    w1 = w2;
    w2 = w3;
  }
  return v;
}

__device__ __forceinline__ void cold_trace(const HopArgs& a, const ColdState* c, int32_t v) {
  int64_t t = c->trace_i;
  int64_t k = a.trace_cnt[t];
  if (k < a.trace_cap) a.trace[t * a.trace_cap + k] = v;
  a.trace_cnt[t] = k + 1;
}

// Persistent work queue: the grid holds as many threads as the GPU keeps resident; each lane
// takes the next exciton slot from a global counter (warp-aggregated atomics), advances it
// through all n_steps steps of the launch on its own, stores it and takes the next one, so no
// lane waits for another lane's exciton.  MSD sums of a single-film run without batches go to
// block-shared bins (added to global memory once per block); otherwise to global memory.
template <int MINB>
__global__ void __launch_bounds__(128, MINB) k_hop_mixed(HopArgs a, int64_t n_steps, unsigned long long* queue,
                                                         int single_film) {
  extern __shared__ double s_mem[];
  LogTab* s_log = reinterpret_cast<LogTab*>(s_mem);  // the log table, read once per hop
  double* s_bins = s_mem + sizeof(LogTab) / sizeof(double);  // [n_steps][3] when single_film
  ColdState* cs = reinterpret_cast<ColdState*>(s_bins + (single_film ? n_steps * 3 : 0)) + threadIdx.x;
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
  uint32_t w0 = 0, w1 = 0, w2 = 0, w3 = 0;
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
  };
  for (;;) {
    // all 32 lanes meet here once per event, so every event starts with the warp converged
    if (!__any_sync(0xffffffffu, alive)) break;
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
      ff = a.e_ff[cur];
      int64_t local = cur - fp->slot0;
      cs->trace_i = (film == 0 && local < a.n_trace) ? local : -1;
      tracing = cs->trace_i >= 0;
      cs->seed = fp->seed;
      cs->stream = (uint64_t)local;
      rn = a.e_draws[cur];
      cold_refill(rn, cs, w0, w1, w2, w3);
      double px, py, pz;
      if (at_site) {
        double4_32a p = a.pos4[site];
        px = p.x;
        py = p.y;
        pz = p.z;
      } else {
        px = a.e_pos[cur];
        py = a.e_pos[ns + cur];
        pz = a.e_pos[2 * ns + cur];
      }
      cs->p[0] = cs->o[0] = px;
      cs->p[1] = cs->o[1] = py;
      cs->p[2] = cs->o[2] = pz;
      cs->d[0] = a.e_delta[cur];
      cs->d[1] = a.e_delta[ns + cur];
      cs->d[2] = a.e_delta[2 * ns + cur];
      rem = a.dt;
      s = 0;
      hs = 0;
      ehops = 0;
      ecross = 0;
      load_rec(site);
    }
    const FilmDev& f = *fp;
    if (dwell_fits(ff, rem)) {
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
            if (tracing) cold_trace(a, cs, -1 - next);
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
      if (n > 0) {
        uint32_t r = cold_next(rn, cs, w0, w1, w2, w3);
        const RowBlock* __restrict__ rb = a.blocks + f.blk0 + blk;
        bool resolved = false;
        if (!(lenf & (kRecExact | kRecLong))) {
          // two- or three-level search for the first FP32 value > u (count of values <= u)
          float u = __uint2float_rn(r) * (1.0f / 2147483647.0f);
          const float4* cq = reinterpret_cast<const float4*>(recp->coarse);
          float4 q0 = __ldg(cq), q1 = __ldg(cq + 1);
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
      ehops++;
      if (tracing) cold_trace(a, cs, nsite);
      if (nsite != site) {
        site = nsite;
        at_site = true;
        load_rec(nsite);
      }
      uint32_t r;
      while ((r = cold_next(rn, cs, w0, w1, w2, w3)) == 0) {
      }
      ff = -inv * kmc_log_unit(u_from_rand(r), s_log);
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
        e.dx = cs->d[0];
        e.dy = cs->d[1];
        e.dz = cs->d[2];
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
      e.trace_i = cs->trace_i;
      e.crossings = 0;
      fly_full(a, e, rem);
      ecross += (uint32_t)e.crossings;
      ff -= rem;
      double dx = cs->d[0] + (e.px - cs->o[0]);
      double dy = cs->d[1] + (e.py - cs->o[1]);
      double dz = cs->d[2] + (e.pz - cs->o[2]);
      e.dx = dx;
      e.dy = dy;
      e.dz = dz;
      e.at_site = false;
      e.g.seed = cs->seed;
      e.g.stream = cs->stream;
      e.g.n = rn;
      e.g.w0 = w0;
      e.g.w1 = w1;
      e.g.w2 = w2;
      e.g.w3 = w3;
      maybe_reinject(a, f, e);
      rn = e.g.n;
      w0 = e.g.w0;
      w1 = e.g.w1;
      w2 = e.g.w2;
      w3 = e.g.w3;
      site = e.site;
      heading = e.heading;
      at_site = e.at_site;
      if (single_film) {
        atomicAdd(&s_bins[s * 3 + 0], dx * dx);
        atomicAdd(&s_bins[s * 3 + 1], dy * dy);
        atomicAdd(&s_bins[s * 3 + 2], dz * dz);
      } else {
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
      cs->p[0] = cs->o[0] = e.px;
      cs->p[1] = cs->o[1] = e.py;
      cs->p[2] = cs->o[2] = e.pz;
      cs->d[0] = dx;
      cs->d[1] = dy;
      cs->d[2] = dz;
      rem = a.dt;
      hs = 0;
      load_rec(site);
    }
  }
  if (single_film) {
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

template <int MINB>
static cudaError_t launch_mixed_t(const HopArgs& a, int64_t n_steps, int grid_blocks, int single_film,
                                  unsigned long long* queue, cudaStream_t s) {
  const int block = 128;
  size_t smem = sizeof(LogTab) + (single_film ? (size_t)n_steps * 3 * sizeof(double) : 0) + block * sizeof(ColdState);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_hop_mixed<MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  int64_t need = (a.n_slots + block - 1) / block;
  int64_t nb = need < grid_blocks ? need : grid_blocks;
  cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  if (nb) k_hop_mixed<MINB><<<(unsigned)nb, block, smem, s>>>(a, n_steps, queue, single_film);
  return cudaGetLastError();
}

template <int MINB>
static int blocks_per_sm_t(int64_t n_steps, int single_film) {
  int nb = 0;
  size_t smem = sizeof(LogTab) + (single_film ? (size_t)n_steps * 3 * sizeof(double) : 0) + 128 * sizeof(ColdState);
  if (smem > 48 * 1024) cudaFuncSetAttribute(k_hop_mixed<MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_hop_mixed<MINB>, 128, smem) != cudaSuccess) return 1;
  return nb > 0 ? nb : 1;
}

// variant: 0, 1, 2 -> kernels compiled for at least 4, 6, 8 resident blocks of 128 threads per SM
cudaError_t launch_hop_mixed(const HopArgs& a, int64_t n_steps, int variant, int grid_blocks, int single_film,
                             unsigned long long* queue, cudaStream_t s) {
  switch (variant) {
    case 1: return launch_mixed_t<6>(a, n_steps, grid_blocks, single_film, queue, s);
    case 2: return launch_mixed_t<8>(a, n_steps, grid_blocks, single_film, queue, s);
    default: return launch_mixed_t<4>(a, n_steps, grid_blocks, single_film, queue, s);
  }
}

int hop_mixed_blocks_per_sm(int variant, int64_t n_steps, int single_film) {
  switch (variant) {
    case 1: return blocks_per_sm_t<6>(n_steps, single_film);
    case 2: return blocks_per_sm_t<8>(n_steps, single_film);
    default: return blocks_per_sm_t<4>(n_steps, single_film);
  }
}

// ============================================================================ self-checks
// u_from_rand against IEEE division for r in [r0, r0 + count)
__global__ void k_u_check(uint32_t r0, uint64_t count, unsigned long long* mism) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  unsigned long long bad = 0;
  for (; i < count; i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t r = r0 + (uint32_t)i;
    if (r == 0) continue;
    double a = u_from_rand(r), b = (double)r / (double)kRandMax;
    bad += (__double_as_longlong(a) != __double_as_longlong(b));
  }
  if (bad) atomicAdd(mism, bad);
}

cudaError_t launch_u_check(uint32_t r0, uint64_t count, unsigned long long* mismatches, cudaStream_t s) {
  k_u_check<<<152 * 8, 256, 0, s>>>(r0, count, mismatches);
  return cudaGetLastError();
}

__global__ void k_math_probe(const double* x, double* lo, double* ao, int64_t n, const LogTab* tab) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  lo[i] = kmc_log(x[i], tab);
  ao[i] = kmc_acos(x[i]);
}

cudaError_t launch_math_probe(const double* x, double* log_out, double* acos_out, int64_t n, const LogTab* tab,
                              cudaStream_t s) {
  int64_t nb = (n + 255) / 256;
  if (nb) k_math_probe<<<(unsigned)nb, 256, 0, s>>>(x, log_out, acos_out, n, tab);
  return cudaGetLastError();
}

}  // namespace kmc
