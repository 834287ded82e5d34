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
#include "kmc_hop_common.cuh"

namespace kmc {

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

// FP32 copy of the positions for the neighbour screen
__global__ void k_pos_f32(const double4_32a* __restrict__ p, float4* __restrict__ out, int64_t n) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const double4_32a v = p[s];
  out[s] = make_float4((float)v.x, (float)v.y, (float)v.z, 0.f);
}

__global__ void k_orient_f32(const double* __restrict__ o, float4* __restrict__ out, int64_t n) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  out[s] = make_float4((float)o[3 * s], (float)o[3 * s + 1], (float)o[3 * s + 2], 0.f);
}

cudaError_t launch_orient_f32(const double* orient, float4* out, int64_t n, cudaStream_t s) {
  const int64_t nb = (n + 255) / 256;
  if (nb) k_orient_f32<<<(unsigned)nb, 256, 0, s>>>(orient, out, n);
  return cudaGetLastError();
}

__global__ void k_load_sites(int64_t n, int32_t n_films, const int64_t* __restrict__ off, const double* __restrict__ pos,
                             const int32_t* __restrict__ lloc, const int32_t* __restrict__ rloc, double4_32a* pos4,
                             int32_t* left, int32_t* right, int32_t* site_film, unsigned long long* bad) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  int lo = 0, hi = n_films;  // the film f with off[f] <= s < off[f + 1]
  while (hi - lo > 1) {
    const int mid = (lo + hi) / 2;
    if (off[mid] <= s)
      lo = mid;
    else
      hi = mid;
  }
  const int64_t s0 = off[lo], ns = off[lo + 1] - s0;
  const int32_t l = lloc[s], r = rloc[s];
  if (l < -1 || r < -1 || l >= ns || r >= ns) atomicMin(bad, (unsigned long long)s);
  left[s] = l < 0 ? -1 : (int32_t)(s0 + l);
  right[s] = r < 0 ? -1 : (int32_t)(s0 + r);
  site_film[s] = lo;
  pos4[s] = make_double4_32a(pos[3 * s], pos[3 * s + 1], pos[3 * s + 2], 0.0);
}

cudaError_t launch_load_sites(int64_t n, int32_t n_films, const int64_t* offsets, const double* pos,
                              const int32_t* left_local, const int32_t* right_local, double4_32a* pos4,
                              int32_t* left, int32_t* right, int32_t* site_film, unsigned long long* bad_site,
                              cudaStream_t s) {
  const int64_t nb = (n + 255) / 256;
  if (nb) k_load_sites<<<(unsigned)nb, 256, 0, s>>>(n, n_films, offsets, pos, left_local, right_local, pos4, left,
                                                       right, site_film, bad_site);
  return cudaGetLastError();
}

cudaError_t launch_pos_f32(const double4_32a* p, float4* out, int64_t n, cudaStream_t s) {
  int64_t nb = (n + 255) / 256;
  if (nb) k_pos_f32<<<(unsigned)nb, 256, 0, s>>>(p, out, n);
  return cudaGetLastError();
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

// ============================================================================ storage order of the sites
// Sites are stored in spatial order: cells of each film in tiles of kOrderTile x kOrderTile
// columns (x fastest inside a tile, tiles row by row), z innermost, the members of a cell in
// reference order.  Every site-indexed array the hop kernels read (records, row blocks, positions,
// links) is laid out in this order, so a compact region of the film is a compact range of
// memory; reference ids are translated at the boundary (perm: slot -> id, rank: id -> slot).
__device__ __forceinline__ int64_t tile_bucket(const FilmDev& f, int64_t local_cell) {
  const int64_t ix = local_cell % f.nx, iy = (local_cell / f.nx) % f.ny, iz = local_cell / ((int64_t)f.nx * f.ny);
  const int64_t ntx = (f.nx + kOrderTile - 1) / kOrderTile;
  const int64_t tile = (iy / kOrderTile) * ntx + ix / kOrderTile;
  return ((tile * kOrderTile + iy % kOrderTile) * kOrderTile + ix % kOrderTile) * f.nz + iz;
}

__device__ __forceinline__ int32_t film_of_cell(const FilmDev* films, int32_t n_films, int64_t c) {
  int32_t lo = 0, hi = n_films - 1;
  while (lo < hi) {
    int32_t mid = (lo + hi + 1) / 2;
    if (films[mid].cell0 <= c) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void k_site_order_sizes(BuildArgs a, const int64_t* __restrict__ ord0, int64_t* __restrict__ sizes) {
  int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= a.n_cells) return;
  const int32_t film = film_of_cell(a.films, a.n_films, c);
  const FilmDev& f = a.films[film];
  sizes[ord0[film] + tile_bucket(f, c - f.cell0)] = a.cell_start[c + 1] - a.cell_start[c];
}

__global__ void k_site_order_fill(BuildArgs a, const int64_t* __restrict__ ord0, const int64_t* __restrict__ start) {
  int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= a.n_cells) return;
  const int32_t film = film_of_cell(a.films, a.n_films, c);
  const FilmDev& f = a.films[film];
  int64_t at = start[ord0[film] + tile_bucket(f, c - f.cell0)];
  for (int64_t m = a.cell_start[c], e = a.cell_start[c + 1]; m < e; ++m, ++at) {
    const int32_t s = a.cell_members[m];
    a.perm[at] = s;
    a.rank[s] = (int32_t)at;
  }
}

cudaError_t build_site_order(const BuildArgs& a, const int64_t* ord0, int64_t n_buckets, int64_t* sizes,
                             int64_t* scan_scratch, int64_t scratch_len, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(sizes, 0, (n_buckets + 1) * sizeof(int64_t), s);
  if (e != cudaSuccess) return e;
  const int64_t nb = (a.n_cells + 255) / 256;
  if (nb == 0) return cudaSuccess;
  k_site_order_sizes<<<(unsigned)nb, 256, 0, s>>>(a, ord0, sizes);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = exclusive_scan_i64(sizes, n_buckets + 1, scan_scratch, scratch_len, s)) != cudaSuccess) return e;
  k_site_order_fill<<<(unsigned)nb, 256, 0, s>>>(a, ord0, sizes);
  return cudaGetLastError();
}

// ids[k] <- rank[ids[k]] (reference ids to storage slots)
__global__ void k_ids_to_slots(int32_t* ids, int64_t n, const int32_t* __restrict__ rank) {
  int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < n) ids[k] = rank[ids[k]];
}

cudaError_t ids_to_slots(int32_t* ids, int64_t n, const int32_t* rank, cudaStream_t s) {
  const int64_t nb = (n + 255) / 256;
  if (nb) k_ids_to_slots<<<(unsigned)nb, 256, 0, s>>>(ids, n, rank);
  return cudaGetLastError();
}

// ============================================================================ K2: neighbour + rate CSR
// Visit the neighbours of site s in find_neighbors order; fn(j) per neighbour (reference id).
// Candidates are screened with FP32 squared distances: a candidate clear of both window edges
// (0.4 nm, r) by the screen's error bound is in or out without FP64 work; only those within
// the bound of an edge take the reference's FP64 test, on the squared distance against the
// window's squared bounds (no root), so the neighbour set is exact.
// The FP64 window test of a pair the FP32 screen left undecided, out of line: it runs for a
// few candidates in 10^4, and the screen loop runs several times faster without FP64 code in it.
static __device__ __noinline__ bool in_window_fp64(const BuildArgs& a, int64_t s, int32_t q) {
  const double4_32a p1 = a.pos4[s], p2 = a.pos4[q];
  const double dR0 = p1.x - p2.x, dR1 = p1.y - p2.y, dR2 = p1.z - p2.z;
  const double e2 = dot3(dR0, dR1, dR2, dR0, dR1, dR2);  // norm3's sum, before its root
  return e2 < a.win_hi2 && e2 > a.win_lo2;
}

// kOutline: the FP64 test as a call (the counting pass, whose loop is otherwise FP64-free and
// runs ~2.8x faster so); inline in the filling pass, whose FP64 rate code makes a call in the
// loop cost more than it saves.
template <bool kOutline, typename F>
__device__ __forceinline__ void for_each_neighbor(const BuildArgs& a, int64_t s, F fn) {
  const FilmDev& f = a.films[a.site_film[s]];
  const float4 p1f = a.pos4f[s];
  // the film's cell grid in 32-bit indices (fewer than 2^31 cells per film)
  const int nx = f.nx, ny = f.ny, nz = f.nz;
  const int64_t* __restrict__ cstart = a.cell_start + f.cell0;
  const int local = (int)(a.cell_of[s] - f.cell0);
  const int ix = local % nx;
  const int iy = (local / nx) % ny;
  const int iz = local / (nx * ny);
  for (int i = ix - 1; i <= ix + 1; ++i) {
    if (i < 0 || i >= nx) continue;
    for (int j = iy - 1; j <= iy + 1; ++j) {
      if (j < 0 || j >= ny) continue;
      for (int k = iz - 1; k <= iz + 1; ++k) {
        if (k < 0 || k >= nz) continue;
        const int lc = i + j * nx + k * nx * ny;
        const int64_t m0 = cstart[lc];
        const int nm = (int)(cstart[lc + 1] - m0);
        const int32_t* __restrict__ cm = a.cell_members + m0;
        for (int t = 0; t < nm; ++t) {
          const int32_t q = cm[t];
          const float4 p2f = a.pos4f[q];
          const float fx = p1f.x - p2f.x, fy = p1f.y - p2f.y, fz = p1f.z - p2f.z;
          const float d2 = fx * fx + fy * fy + fz * fz;
          if (d2 >= a.scr.out_hi2 || d2 <= a.scr.out_lo2) continue;  // surely outside the window
          if (!(d2 < a.scr.in_hi2 && d2 > a.scr.in_lo2)) {  // not surely inside
            if (kOutline) {
              if (!in_window_fp64(a, s, q)) continue;
            } else {
              const double4_32a p1 = a.pos4[s], p2 = a.pos4[q];
              const double dR0 = p1.x - p2.x, dR1 = p1.y - p2.y, dR2 = p1.z - p2.z;
              const double e2 = dot3(dR0, dR1, dR2, dR0, dR1, dR2);
              if (!(e2 < a.win_hi2 && e2 > a.win_lo2)) continue;
            }
          }
          fn(q);
        }
      }
    }
  }
}

// Both passes take the sites in storage order (thread i: site perm[i]), so the threads of a warp
// scan the same cells and write neighbouring rows.
// The longest row and the empty rows are reduced over the warp first: one atomic per warp, not
// one per site on the same two words.
__global__ void k_nbr_count(BuildArgs a) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool live = i < a.n_sites;
  unsigned n = 0;
  if (live) {
    const int64_t s = a.perm[i];
    for_each_neighbor<true>(a, s, [&](int32_t) { ++n; });
    a.counts[s] = n;
  }
  const unsigned m = __activemask();
  const unsigned kmax = __reduce_max_sync(m, n);
  const unsigned empty = __popc(__ballot_sync(m, live && n == 0));
  if ((threadIdx.x & 31) == __ffs(m) - 1) {
    atomicMax(&a.stats[0], (unsigned long long)kmax);
    if (empty) atomicAdd(&a.stats[1], (unsigned long long)empty);
  }
}

// Row of site s (reference id) into storage slot rank[s]; neighbour ids and links are stored as
// storage slots, so the hop kernels never translate ids.  Two phases: the screen collects the
// neighbours' reference ids in list order into the row's id slots, then the FP64 pair geometry
// runs over that list, so the lanes of a warp do their FP64 work together instead of only on
// the candidates each happens to accept.
__global__ void k_nbr_fill(BuildArgs a) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= a.n_sites) return;
  const int64_t s = a.perm[i];
  const FilmDev& f = a.films[a.site_film[s]];
  double4_32a p1 = a.pos4[s];
  double a1v[3] = {a.orient[3 * s], a.orient[3 * s + 1], a.orient[3 * s + 2]};
  const int64_t si = i;  // the row's storage slot (rank[s])
  const int64_t bo = a.blkptr[si];
  double* cump = a.cump + bo * 8;  // this row's FP64 cumulative rates (8 per block)
  int64_t k = 0;
  for_each_neighbor<false>(a, s, [&](int32_t q) {
    a.blocks[bo + (k >> 3)].col[k & 7] = q;
    ++k;
  });
  // Pass 1: every entry's rate into its cump slot.  With the FP32 lookup (2-D tables), a pair
  // clear of its cell's widened bounds takes the entry the FP64 lookup would take, without FP64
  // work; the few others are listed for pass 2, so that a warp runs the FP64 lookup a few times
  // per row instead of on every entry some lane could not decide.
  const bool f32 = a.d2_above_f != nullptr;
  constexpr int kUndecided = 8;
  int32_t undecided[kUndecided];
  int n_und = 0;
  bool all = !f32;  // FP64 for every entry (no FP32 lookup, or the list overflowed)
  if (f32) {
    const float4 p1f = a.pos4f[s], o1f = a.orient4f[s];
    const int n0 = a.table.n[0], n1 = a.table.n[1];
    for (int64_t j = 0; j < k; ++j) {
      const int32_t q = a.blocks[bo + (j >> 3)].col[j & 7];
      const float4 p2f = a.pos4f[q], o2f = a.orient4f[q];
      const float fx = p1f.x - p2f.x, fy = p1f.y - p2f.y, fz = p1f.z - p2f.z;
      const float d2f = fx * fx + fy * fy + fz * fz;
      const float acf = fabsf(o1f.x * o2f.x + o1f.y * o2f.y + o1f.z * o2f.z);
      int c0 = (int)floorf((sqrtf(d2f) - a.table.g0f[0]) * a.table.ihf[0] + 0.5f);
      c0 = c0 < 0 ? 0 : (c0 > n0 - 1 ? n0 - 1 : c0);
      int c1 = (int)floorf((acosf(fminf(acf, 1.f)) - a.table.g0f[1]) * a.table.ihf[1] + 0.5f);
      c1 = c1 < 0 ? 0 : (c1 > n1 - 1 ? n1 - 1 : c1);
      // |cos theta| above the first angle bound: angle index 0 on both FP64 paths (the fast one,
      // and the exact one that parallel pairs with |cos| > 1 by rounding take)
      if ((c0 == 0 || d2f > a.d2_above_f[c0 - 1]) && (c0 == n0 - 1 || d2f < a.d2_below_f[c0]) &&
          (c1 == 0 || acf < a.cos_below_f[c1 - 1]) && (c1 == n1 - 1 || acf > a.cos_above_f[c1])) {
        cump[j] = a.table.rate[pair_table(a.table, s, q) + (int64_t)c0 * n1 + c1];
      } else if (n_und < kUndecided) {
        undecided[n_und++] = (int32_t)j;
      } else {
        all = true;
      }
    }
  }
  // Pass 2: the FP64 lookup (pair geometry in the reference's operations) for the listed
  // entries, or for every entry
  const int64_t n2 = all ? k : n_und;
  for (int64_t t = 0; t < n2; ++t) {
    const int64_t j = all ? t : undecided[t];
    const int32_t q = a.blocks[bo + (j >> 3)].col[j & 7];
    const double4_32a p2 = a.pos4[q];
    const double dR0 = p1.x - p2.x, dR1 = p1.y - p2.y, dR2 = p1.z - p2.z;
    double a2v[3] = {a.orient[3 * (int64_t)q], a.orient[3 * (int64_t)q + 1], a.orient[3 * (int64_t)q + 2]};
    if (a.table.kind != 4) {
      cump[j] = pair_rate_2d(a.table, a1v, a2v, dR0, dR1, dR2, pair_table(a.table, s, q), p1, p2);
    } else {
      const double distance = norm3(dR0, dR1, dR2);
      cump[j] = pair_rate(a.table, p1, a1v, p2, a2v, dR0, dR1, dR2, distance, pair_table(a.table, s, q));
    }
  }
  // Pass 3: the running sum in list order (scatterer.cpp:78-80) and the neighbours as storage slots
  double run = 0.0;
  bool negative = false;
  for (int64_t j = 0; j < k; ++j) {
    const double rate = cump[j];
    negative |= rate < 0;
    run = (j == 0) ? rate : run + rate;
    cump[j] = run;
    a.blocks[bo + (j >> 3)].col[j & 7] = a.rank[a.blocks[bo + (j >> 3)].col[j & 7]];
  }
  double tot = k > 0 ? run : 0.0;
  double inv = 1. / tot;
  a.total[si] = tot;
  a.inv_total[si] = inv;
  bool exact = negative || !(tot > 0.0) || !(tot < __longlong_as_double(0x7FF0000000000000ll));
  if (exact && k > 0) atomicAdd(&a.stats[2], 1ull);
  // FP32 normalised values, padding, second and first search levels.  cum * (1/total) instead of
  // cum / total: within 2^-52 of the quotient before the FP32 rounding (the mixed kernel's
  // margins are 2^-20), monotone along the row, and one FP64 multiply instead of a division
  const float kInf = __int_as_float(0x7f800000);
  const int64_t nb = (k + 7) / 8;
  for (int64_t j = 0; j < nb; ++j) {
    RowBlock& blk = a.blocks[bo + j];
    for (int i = 0; i < 8; ++i) {
      int64_t q = 8 * j + i;
      if (q < k) {
        blk.c[i] = exact ? 0.0f : (float)(cump[q] * inv);
      } else {
        blk.c[i] = kInf;
        blk.col[i] = -1;
        cump[q] = __longlong_as_double(0x7FF0000000000000ll);
      }
    }
    int64_t last = min(8 * j + 7, k - 1);
    a.blast[bo + j] = exact ? 0.0f : (float)(cump[last] * inv);
  }
  SiteRec r;
  r.inv_total = inv;
  r.blk = (uint32_t)(bo - f.blk0);
  r.len_flags = (uint32_t)k | (exact ? kRecExact : 0u) | (nb > 64 ? kRecLong : 0u);
  r.left = a.left[s] >= 0 ? a.rank[a.left[s]] : -1;
  r.right = a.right[s] >= 0 ? a.rank[a.right[s]] : -1;
  r.lt_hi_l = 0;
  r.lt_hi_r = 0;
  const int64_t G = nb <= 8 ? 1 : (nb + 7) / 8;
  for (int i = 0; i < 8; ++i) {
    if (i * G < nb && !exact) {
      int64_t last = min(8 * G * (i + 1) - 1, k - 1);
      r.coarse[i] = (float)(cump[last] * inv);
    } else {
      r.coarse[i] = kInf;
    }
  }
  a.rec[si] = r;
  a.pos4i[si] = p1;
  a.left_i[si] = r.left;
  a.right_i[si] = r.right;
}

// blocks per row in storage order, from the row pointers (reference order):
// blkptr[i] = ceil(len(perm[i]) / 8), scanned afterwards
__global__ void k_blk_counts(BuildArgs a) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i > a.n_sites) return;
  if (i == a.n_sites) {
    a.blkptr[i] = 0;
    return;
  }
  const int64_t s = a.perm[i];
  a.blkptr[i] = (a.rowptr[s + 1] - a.rowptr[s] + 7) / 8;
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
// Per site and link: the flight time of the link (fly's dist / v) and the unit vector toward the
// neighbour (fly's normalise(next - pos)), with the operations of particle::fly from the site
// position, so that a flight starting at a site needs neither a root nor a division.
__global__ void k_link_times(const double4_32a* __restrict__ pos4, const int32_t* __restrict__ left,
                             const int32_t* __restrict__ right, SiteRec* rec, double2* lt64, double* ulink, int64_t n,
                             double v) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  double4_32a p = pos4[s];
  double tl = 0, tr = 0;
  double u[6] = {0, 0, 0, 0, 0, 0};
  int32_t l = left[s], r = right[s];
  for (int side = 0; side < 2; ++side) {
    const int32_t nb = side ? r : l;
    if (nb < 0) continue;
    double4_32a t = pos4[nb];
    const double lt = norm3(p.x - t.x, p.y - t.y, p.z - t.z) / v;
    const double e0 = t.x - p.x, e1 = t.y - p.y, e2 = t.z - p.z;
    const double nn = norm3(e0, e1, e2);
    const double den = nn != 0 ? nn : 1.0;
    u[3 * side] = e0 / den;
    u[3 * side + 1] = e1 / den;
    u[3 * side + 2] = e2 / den;
    if (side)
      tr = lt;
    else
      tl = lt;
  }
  lt64[s] = make_double2(tl, tr);
  for (int k = 0; k < 6; ++k) ulink[6 * s + k] = u[k];
  rec[s].lt_hi_l = (uint32_t)((uint64_t)__double_as_longlong(tl) >> 32);
  rec[s].lt_hi_r = (uint32_t)((uint64_t)__double_as_longlong(tr) >> 32);
}

cudaError_t launch_link_times(const double4_32a* pos4, const int32_t* left, const int32_t* right, SiteRec* rec,
                              double2* lt64, double* ulink, int64_t n, double v, cudaStream_t s) {
  int64_t nb = (n + 255) / 256;
  if (nb) k_link_times<<<(unsigned)nb, 256, 0, s>>>(pos4, left, right, rec, lt64, ulink, n, v);
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
  int32_t site = (f.mode == 1) ? a.rank[f.site0 + dice] : a.inject[f.inj0 + dice];  // storage slot
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

// ============================================================================ work order
// Order in which the mixed kernel's work queue hands out exciton slots: by the storage slot of
// the exciton's current site (sites are stored in spatial order), in buckets of kOrderSpan slots.
// The excitons in flight at one time then hop over a compact part of the film whose rows stay in
// L2.  The order decides only which exciton a lane takes next, never a result.
__global__ void k_order_count(HopArgs a, int64_t n_buckets, int64_t* __restrict__ bucket,
                              unsigned long long* __restrict__ count) {
  int64_t slot = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (slot >= a.n_slots) return;
  const int64_t b = (a.e_flags[slot] & kExActive) ? (int64_t)(a.e_site[slot] / kOrderSpan) : n_buckets;  // empty slots last
  bucket[slot] = b;
  atomicAdd(&count[b], 1ull);
}

__global__ void k_order_fill(int64_t n_slots, const int64_t* __restrict__ bucket, unsigned long long* __restrict__ start,
                             int32_t* __restrict__ order) {
  int64_t slot = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (slot >= n_slots) return;
  unsigned long long at = atomicAdd(&start[bucket[slot]], 1ull);
  order[at] = (int32_t)slot;
}

int scan_kernel_count(int64_t n) {
  if (n <= 0) return 0;
  int64_t tiles = (n + kScanTile - 1) / kScanTile;
  return tiles == 1 ? 1 : 2 + scan_kernel_count(tiles);
}

int64_t order_buckets(const FilmDev& f) {
  const int64_t ntx = (f.nx + kOrderTile - 1) / kOrderTile, nty = (f.ny + kOrderTile - 1) / kOrderTile;
  return ntx * nty * kOrderTile * kOrderTile * f.nz;
}

cudaError_t build_work_order(const HopArgs& a, int64_t n_buckets, int64_t* bucket, int64_t* count,
                             int64_t* scan_scratch, int64_t scratch_len, int32_t* order, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(count, 0, (n_buckets + 1) * sizeof(int64_t), s);
  if (e != cudaSuccess) return e;
  const int64_t nb = (a.n_slots + 255) / 256;
  if (nb == 0) return cudaSuccess;
  auto* cnt = reinterpret_cast<unsigned long long*>(count);
  k_order_count<<<(unsigned)nb, 256, 0, s>>>(a, n_buckets, bucket, cnt);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = exclusive_scan_i64(count, n_buckets + 1, scan_scratch, scratch_len, s)) != cudaSuccess) return e;
  k_order_fill<<<(unsigned)nb, 256, 0, s>>>(a.n_slots, bucket, cnt, order);
  return cudaGetLastError();
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
    if (e.active && !dead) dead = !step_fp64(a, e, a.dt);
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
// Variants of the mixed kernel: (threads per block, resident blocks per SM the registers are
// budgeted for).  The log table is staged once per block, so fewer, larger blocks leave more of
// the SM's shared-memory/L1 array to the L1 cache.
//   0: 128 x 4   1: 128 x 6   2: 128 x 8   3: 256 x 3   4: 768 x 1   5: 1024 x 1
cudaError_t launch_hop_mixed(const HopArgs& a, int64_t n_steps, int variant, int grid_blocks, int single_film,
                             unsigned long long* queue, cudaStream_t s) {
  if (variant >= 3) return launch_hop_mixed_large(a, n_steps, variant, grid_blocks, single_film, queue, s);
  return launch_hop_mixed_small(a, n_steps, variant, grid_blocks, single_film, queue, s);
}

int hop_mixed_blocks_per_sm(int variant, int64_t n_steps, int single_film) {
  if (variant >= 3) return hop_mixed_blocks_per_sm_large(variant, n_steps, single_film);
  return hop_mixed_blocks_per_sm_small(variant, n_steps, single_film);
}

// ============================================================================ self-checks
// u_from_rand against IEEE division for r in [r0, r0 + count)
// and the dwell-time logs kmc_log_unit and kmc_dwell_log against the general kmc_log on the
// same uniform
__global__ void k_u_check(uint32_t r0, uint64_t count, unsigned long long* mism, const LogTab* tab) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  unsigned long long bad = 0;
  for (; i < count; i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t r = r0 + (uint32_t)i;
    if (r == 0) continue;
    double a = u_from_rand(r), b = (double)r / (double)kRandMax;
    bad += (__double_as_longlong(a) != __double_as_longlong(b));
    bad += (__double_as_longlong(kmc_log_unit(a, tab)) != __double_as_longlong(kmc_log(b, tab)));
    bad += (__double_as_longlong(kmc_dwell_log(r, tab)) != __double_as_longlong(kmc_log(b, tab)));
  }
  if (bad) atomicAdd(mism, bad);
}

cudaError_t launch_u_check(uint32_t r0, uint64_t count, unsigned long long* mismatches, const LogTab* tab,
                           cudaStream_t s) {
  k_u_check<<<152 * 8, 256, 0, s>>>(r0, count, mismatches, tab);
  return cudaGetLastError();
}

// L2 read bandwidth: every thread streams 16-byte L2-only loads (ld.global.cg) over an
// L2-resident buffer; the XOR of what it read keeps the loads alive
__global__ void __launch_bounds__(512) k_l2_probe(const int4* __restrict__ buf, int64_t n16, int reps,
                                                  unsigned long long* sink) {
  uint32_t acc = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int r = 0; r < reps; ++r)
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n16; i += stride) {
      const int4 v = __ldcg(buf + i);
      acc ^= (uint32_t)(v.x ^ v.y ^ v.z ^ v.w);
    }
  if (acc == 0x9E3779B9u) atomicAdd(sink, 1ull);
}

cudaError_t launch_l2_probe(const void* buf, int64_t bytes, int reps, int n_sms, unsigned long long* sink,
                            cudaStream_t s) {
  k_l2_probe<<<(unsigned)(n_sms * 4), 512, 0, s>>>(reinterpret_cast<const int4*>(buf), bytes / 16, reps, sink);
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
