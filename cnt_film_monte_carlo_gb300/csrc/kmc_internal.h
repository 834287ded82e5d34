// kmc_internal.h -- device data layout and kernel launchers of the engine (not part of the ABI).
#pragma once
#include <cuda_runtime.h>

#include <nvtx3/nvToolsExt.h>

#include <cstdint>

#include "kmc_device.cuh"

// bits of the device error word
#define KMC_ERR_HOP_CAP_CODE 1   // an exciton exceeded the hop cap of one step
#define KMC_ERR_CELL_CODE 2      // a site fell outside the cell grid
#define KMC_ERR_FLIGHT_CODE 4    // a free flight crossed more than kMaxCrossings links
#define KMC_ERR_CAPACITY_CODE 8  // contacts mode: fewer empty slots than new excitons
#define KMC_ERR_CHECK_CODE 16    // KMC_CHECK builds: an index or counter failed its bounds check

// Device bounds checks of the KMC_CHECK build (libcntkmc_check.so): KMC_DCHECK(err, cond) is
// false, and sets KMC_ERR_CHECK_CODE in the error word, when cond fails; the caller then skips
// or replaces the access it guards, so that the kernel stays in bounds and the host reports the
// failure after the launch.  In the normal build it is the constant true and compiles away.
#ifdef KMC_CHECK
#define KMC_DCHECK(err, cond) ((cond) ? true : (atomicOr((err), KMC_ERR_CHECK_CODE), false))
#else
#define KMC_DCHECK(err, cond) true
#endif

struct kmc_ctx;  // the engine context (include/cntkmc.h; defined in cntkmc_api.cu)

namespace kmc {

// NVTX range over the host span of an entry point or one of its phases (build, launch, reduce),
// for Nsight Systems timelines; without a tool attached a push/pop is a branch on a null hook.
// next() closes the current phase and opens the following one; early returns close it.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  void next(const char* name) {
    nvtxRangePop();
    nvtxRangePushA(name);
  }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// Per-film constants (device copy).
struct FilmDev {
  int64_t site0, n_sites;   // film's sites in the global site arrays
  int64_t cell0, n_cells;   // film's cells in the global cell arrays
  int64_t nnz0, nnz;        // film's neighbour entries in the global CSR arrays
  int64_t blk0, nblk;       // film's 8-entry blocks in the blocked (mixed-precision) row arrays
  int32_t nx, ny, nz, mode; // cell grid; injection mode
  double mn[3];             // domain minimum (cell origin)
  double r;                 // cell side = max hopping radius
  int64_t inj0, n_inj;      // injection sites (storage slots) in the inject array
  double rmin[3], rmax[3];  // removal domain (mode 0)
  uint64_t seed;            // Philox key
  int64_t slot0, n_exc;     // exciton slots (padded to whole warps)
};

// Per-site record read once per hop by the mixed kernel: one 64-byte line.  coarse[] is the
// first level of the row search: the FP32 normalised cumulative rate at the end of each group
// of G blocks (G = 1 for rows of up to 64 entries, ceil(blocks/8) up to 512 entries), +inf
// past the row end.
struct __align__(64) SiteRec {
  double inv_total;   // 1 / total rate (inf for an empty list)
  uint32_t blk;       // film-local index of the row's first 8-entry block
  uint32_t len_flags; // row length (low 24 bits) | flags
  int32_t left, right;// tube neighbours (storage slots) or -1
  uint32_t lt_hi_l;   // high 32 bits of the FP64 link time to the left / right neighbour
  uint32_t lt_hi_r;
  float coarse[8];
};
// One 64-byte block of a neighbour row: 8 FP32 values of cum/total and the 8 neighbours
// (storage slots); entries past the row end hold +inf and -1.
struct __align__(64) RowBlock {
  float c[8];
  int32_t col[8];
};
constexpr uint32_t kRecExact = 1u << 24;  // row resolved in FP64 only (non-finite/zero total, negative rate)
constexpr uint32_t kRecLong = 1u << 25;   // row longer than 512 entries: FP32 bisection over the blocks
constexpr uint32_t kLenMask = (1u << 24) - 1;

struct TableDev {
  int32_t kind;
  int32_t n[4];
  const double* grid[4];
  const double* rate;
  double inv_h[4];  // (n - 1) / (grid[n-1] - grid[0]) for ascending grids, 0: always scan in full
  const int32_t* species;  // kind 3: chirality of each site (reference id); pair table
                           // (species[donor], species[acceptor]) of n[2] x n[2]
  // 2-D tables (kinds 2, 3) with ascending grids: the squared distances between neighbouring
  // distance-grid points (m_k^2, m_k = (g_k + g_k+1) / 2, ascending) and the cosines of the
  // midpoints of the angle grid (cos m_k, descending), each with the lookup's safety margin
  // applied on the host: d2_above[k] = m_k^2 (1 + 1e-12), d2_below[k] = m_k^2 (1 - 1e-12),
  // cos_below[k] = cos m_k - 1e-13, cos_above[k] = cos m_k + 1e-13; nullptr when the grids do
  // not allow it (the lookup then always takes the exact path).  g0f, ihf: the first grid points
  // and inverse spacings of both grids in FP32 (the index estimate).
  const double* d2_above;
  const double* d2_below;
  const double* cos_below;
  const double* cos_above;
  float g0f[2], ihf[2];
};

// Exciton flags
constexpr uint32_t kExHeading = 1u;  // heading right
constexpr uint32_t kExAtSite = 2u;   // position equals the current site's position (mixed kernel)
constexpr uint32_t kExActive = 4u;   // slot holds an exciton (not warp padding)

struct HopArgs {
  // sites: every array indexed by storage slot (spatial order), except rowptr
  const double4_32a* pos4;
  const int32_t* left;
  const int32_t* right;
  const int64_t* rowptr;  // reference-order CSR offsets (read-back)
  const int64_t* blkptr;  // first row block of each site (global)
  const double* total;
  const double* inv_total;
  const SiteRec* rec;
  const RowBlock* blocks; // blocked rows (global block index)
  const float* blast;     // last FP32 value of every block (second search level of long rows)
  const double* cump;     // FP64 cumulative rates in the blocked layout (8 per block)
  const double2* lt64;    // exact link times (left, right)
  const double* ulink;    // [site][6]: unit vectors toward the left and the right neighbour
  int64_t n_sites, n_blocks;  // extents of the site and row-block arrays (KMC_CHECK bounds)
  // films and excitons
  const FilmDev* films;
  const int32_t* warp_film;
  const int32_t* inject;
  int32_t* e_site;
  uint32_t* e_flags;
  double* e_pos;    // [3][n_slots]
  double* e_delta;  // [3][n_slots]
  double* e_ff;
  uint64_t* e_draws;
  uint64_t* e_hops;
  int64_t n_slots;
  const int32_t* order;  // mixed kernel: slot handed out at queue position q (nullptr: q itself)
  const int32_t* rank;   // reference site id -> storage slot (exciton creation)
  // output
  double* msd;      // [n_films][msd_cap][msd_batches][3]
  int64_t msd_cap;
  int32_t msd_batches; // excitons of a film are split into batches by warp: ((local / 32) mod batches)
  int64_t step0;
  int32_t* trace;
  int64_t* trace_cnt;
  int64_t n_trace, trace_cap;
  const LogTab* logtab;
  unsigned long long* counters;  // [0] hops [1] crossings [2] exact re-resolves
  int32_t* err;
  int64_t hop_cap;
  double dt, v;
  int32_t hold_short;     // mixed kernel: batch the ends of short steps across a warp (order only)
};

// FP32 screen of candidate pairs: squared-distance bounds (m^2) outside of which a pair is
// surely out of / surely inside the window (kMinHopDist, r_max), whatever the FP32 rounding
struct PairScreen {
  float out_lo2, out_hi2;  // d2 <= out_lo2 or d2 >= out_hi2: outside
  float in_lo2, in_hi2;    // in_lo2 < d2 < in_hi2: inside
};

struct BuildArgs {
  int32_t n_films;
  const double4_32a* pos4;
  const float4* pos4f;     // FP32 copy of pos4
  PairScreen scr;
  // 2-D tables: the lookup's bounds widened by the worst FP32 error of a pair's squared distance
  // (from pos4f) and of its |cos theta| (from orient4f), rounded outward to FP32, so that an FP32
  // pair inside its cell's bounds is surely where the FP64 lookup puts it.  nullptr: no FP32
  // lookup.
  const float4* orient4f;  // FP32 copy of orient (x, y, z, 0)
  const float* d2_above_f;
  const float* d2_below_f;
  const float* cos_below_f;
  const float* cos_above_f;
  // find_neighbors' window kMinHopDist < sqrt(d2) < r_max (FP64 root, scatterer.cpp:43) as
  // d2 > win_lo2 && d2 < win_hi2: the root is correctly rounded and monotone, so these squared
  // bounds (found on the host) give the same answer for every double d2 without a root
  double win_lo2, win_hi2;
  const double* orient;    // [n][3]
  const int32_t* site_film;
  const FilmDev* films;
  int64_t n_sites;
  int64_t* cell_of;        // [n]
  int64_t* cell_start;     // [n_cells + 1]
  int64_t* cell_cursor;    // [n_cells]
  int32_t* cell_members;   // [n]
  int64_t n_cells;
  TableDev table;
  double r_max;
  int64_t* counts;         // [n + 1] -> rowptr
  int64_t* rowptr;
  double* total;
  double* inv_total;
  int64_t* blkptr;         // [n + 1] first block of each row (global)
  RowBlock* blocks;
  float* blast;
  double* cump;
  SiteRec* rec;
  const int32_t* left;
  const int32_t* right;
  int32_t* err;
  unsigned long long* stats;  // [0] longest row [1] empty rows [2] rows resolved in FP64 only
  // storage order: perm[slot] = reference id, rank[id] = slot; per-slot copies for the hop kernels
  int32_t* perm;
  int32_t* rank;
  double4_32a* pos4i;
  int32_t* left_i;   // links as storage slots (-1: tube end)
  int32_t* right_i;
};

// launchers (kmc_kernels.cu); all return cudaError_t of the launch
cudaError_t launch_pos_f32(const double4_32a* p, float4* out, int64_t n, cudaStream_t s);
cudaError_t launch_orient_f32(const double* orient, float4* out, int64_t n, cudaStream_t s);  // [n][3] -> float4
// The loaded films' sites on the device: positions [n][3] -> pos4, film-local links -> global
// links, the film of every site (offsets[n_films + 1]).  A link outside its film sets *bad_site
// to the smallest such site index (initialised to INT64_MAX by the caller).
cudaError_t launch_load_sites(int64_t n, int32_t n_films, const int64_t* offsets, const double* pos,
                              const int32_t* left_local, const int32_t* right_local, double4_32a* pos4,
                              int32_t* left, int32_t* right, int32_t* site_film, unsigned long long* bad_site,
                              cudaStream_t s);
cudaError_t launch_cell_ids(const BuildArgs& a, cudaStream_t s);
cudaError_t launch_cell_fill(const BuildArgs& a, cudaStream_t s);
cudaError_t launch_nbr_count(const BuildArgs& a, cudaStream_t s);
cudaError_t launch_nbr_fill(const BuildArgs& a, cudaStream_t s);
cudaError_t launch_blk_counts(const BuildArgs& a, cudaStream_t s);
cudaError_t exclusive_scan_i64(int64_t* data, int64_t n, int64_t* scratch, int64_t scratch_len, cudaStream_t s);
int64_t scan_scratch_len(int64_t n);
cudaError_t launch_link_times(const double4_32a* pos4, const int32_t* left, const int32_t* right, SiteRec* rec,
                              double2* lt64, double* ulink, int64_t n, double v, cudaStream_t s);
cudaError_t launch_init_excitons(const HopArgs& a, cudaStream_t s);
// spatial storage order of the sites (see tile_bucket): tiles of kOrderTile x kOrderTile cell
// columns; order_buckets(f) = tiled cell buckets of one film (with padding)
constexpr int kOrderTile = 16;
int64_t order_buckets(const FilmDev& f);
cudaError_t build_site_order(const BuildArgs& a, const int64_t* ord0, int64_t n_buckets, int64_t* sizes,
                             int64_t* scan_scratch, int64_t scratch_len, cudaStream_t s);
cudaError_t ids_to_slots(int32_t* ids, int64_t n, const int32_t* rank, cudaStream_t s);
// work order of the exciton slots: rebuilt before every mixed launch from the slots' current
// sites (bucket = storage slot / kOrderSpan; bucket[n_slots], count[n_buckets + 1])
constexpr int kOrderSpan = 16;
int scan_kernel_count(int64_t n);  // kernels exclusive_scan_i64 launches for n elements
cudaError_t build_work_order(const HopArgs& a, int64_t n_buckets, int64_t* bucket, int64_t* count,
                             int64_t* scan_scratch, int64_t scratch_len, int32_t* order, cudaStream_t s);
cudaError_t launch_hop_fp64(const HopArgs& a, int64_t n_steps, int block, cudaStream_t s);
cudaError_t launch_hop_mixed(const HopArgs& a, int64_t n_steps, int variant, int grid_blocks, int single_film,
                             unsigned long long* queue, cudaStream_t s);
int hop_mixed_blocks_per_sm(int variant, int64_t n_steps, int single_film);
// per-translation-unit halves of the two above (kmc_mixed_small.cu: variants 0-2,
// kmc_mixed_large.cu: variants 3-5)
cudaError_t launch_hop_mixed_small(const HopArgs& a, int64_t n_steps, int variant, int grid_blocks, int single_film,
                                   unsigned long long* queue, cudaStream_t s);
cudaError_t launch_hop_mixed_large(const HopArgs& a, int64_t n_steps, int variant, int grid_blocks, int single_film,
                                   unsigned long long* queue, cudaStream_t s);
int hop_mixed_blocks_per_sm_small(int variant, int64_t n_steps, int single_film);
int hop_mixed_blocks_per_sm_large(int variant, int64_t n_steps, int single_film);
constexpr int kMixedVariants = 6;
// Contacts (steady-state flux) mode: the exciton slots, the y slabs and the per-step outputs.
struct ContactArgs {
  int32_t* e_site;
  uint32_t* e_flags;
  double* e_pos;     // [3][n_slots]
  double* e_delta;   // [3][n_slots]
  double* e_ff;
  uint64_t* e_draws;
  uint64_t* e_hops;
  double* y_old;     // y at the start of the step (particle::step's _old_pos(1))
  int64_t n_slots;
  const double4_32a* pos4;  // sites (storage order)
  const double* inv_total;
  const LogTab* logtab;
  uint64_t seed;            // Philox key; slot k draws from stream k
  int32_t n_seg;
  double ymin, dy;
  const double* y_if;       // [n_seg - 1] interface positions (save_currents)
  double rem_y1[2], rem_y2[2];  // repopulation slabs of contact 1 and contact n_seg
  const int32_t* c_list[2];     // contact sites (storage slots), in site order
  int64_t c_n[2], c_pop[2];
  int64_t* blk_a;           // [blocks + 1] empty slots per block, then their exclusive scan
  int64_t* blk_b;
  int64_t* step;            // index of the step being run (device counter)
  unsigned long long* pop;  // [steps][n_seg] excitons per segment
  unsigned long long* diff; // [steps][n_seg] interface crossings as a difference array
  unsigned long long* n_live;  // [steps] excitons after repopulation
  int64_t steps_cap;        // rows of pop, diff and n_live (KMC_CHECK bounds)
  int32_t* err;
};
int64_t contacts_blocks(int64_t n_slots);
// slots [0, n_initial) get create_particles' excitons (part_first[n_seg + 1]: first exciton of
// each segment; seg_off[n_seg + 1] into seg_sites), the rest are emptied
cudaError_t launch_contacts_init(const ContactArgs& a, const int32_t* seg_sites, const int64_t* seg_off,
                                 const int64_t* part_first, int64_t n_initial, cudaStream_t s);
// after a hop launch of one step: the metrics, both repopulations, the step counter
cudaError_t enqueue_contacts_step(const ContactArgs& a, int64_t* scan_scratch, int64_t scratch_len, cudaStream_t s);
int contacts_kernel_count(int64_t n_slots);
// track_particle: track k (of first..) draws from Philox stream kTrackStream0 + k, apart from the
// exciton slots' streams (< 2^31)
constexpr uint64_t kTrackStream0 = 1ull << 32;
cudaError_t launch_contacts_track(const HopArgs& h, const ContactArgs& a, int64_t first, int32_t n_tracks,
                                  int64_t max_steps, double* path, int64_t* len, int32_t* arrived, cudaStream_t s);
cudaError_t launch_u_check(uint32_t r0, uint64_t count, unsigned long long* mismatches, const LogTab* tab,
                           cudaStream_t s);
cudaError_t launch_l2_probe(const void* buf, int64_t bytes, int reps, int n_sms, unsigned long long* sink,
                            cudaStream_t s);
cudaError_t launch_math_probe(const double* x, double* log_out, double* acos_out, int64_t n, const LogTab* tab,
                              cudaStream_t s);

// ---- learned pair-rate surrogate (kmc_mlp.cu): 4 -> 64 -> 64 -> 1, GELU, BF16 weight matrices
constexpr int kMlpH = 64;
constexpr int kMlpOffW1 = 0, kMlpOffB1 = 256, kMlpOffW2 = 320, kMlpOffB2 = 4416, kMlpOffW3 = 4480,
              kMlpOffB3 = 4544, kMlpOffE = 4548;
constexpr int kMlpChunk = 128;  // samples per block pass of the gradient kernel (one per thread)
struct MlpDev {
  int32_t n_species, n_params;
  double d_min, inv_span;     // log-distance input: ln(d / d_min) inv_span - 1
  double log_mean, log_scale; // ln rate = y log_scale + log_mean
  const float* master;        // [n_params] FP32 master parameters (biases, embedding read here)
  const uint16_t* wbf;        // [n_params] BF16 copies (weight-matrix entries used)
  float* image;               // [kMlpImageFloats] the gradient kernel's shared-memory weights
};
// The network as the gradient kernel holds it in shared memory: W2 and W2^T with 68-word rows,
// W1, b1, b2, w3, the embedding, b3 (FP32; matrices widened from BF16).  Kept in global memory
// by the update kernel so that each gradient launch copies it with 16-byte loads.
constexpr int kMlpImageFloats = 2 * kMlpH * 68 + kMlpH * 4 + 3 * kMlpH + 2 * 8 * 8 + 4;
struct MlpStep {
  float lr, beta1, beta2, eps;
  float c1, c2;               // Adam bias corrections 1 / (1 - beta^t)
  double inv_count;           // 1 / samples of the step (loss = sum r^2 inv_count)
  int32_t update;             // 0: only reduce the gradient
  int32_t loss_slot;          // scheduled steps: the loss goes to loss_out[loss_slot] (-1: not kept)
};
size_t mlp_grad_smem_bytes();
cudaError_t launch_mlp_image(const MlpDev& m, cudaStream_t s);  // the image from master / wbf
// labelled samples -> {log-distance input, angle input, pair bits, normalised label}
cudaError_t launch_mlp_samples(const MlpDev& m, const double* dist, const double* theta, const int32_t* pair,
                               const double* log_rate, int64_t n, float4* out, cudaStream_t s);
// per-block gradient partials part[grid][n_params] and squared-error sums part_loss[grid] of
// samples [first, first + count)
// step_ctr (optional): block 0 adds 1 when the launch starts (the scheduled training loop)
cudaError_t launch_mlp_grad(const MlpDev& m, const float4* samples, int64_t first, int64_t count, float* part,
                            double* part_loss, int grid, cudaStream_t s, unsigned long long* step_ctr = nullptr);
// sum of the partials in block order (grad_out, loss_out optional) and, if st.update, one Adam
// step of master (and its BF16 copy).  With sched, the step is sched[*step_ctr - 1] (the counter
// the gradient launch advanced) and its loss goes to loss_out[loss_slot]: a CUDA graph of launches
// with fixed arguments then runs every step of a schedule.
cudaError_t launch_mlp_update(const MlpDev& m, float* master, uint16_t* wbf, float* mom1, float* mom2,
                              const float* part, const double* part_loss, int grid, const MlpStep& st,
                              float* grad_out, double* loss_out, cudaStream_t s, const MlpStep* sched = nullptr,
                              const unsigned long long* step_ctr = nullptr);
cudaError_t launch_mlp_bf16(const float* master, uint16_t* wbf, int32_t n, cudaStream_t s);
cudaError_t launch_mlp_predict(const MlpDev& m, const double* dist, const double* theta, const int32_t* pair,
                               int64_t n, double* log_rate, cudaStream_t s);
cudaError_t launch_mlp_table(const MlpDev& m, const double* dist, int32_t nd, const double* theta, int32_t nt,
                             double* rate, cudaStream_t s);

// a context's device and stream, and its error message, for the modules outside cntkmc_api.cu
int ctx_device(const kmc_ctx* c);
cudaStream_t ctx_stream(const kmc_ctx* c);
void ctx_set_error(kmc_ctx* c, const char* msg);

}  // namespace kmc
