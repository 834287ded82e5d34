// cntkmc_api.cu -- implementation of the C ABI in include/cntkmc.h (context, device memory,
// launch sequencing).  The kernels are in kmc_kernels.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/cntkmc.h"
#include "kmc_abi_guard.h"
#include "kmc_internal.h"

using kmc::FilmDev;

namespace {

// Owning device buffer (freed on destruction; movable, not copyable), so early error returns
// leak nothing.
template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) {
    o.p = nullptr;
    o.n = 0;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      n = o.n;
      o.p = nullptr;
      o.n = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  cudaError_t alloc(size_t count) {
    release();
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    n = count;
    return cudaSuccess;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

const uint64_t kLogTab[1 << KMC_LOG_TABLE_BITS][2] = KMC_FX_TAB_INIT;

}  // namespace

struct kmc_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string err;
  // films (host copies)
  int32_t n_films = 0;
  int64_t n_sites = 0;
  std::vector<int64_t> film_off;
  std::vector<double> pos;  // [n][3]
  std::vector<FilmDev> films;
  std::vector<std::array<double, 6>> domains;
  bool film_loaded = false;
  DevBuf<double4_32a> d_pos4;
  DevBuf<float4> d_pos4f;  // FP32 copy for the neighbour screen
  DevBuf<double> d_orient;
  DevBuf<int32_t> d_left, d_right, d_site_film;
  DevBuf<FilmDev> d_films;
  // table
  bool has_table = false;
  kmc::TableDev table{};
  DevBuf<double> d_grid[4], d_rate, d_cut[4];  // d2_above, d2_below, cos_below, cos_above
  std::vector<double> h_cut[4];                 // host copies of d_cut (the FP32 lookup's bounds)
  // chirality of each site (read by KMC_TABLE_2D_SPECIES tables); 0 = not set
  int32_t n_species = 0;
  DevBuf<int32_t> d_species;
  // learned pair-rate surrogate
  bool mlp_ready = false;
  kmc_mlp_shape mlp_shape{};
  int32_t mlp_np = 0;
  int64_t mlp_adam_t = 0, mlp_n_samples = 0;
  DevBuf<float> d_mlp_master, d_mlp_m1, d_mlp_m2, d_mlp_part, d_mlp_grad, d_mlp_image;
  DevBuf<uint16_t> d_mlp_wbf;
  DevBuf<double> d_mlp_ploss, d_mlp_loss;
  DevBuf<float4> d_mlp_samples;
  // neighbours
  bool built = false;
  double r_max = 0;
  int64_t nnz = 0, n_cells = 0;
  DevBuf<int64_t> d_cell_of, d_cell_start, d_cell_cursor, d_rowptr, d_scan;
  DevBuf<int32_t> d_cell_members;
  DevBuf<double> d_total, d_inv_total;
  DevBuf<int64_t> d_blkptr;
  DevBuf<kmc::RowBlock> d_blocks;
  DevBuf<float> d_blast;
  DevBuf<double> d_cump;
  int64_t nblk = 0;
  DevBuf<kmc::SiteRec> d_rec;
  DevBuf<double2> d_lt64;
  DevBuf<double> d_ulink;
  // spatial storage order of the sites: perm[slot] = reference id, rank[id] = slot; the
  // hop kernels read positions and links per slot
  DevBuf<int32_t> d_perm, d_rank, d_left_i, d_right_i;
  DevBuf<double4_32a> d_pos4i;
  std::vector<int32_t> h_perm;
  double lt_v = -1;
  // excitons
  bool inited = false;
  int64_t n_slots = 0, n_exc_total = 0;
  std::vector<int64_t> n_exc;
  DevBuf<int32_t> d_warp_film, d_inject, d_e_site;
  DevBuf<uint32_t> d_e_flags;
  DevBuf<double> d_e_pos, d_e_delta, d_e_ff;
  DevBuf<uint64_t> d_e_draws, d_e_hops;
  // msd and trace
  DevBuf<double> d_msd;
  int64_t msd_cap = 0, steps_done = 0;
  int32_t msd_batches = 1;
  int64_t n_trace = 0, trace_cap = 0;
  DevBuf<int32_t> d_trace;
  DevBuf<int64_t> d_trace_cnt;
  // misc
  DevBuf<kmc::LogTab> d_logtab;
  DevBuf<unsigned long long> d_counters, d_stats, d_queue;
  int n_sms = 0;
  DevBuf<int32_t> d_err;
  int64_t hop_cap = 100000000LL;
  int steps_per_launch = 32;
  int block = 128;
  int mixed_variant = 1;
  kmc_run_stats stats{};
  // spatial work order of the mixed kernel (built per launch when in effect)
  int32_t work_order = KMC_ORDER_AUTO;
  int64_t n_obuckets = 0;
  DevBuf<int64_t> d_obucket, d_ocount, d_oscan;
  DevBuf<int32_t> d_order;
  // the launch sequence of a run is captured into a CUDA graph and replayed
  bool use_graph = true;
  cudaGraphExec_t gexec = nullptr;
  // steps of the last run averaged fewer than kShortStepHops hops per exciton: the mixed kernel
  // batches step ends across each warp (see k_hop_mixed)
  bool short_steps = true;
  // contacts (steady-state flux) mode
  bool contacts = false;
  kmc::ContactArgs cargs{};
  int64_t c_steps = 0;
  DevBuf<int32_t> d_c_list;  // contact-1 sites then contact-n sites (storage slots)
  DevBuf<double> d_c_yif, d_y_old;
  DevBuf<int64_t> d_c_blk_a, d_c_blk_b, d_c_scan, d_c_step;
  DevBuf<unsigned long long> d_c_pop, d_c_diff, d_c_live;
  cudaGraphExec_t cgexec = nullptr;  // one contacts step, replayed
  // what the captured contacts step depends on; an unchanged key replays it without a new capture
  struct ContactsGraphKey {
    double dt, v;
    int32_t precision, variant, ordered, grid_blocks, single_film, hold_short;
    int64_t hop_cap, n_trace, n_slots;
    const void *pop, *diff, *live, *msd, *order, *cargs_step;
  } cgkey{};
  bool cgkey_valid = false;
  int c_launches = 0;
};

#define FAIL(ctx, code, ...)                                          \
  do {                                                                \
    char _b[512];                                                     \
    std::snprintf(_b, sizeof _b, __VA_ARGS__);                        \
    (ctx)->err = _b;                                                  \
    return (code);                                                    \
  } while (0)
#define CK(ctx, call)                                                                              \
  do {                                                                                             \
    cudaError_t _e = (call);                                                                       \
    if (_e != cudaSuccess) FAIL(ctx, _e == cudaErrorMemoryAllocation ? KMC_ERR_NOMEM : KMC_ERR_CUDA, \
                                "%s: %s (%s:%d)", #call, cudaGetErrorString(_e), __FILE__, __LINE__); \
  } while (0)

// Film, table, species, neighbour lists, trace or batch settings changed: the excitons (and a
// contacts set-up, whose slot lists and captured step hold the old buffers' addresses) are gone.
static void drop_excitons(kmc_ctx* c) {
  c->inited = false;
  c->contacts = false;
  c->cgkey_valid = false;
}

template <typename T>
static cudaError_t upload(DevBuf<T>& b, const T* h, size_t n, cudaStream_t s) {
  cudaError_t e = b.alloc(n);
  if (e != cudaSuccess) return e;
  if (n) e = cudaMemcpyAsync(b.p, h, n * sizeof(T), cudaMemcpyHostToDevice, s);
  return e;
}

namespace kmc {
int ctx_device(const kmc_ctx* c) { return c->device; }
cudaStream_t ctx_stream(const kmc_ctx* c) { return c->stream; }
void ctx_set_error(kmc_ctx* c, const char* msg) { c->err = msg; }
int abi_fail(kmc_ctx* c, const char* fn) noexcept {
  const char* what = nullptr;
  const int code = abi_status(&what);
  if (c) {
    try {
      c->err = std::string(fn) + ": " + what;
    } catch (...) {  // no room for the message: the status alone
    }
  }
  return code;
}
}  // namespace kmc

extern "C" {

kmc_ctx* kmc_create(int device, int* status) try {
  auto set = [&](int v) {
    if (status) *status = v;
  };
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0) {
    set(KMC_ERR_NO_DEVICE);
    return nullptr;
  }
  if (cudaSetDevice(device) != cudaSuccess) {
    set(KMC_ERR_NO_DEVICE);
    return nullptr;
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess || prop.major != 10) {
    set(KMC_ERR_NO_DEVICE);
    return nullptr;
  }
  kmc_ctx* c = new kmc_ctx();
  c->device = device;
  c->n_sms = prop.multiProcessorCount;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
      upload(c->d_logtab, reinterpret_cast<const kmc::LogTab*>(kLogTab), 1, c->stream) != cudaSuccess ||
      c->d_counters.alloc(4) != cudaSuccess || c->d_stats.alloc(4) != cudaSuccess || c->d_err.alloc(1) != cudaSuccess ||
      c->d_queue.alloc(1) != cudaSuccess ||
      cudaMemsetAsync(c->d_counters.p, 0, 4 * sizeof(unsigned long long), c->stream) != cudaSuccess ||
      cudaMemsetAsync(c->d_err.p, 0, sizeof(int32_t), c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess) {
    set(KMC_ERR_CUDA);
    kmc_destroy(c);
    return nullptr;
  }
  set(KMC_OK);
  return c;
} catch (...) {
  const char* what = nullptr;
  const int code = kmc::abi_status(&what);
  if (status) *status = code;
  return nullptr;
}

void kmc_destroy(kmc_ctx* c) try {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (auto* b : {&c->d_orient, &c->d_total, &c->d_inv_total, &c->d_rate, &c->d_e_pos, &c->d_e_delta,
                  &c->d_e_ff, &c->d_msd})
    b->release();
  for (auto& g : c->d_grid) g.release();
  for (auto* b : {&c->d_left, &c->d_right, &c->d_site_film, &c->d_cell_members, &c->d_warp_film,
                  &c->d_inject, &c->d_e_site, &c->d_trace, &c->d_err})
    b->release();
  for (auto* b : {&c->d_cell_of, &c->d_cell_start, &c->d_cell_cursor, &c->d_rowptr, &c->d_scan, &c->d_trace_cnt})
    b->release();
  c->d_pos4.release();
  c->d_pos4f.release();
  c->d_films.release();
  c->d_blkptr.release();
  c->d_blocks.release();
  c->d_blast.release();
  c->d_cump.release();
  c->d_rec.release();
  c->d_lt64.release();
  c->d_e_flags.release();
  c->d_e_draws.release();
  c->d_e_hops.release();
  c->d_logtab.release();
  c->d_counters.release();
  c->d_stats.release();
  c->d_queue.release();
  for (auto* b : {&c->d_obucket, &c->d_ocount, &c->d_oscan}) b->release();
  for (auto* b : {&c->d_order, &c->d_perm, &c->d_rank, &c->d_left_i, &c->d_right_i}) b->release();
  c->d_pos4i.release();
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->cgexec) cudaGraphExecDestroy(c->cgexec);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
} catch (...) {
}

const char* kmc_last_error(const kmc_ctx* c) { return c ? c->err.c_str() : "null context"; }

// The positions of every site on the host ([n][3], reference order), fetched from the device
// the first time a host-side step needs them (region injection, contacts set-up, restored
// exciton states); kmc_load_film does not keep a host copy.
static int host_positions(kmc_ctx* c) {
  const int64_t n = c->n_sites;
  if ((int64_t)c->pos.size() == 3 * n) return KMC_OK;
  std::vector<double4_32a> p4((size_t)n);
  CK(c, cudaMemcpyAsync(p4.data(), c->d_pos4.p, (size_t)n * sizeof(double4_32a), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  c->pos.resize(3 * (size_t)n);
  for (int64_t s = 0; s < n; ++s) {
    c->pos[3 * s] = p4[s].x;
    c->pos[3 * s + 1] = p4[s].y;
    c->pos[3 * s + 2] = p4[s].z;
  }
  return KMC_OK;
}

int kmc_load_film(kmc_ctx* c, const kmc_film* f) try {
  if (!c) return KMC_ERR_ARG;
  if (!f || f->n_films < 1 || !f->film_site_offsets || !f->pos || !f->orient || !f->left || !f->right)
    FAIL(c, KMC_ERR_ARG, "kmc_load_film: missing arrays");
  CK(c, cudaSetDevice(c->device));
  kmc::NvtxRange nv("kmc_load_film");
  c->film_loaded = false;  // until every check below has passed
  c->built = false;
  drop_excitons(c);
  const int32_t nf = f->n_films;
  const int64_t n = f->film_site_offsets[nf];
  if (f->film_site_offsets[0] != 0 || n <= 0 || n >= (1LL << 31)) FAIL(c, KMC_ERR_ARG, "kmc_load_film: bad offsets");
  c->films.assign(nf, FilmDev{});
  c->domains.assign(nf, {});
  for (int32_t i = 0; i < nf; ++i) {
    const int64_t s0 = f->film_site_offsets[i], s1 = f->film_site_offsets[i + 1];
    if (s1 <= s0) FAIL(c, KMC_ERR_ARG, "kmc_load_film: film %d has no sites", i);
    c->films[i].site0 = s0;
    c->films[i].n_sites = s1 - s0;
  }
  // the raw arrays go to the device as they are (the copies overlap the domains below); a kernel
  // forms the padded positions, the global links and each site's film
  DevBuf<double> d_pos_raw;
  DevBuf<int32_t> d_l_raw, d_r_raw;
  DevBuf<int64_t> d_off;
  DevBuf<unsigned long long> d_bad;
  CK(c, upload(d_off, f->film_site_offsets, (size_t)nf + 1, c->stream));
  CK(c, upload(d_pos_raw, f->pos, 3 * (size_t)n, c->stream));
  CK(c, upload(d_l_raw, f->left, (size_t)n, c->stream));
  CK(c, upload(d_r_raw, f->right, (size_t)n, c->stream));
  CK(c, upload(c->d_orient, f->orient, 3 * (size_t)n, c->stream));
  CK(c, d_bad.alloc(1));
  CK(c, cudaMemsetAsync(d_bad.p, 0xFF, sizeof(unsigned long long), c->stream));
  CK(c, c->d_pos4.alloc(n));
  CK(c, c->d_left.alloc(n));
  CK(c, c->d_right.alloc(n));
  CK(c, c->d_site_film.alloc(n));
  CK(c, kmc::launch_load_sites(n, nf, d_off.p, d_pos_raw.p, d_l_raw.p, d_r_raw.p, c->d_pos4.p, c->d_left.p,
                               c->d_right.p, c->d_site_film.p, d_bad.p, c->stream));
  // find_simulation_domain of every film (monte_carlo.h:328-340), on the host threads
  {
    const unsigned nt = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), (unsigned)nf));
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < nt; ++t)
      pool.emplace_back([&, t]() {
        for (int32_t i = (int32_t)t; i < nf; i += (int32_t)nt) {
          const FilmDev& fd = c->films[i];
          double mn[3], mx[3];
          kmc_domain(fd.n_sites, f->pos + 3 * fd.site0, mn, mx);
          for (int k = 0; k < 3; ++k) {
            c->domains[i][k] = mn[k];
            c->domains[i][3 + k] = mx[k];
          }
        }
      });
    for (auto& th : pool) th.join();
  }
  for (int32_t i = 0; i < nf; ++i)
    for (int k = 0; k < 3; ++k) c->films[i].mn[k] = c->domains[i][k];
  unsigned long long bad = 0;
  CK(c, cudaMemcpyAsync(&bad, d_bad.p, sizeof bad, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  if (bad != ~0ull) FAIL(c, KMC_ERR_ARG, "kmc_load_film: bad link at %lld", (long long)bad);
  c->n_films = nf;
  c->n_sites = n;
  c->film_off.assign(f->film_site_offsets, f->film_site_offsets + nf + 1);
  c->pos.clear();  // the host copy of the positions is fetched from the device when first needed
  c->film_loaded = true;
  c->n_species = 0;
  c->built = false;
  drop_excitons(c);
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_load_film");
}

int kmc_set_site_species(kmc_ctx* c, const int32_t* species, int32_t n_species) try {
  if (!c) return KMC_ERR_ARG;
  if (!c->film_loaded) FAIL(c, KMC_ERR_STATE, "kmc_set_site_species: load a film first");
  if (!species || n_species < 1 || n_species > KMC_MAX_SPECIES)
    FAIL(c, KMC_ERR_ARG, "kmc_set_site_species: need species[n_sites] and 1 <= n_species <= %d", KMC_MAX_SPECIES);
  for (int64_t i = 0; i < c->n_sites; ++i)
    if (species[i] < 0 || species[i] >= n_species)
      FAIL(c, KMC_ERR_ARG, "kmc_set_site_species: site %lld has species %d", (long long)i, species[i]);
  CK(c, cudaSetDevice(c->device));
  CK(c, upload(c->d_species, species, (size_t)c->n_sites, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  c->n_species = n_species;
  c->built = false;
  drop_excitons(c);
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_set_site_species");
}

int kmc_set_rate_table(kmc_ctx* c, const kmc_table* t) try {
  if (!c) return KMC_ERR_ARG;
  if (!t || (t->kind != KMC_TABLE_4D && t->kind != KMC_TABLE_2D && t->kind != KMC_TABLE_2D_SPECIES) || !t->rate)
    FAIL(c, KMC_ERR_ARG, "kmc_set_rate_table: kind must be 4, 2 or 3");
  if (t->kind == KMC_TABLE_2D_SPECIES && (t->n[2] < 1 || t->n[2] > KMC_MAX_SPECIES))
    FAIL(c, KMC_ERR_ARG, "kmc_set_rate_table: species table needs 1 <= n[2] <= %d", KMC_MAX_SPECIES);
  CK(c, cudaSetDevice(c->device));
  kmc::NvtxRange nv("kmc_set_rate_table");
  int dims = t->kind == KMC_TABLE_4D ? 4 : 2;
  int64_t nr = t->kind == KMC_TABLE_2D_SPECIES ? (int64_t)t->n[2] * t->n[2] : 1;
  c->table = kmc::TableDev{};
  c->table.kind = t->kind;
  for (int d = 0; d < dims; ++d) {
    if (t->n[d] < 1 || !t->grid[d]) FAIL(c, KMC_ERR_ARG, "kmc_set_rate_table: grid %d empty", d);
    if (t->n[d] > (int64_t(1) << 34) / nr) FAIL(c, KMC_ERR_ARG, "kmc_set_rate_table: more than 2^34 rates");
    nr *= t->n[d];
    CK(c, upload(c->d_grid[d], t->grid[d], t->n[d], c->stream));
    c->table.n[d] = t->n[d];
    c->table.grid[d] = c->d_grid[d].p;
    // windowed nearest-point search only for strictly ascending grids
    bool asc = t->n[d] >= 8;
    for (int32_t i = 1; i < t->n[d] && asc; ++i) asc = t->grid[d][i] > t->grid[d][i - 1];
    double span = t->grid[d][t->n[d] - 1] - t->grid[d][0];
    c->table.inv_h[d] = (asc && span > 0) ? (double)(t->n[d] - 1) / span : 0.0;
  }
  if (t->kind == KMC_TABLE_2D_SPECIES) c->table.n[2] = t->n[2];
  CK(c, upload(c->d_rate, t->rate, nr, c->stream));
  c->table.rate = c->d_rate.p;
  for (auto& v : c->h_cut) v.clear();
  // 2-D tables: grid midpoints for the neighbour build's lookup without sqrt and arccosine
  // (pair_rate_2d); the distance grid must be non-negative and the angle grid inside [0, pi],
  // where the square and the cosine are monotonic
  if (dims == 2 && c->table.inv_h[0] > 0 && c->table.inv_h[1] > 0 && t->grid[0][0] >= 0 && t->grid[1][0] >= 0 &&
      t->grid[1][t->n[1] - 1] <= 3.141592653589793) {
    std::vector<double> cut[4] = {std::vector<double>(t->n[0] - 1), std::vector<double>(t->n[0] - 1),
                                  std::vector<double>(t->n[1] - 1), std::vector<double>(t->n[1] - 1)};
    for (int32_t k = 0; k + 1 < t->n[0]; ++k) {
      const double m = (t->grid[0][k] + t->grid[0][k + 1]) / 2;
      cut[0][k] = (m * m) * (1.0 + 1e-12);
      cut[1][k] = (m * m) * (1.0 - 1e-12);
    }
    for (int32_t k = 0; k + 1 < t->n[1]; ++k) {
      const double cm = std::cos((t->grid[1][k] + t->grid[1][k + 1]) / 2);
      cut[2][k] = cm - 1e-13;
      cut[3][k] = cm + 1e-13;
    }
    for (int q = 0; q < 4; ++q) {
      CK(c, upload(c->d_cut[q], cut[q].data(), cut[q].size(), c->stream));
      c->h_cut[q] = cut[q];
    }
    c->table.d2_above = c->d_cut[0].p;
    c->table.d2_below = c->d_cut[1].p;
    c->table.cos_below = c->d_cut[2].p;
    c->table.cos_above = c->d_cut[3].p;
    for (int d = 0; d < 2; ++d) {
      c->table.g0f[d] = (float)t->grid[d][0];
      c->table.ihf[d] = (float)c->table.inv_h[d];
    }
  }
  CK(c, cudaStreamSynchronize(c->stream));
  c->has_table = true;
  c->built = false;
  drop_excitons(c);
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_set_rate_table");
}

// Bounds of the FP32 pair screen.  With M the largest coordinate magnitude, the FP32 distance of
// a pair differs from the FP64 one by at most sqrt(3) 2^-23 M + 5 2^-24 d (rounding of the
// coordinates, the difference, the squares and the sum); the margin m = 2^-20 (M + r) is eight
// times that, and each squared bound is rounded outward, so "surely outside / inside" never
// disagrees with the FP64 test.
static kmc::PairScreen pair_screen(double r, double M) {
  const double m = std::ldexp(M, -20) + std::ldexp(r, -20);
  auto up = [](double v) {
    float f = (float)v;
    return (double)f < v ? std::nextafterf(f, INFINITY) : f;
  };
  auto dn = [](double v) {
    float f = (float)v;
    return (double)f > v ? std::nextafterf(f, -INFINITY) : f;
  };
  const double lo = kmc::kMinHopDist;
  kmc::PairScreen sc;
  sc.out_hi2 = up((r + m) * (r + m));
  sc.out_lo2 = lo > m ? dn((lo - m) * (lo - m)) : 0.f;
  sc.in_lo2 = up((lo + m) * (lo + m));
  sc.in_hi2 = r > m ? dn((r - m) * (r - m)) : 0.f;
  if (!(sc.in_lo2 < sc.in_hi2)) sc.in_lo2 = sc.in_hi2 = 0.f;  // no pair is surely inside
  return sc;
}

// The largest double x with sqrt(x) <= v (le) or the smallest with sqrt(x) >= v (ge), sqrt
// correctly rounded (IEEE 754, as on the device): the window test on squared distances.
static double sqrt_bound(double v, bool ge) {
  double x = v * v;
  if (ge) {
    while (x > 0 && std::sqrt(std::nextafter(x, 0.0)) >= v) x = std::nextafter(x, 0.0);
    while (std::sqrt(x) < v) x = std::nextafter(x, INFINITY);
  } else {
    while (std::sqrt(std::nextafter(x, INFINITY)) <= v) x = std::nextafter(x, INFINITY);
    while (x > 0 && std::sqrt(x) > v) x = std::nextafter(x, 0.0);
  }
  return x;
}

int kmc_build_neighbors(kmc_ctx* c, double r_max, kmc_nbr_stats* st) try {
  if (!c) return KMC_ERR_ARG;
  if (!c->film_loaded || !c->has_table) FAIL(c, KMC_ERR_STATE, "kmc_build_neighbors: load a film and a rate table first");
  if (!(r_max > 0)) FAIL(c, KMC_ERR_ARG, "kmc_build_neighbors: radius must be positive");
  if (c->table.kind == KMC_TABLE_2D_SPECIES && c->n_species != c->table.n[2])
    FAIL(c, KMC_ERR_STATE, "kmc_build_neighbors: the species table has %d chiralities, the sites %d", c->table.n[2],
         c->n_species);
  CK(c, cudaSetDevice(c->device));
  kmc::NvtxRange nv("kmc_build_neighbors");
  kmc::NvtxRange phase("build: cell grids");
  const int64_t n = c->n_sites;
  // cell grids, monte_carlo.h:375-387: n_d = ceil((max - min) / r) + 1
  int64_t ncell = 0;
  for (int32_t i = 0; i < c->n_films; ++i) {
    FilmDev& fd = c->films[i];
    const auto& d = c->domains[i];
    double nd[3];
    for (int k = 0; k < 3; ++k) nd[k] = std::ceil((d[3 + k] - d[k]) / r_max) + 1;
    if (!(nd[0] * nd[1] * nd[2] < 2147483648.0))  // cell indices within a film are 32-bit
      FAIL(c, KMC_ERR_ARG, "kmc_build_neighbors: cell grid too large (2^31 cells per film)");
    fd.nx = (int32_t)nd[0];
    fd.ny = (int32_t)nd[1];
    fd.nz = (int32_t)nd[2];
    fd.r = r_max;
    fd.cell0 = ncell;
    fd.n_cells = (int64_t)fd.nx * fd.ny * fd.nz;
    ncell += fd.n_cells;
  }
  c->n_cells = ncell;
  CK(c, upload(c->d_films, c->films.data(), c->films.size(), c->stream));
  CK(c, c->d_cell_of.alloc(n));
  CK(c, c->d_cell_start.alloc(ncell + 1));
  CK(c, c->d_cell_cursor.alloc(ncell));
  CK(c, c->d_cell_members.alloc(n));
  CK(c, c->d_rowptr.alloc(n + 1));
  // buckets of the spatial storage order (tiles of cell columns, film by film)
  std::vector<int64_t> ord0(c->n_films);
  int64_t n_tb = 0;
  for (int32_t i = 0; i < c->n_films; ++i) {
    ord0[i] = n_tb;
    n_tb += kmc::order_buckets(c->films[i]);
  }
  DevBuf<int64_t> d_ord0, d_tsizes;
  CK(c, upload(d_ord0, ord0.data(), ord0.size(), c->stream));
  CK(c, d_tsizes.alloc(n_tb + 1));
  int64_t sl = std::max(std::max(kmc::scan_scratch_len(ncell + 1), kmc::scan_scratch_len(n + 1)),
                        kmc::scan_scratch_len(n_tb + 1));
  CK(c, c->d_scan.alloc(sl));
  CK(c, c->d_perm.alloc(n));
  CK(c, c->d_rank.alloc(n));
  CK(c, cudaMemsetAsync(c->d_cell_start.p, 0, (ncell + 1) * sizeof(int64_t), c->stream));
  CK(c, cudaMemsetAsync(c->d_cell_cursor.p, 0, ncell * sizeof(int64_t), c->stream));
  CK(c, cudaMemsetAsync(c->d_rowptr.p, 0, (n + 1) * sizeof(int64_t), c->stream));
  CK(c, cudaMemsetAsync(c->d_stats.p, 0, 4 * sizeof(unsigned long long), c->stream));
  CK(c, cudaMemsetAsync(c->d_err.p, 0, sizeof(int32_t), c->stream));
  double max_coord = 0;
  for (const auto& d : c->domains)  // the largest coordinate magnitude: the films' domain bounds
    for (double v : d) max_coord = std::max(max_coord, std::fabs(v));
  CK(c, c->d_pos4f.alloc(n));
  CK(c, kmc::launch_pos_f32(c->d_pos4.p, c->d_pos4f.p, n, c->stream));
  kmc::BuildArgs a{};
  a.n_films = c->n_films;
  a.pos4f = c->d_pos4f.p;
  a.scr = pair_screen(r_max, max_coord);
  // The FP32 table lookup of the fill pass: the 2-D lookup's bounds widened by the largest FP32
  // error of a pair's squared distance and of its |cos theta|, then rounded outward to FP32.
  // With u = 2^-24 and M the largest coordinate magnitude, a component of dR formed from FP32
  // positions is off by at most d = 2uM + u r + 2u^2 M, so the sum of squares by at most
  // d (2 sqrt(3) r + 3 d), and its three FP32 roundings add 3.01u (r + d)^2; taken 1.5 times.
  // |cos theta| from FP32 unit vectors: at most 5.1u (two roundings of the components, three
  // of the products and sums), taken as 1e-6.
  DevBuf<float4> d_orient4f;
  DevBuf<float> d_cutf[4];
  if (c->table.d2_above && !c->h_cut[0].empty()) {
    const double u = std::ldexp(1.0, -24);
    const double d = 2 * u * max_coord + u * r_max + 2 * u * u * max_coord;
    const double eps_d2 = 1.5 * (d * (2 * std::sqrt(3.0) * r_max + 3 * d) + 3.01 * u * (r_max + d) * (r_max + d));
    const double eps_c = 1e-6;
    auto up = [](double v) {
      float f = (float)v;
      return (double)f < v ? std::nextafterf(f, INFINITY) : f;
    };
    auto dn = [](double v) {
      float f = (float)v;
      return (double)f > v ? std::nextafterf(f, -INFINITY) : f;
    };
    std::vector<float> cf[4];
    for (double v : c->h_cut[0]) cf[0].push_back(up(v + eps_d2));
    for (double v : c->h_cut[1]) cf[1].push_back(dn(v - eps_d2));
    for (double v : c->h_cut[2]) cf[2].push_back(dn(v - eps_c));
    for (double v : c->h_cut[3]) cf[3].push_back(up(v + eps_c));
    for (int q = 0; q < 4; ++q) CK(c, upload(d_cutf[q], cf[q].data(), cf[q].size(), c->stream));
    CK(c, d_orient4f.alloc(n));
    CK(c, kmc::launch_orient_f32(c->d_orient.p, d_orient4f.p, n, c->stream));
    a.orient4f = d_orient4f.p;
    a.d2_above_f = d_cutf[0].p;
    a.d2_below_f = d_cutf[1].p;
    a.cos_below_f = d_cutf[2].p;
    a.cos_above_f = d_cutf[3].p;
  }
  a.win_lo2 = sqrt_bound(kmc::kMinHopDist, false);  // d2 > win_lo2  <=>  sqrt(d2) > kMinHopDist
  a.win_hi2 = sqrt_bound(r_max, true);              // d2 < win_hi2  <=>  sqrt(d2) < r_max
  a.perm = c->d_perm.p;
  a.rank = c->d_rank.p;
  a.pos4 = c->d_pos4.p;
  a.orient = c->d_orient.p;
  a.site_film = c->d_site_film.p;
  a.films = c->d_films.p;
  a.n_sites = n;
  a.cell_of = c->d_cell_of.p;
  a.cell_start = c->d_cell_start.p;
  a.cell_cursor = c->d_cell_cursor.p;
  a.cell_members = c->d_cell_members.p;
  a.n_cells = ncell;
  a.table = c->table;
  a.table.species = c->table.kind == KMC_TABLE_2D_SPECIES ? c->d_species.p : nullptr;
  a.r_max = r_max;
  a.counts = c->d_rowptr.p;
  a.rowptr = c->d_rowptr.p;
  a.left = c->d_left.p;
  a.right = c->d_right.p;
  a.err = c->d_err.p;
  a.stats = c->d_stats.p;
  phase.next("build: cells and site order");
  CK(c, cudaEventRecord(c->ev0, c->stream));
  CK(c, kmc::launch_cell_ids(a, c->stream));
  CK(c, kmc::exclusive_scan_i64(c->d_cell_start.p, ncell + 1, c->d_scan.p, (int64_t)c->d_scan.n, c->stream));
  CK(c, kmc::launch_cell_fill(a, c->stream));
  CK(c, kmc::build_site_order(a, d_ord0.p, n_tb, d_tsizes.p, c->d_scan.p, (int64_t)c->d_scan.n, c->stream));
  phase.next("build: row lengths");
  CK(c, kmc::launch_nbr_count(a, c->stream));
  CK(c, kmc::exclusive_scan_i64(c->d_rowptr.p, n + 1, c->d_scan.p, (int64_t)c->d_scan.n, c->stream));
  CK(c, c->d_blkptr.alloc(n + 1));
  a.blkptr = c->d_blkptr.p;
  CK(c, kmc::launch_blk_counts(a, c->stream));
  CK(c, kmc::exclusive_scan_i64(c->d_blkptr.p, n + 1, c->d_scan.p, (int64_t)c->d_scan.n, c->stream));
  std::vector<int64_t> nnz0(c->n_films + 1), blk0(c->n_films + 1);
  for (int32_t i = 0; i <= c->n_films; ++i) {
    CK(c, cudaMemcpyAsync(&nnz0[i], c->d_rowptr.p + c->film_off[i], sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaMemcpyAsync(&blk0[i], c->d_blkptr.p + c->film_off[i], sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
  }
  CK(c, cudaStreamSynchronize(c->stream));
  int32_t herr = 0;
  CK(c, cudaMemcpy(&herr, c->d_err.p, sizeof herr, cudaMemcpyDeviceToHost));
  if (herr) FAIL(c, KMC_ERR_ARG, "kmc_build_neighbors: a site lies outside its film's cell grid (non-finite position?)");
  c->nnz = nnz0[c->n_films];
  c->nblk = blk0[c->n_films];
  for (int32_t i = 0; i < c->n_films; ++i) {
    c->films[i].nnz0 = nnz0[i];
    c->films[i].nnz = nnz0[i + 1] - nnz0[i];
    c->films[i].blk0 = blk0[i];
    c->films[i].nblk = blk0[i + 1] - blk0[i];
    if (c->films[i].nnz >= (1LL << 32)) FAIL(c, KMC_ERR_ARG, "kmc_build_neighbors: film %d has >= 2^32 neighbour entries", i);
  }
  CK(c, cudaMemcpyAsync(c->d_films.p, c->films.data(), c->films.size() * sizeof(FilmDev), cudaMemcpyHostToDevice, c->stream));
  CK(c, c->d_blocks.alloc(c->nblk));
  CK(c, c->d_blast.alloc(c->nblk));
  CK(c, c->d_cump.alloc(c->nblk * 8));
  CK(c, c->d_total.alloc(n));
  CK(c, c->d_inv_total.alloc(n));
  CK(c, c->d_rec.alloc(n));
  CK(c, c->d_lt64.alloc(n));
  CK(c, c->d_ulink.alloc(6 * (size_t)n));
  CK(c, c->d_pos4i.alloc(n));
  CK(c, c->d_left_i.alloc(n));
  CK(c, c->d_right_i.alloc(n));
  a.pos4i = c->d_pos4i.p;
  a.left_i = c->d_left_i.p;
  a.right_i = c->d_right_i.p;
  a.blocks = c->d_blocks.p;
  a.blast = c->d_blast.p;
  a.cump = c->d_cump.p;
  a.total = c->d_total.p;
  a.inv_total = c->d_inv_total.p;
  a.rec = c->d_rec.p;
  phase.next("build: rows");
  CK(c, kmc::launch_nbr_fill(a, c->stream));
  CK(c, cudaEventRecord(c->ev1, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  float ms = 0;
  CK(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  unsigned long long hs[4];
  CK(c, cudaMemcpy(hs, c->d_stats.p, sizeof hs, cudaMemcpyDeviceToHost));
  c->h_perm.resize(n);
  CK(c, cudaMemcpy(c->h_perm.data(), c->d_perm.p, n * sizeof(int32_t), cudaMemcpyDeviceToHost));
  c->r_max = r_max;
  c->lt_v = -1;
  c->built = true;
  drop_excitons(c);
  if (st) {
    st->n_sites = n;
    st->nnz = c->nnz;
    st->k_mean = (double)c->nnz / (double)n;
    st->k_max = (int32_t)hs[0];
    st->n_cells = ncell;
    st->isolated = (int64_t)hs[1];
    st->exact_only = (int64_t)hs[2];
    st->build_ms = ms;
  }
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_build_neighbors");
}

int kmc_set_trace(kmc_ctx* c, int64_t n_trace, int64_t cap) try {
  if (!c) return KMC_ERR_ARG;
  if (n_trace < 0 || cap < 0 || (n_trace > 0 && cap == 0)) FAIL(c, KMC_ERR_ARG, "kmc_set_trace: bad sizes");
  // the trace buffer holds n_trace x cap entries, which the hop kernels index as t * cap + k:
  // the product is bounded (2^36 entries, 256 GiB) so that it can neither wrap nor be sized short
  if (n_trace > 0 && cap > (int64_t(1) << 36) / n_trace)
    FAIL(c, KMC_ERR_ARG, "kmc_set_trace: n_trace x cap above 2^36 entries");
  c->n_trace = n_trace;
  c->trace_cap = cap;
  drop_excitons(c);
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_set_trace");
}

int kmc_set_hop_cap(kmc_ctx* c, int64_t cap) try {
  if (!c) return KMC_ERR_ARG;
  if (cap < 1) FAIL(c, KMC_ERR_ARG, "kmc_set_hop_cap: cap must be >= 1");
  c->hop_cap = cap;
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_set_hop_cap");
}

int kmc_init_excitons(kmc_ctx* c, const kmc_inject* inj) try {
  if (!c) return KMC_ERR_ARG;
  if (!c->built) FAIL(c, KMC_ERR_STATE, "kmc_init_excitons: build the neighbour lists first");
  if (!inj || !inj->n_excitons || !inj->seeds) FAIL(c, KMC_ERR_ARG, "kmc_init_excitons: missing arrays");
  if (inj->mode != KMC_INJECT_REGION && inj->mode != KMC_INJECT_UNIFORM) FAIL(c, KMC_ERR_ARG, "kmc_init_excitons: bad mode");
  CK(c, cudaSetDevice(c->device));
  kmc::NvtxRange nv("kmc_init_excitons");
  const int nsec = inj->n_sections;
  if (inj->mode == KMC_INJECT_REGION && !(nsec > 1 && nsec % 2 == 1 && nsec < 1000))
    FAIL(c, KMC_ERR_ARG, "kmc_init_excitons: number of sections must be odd and > 1");
  if (inj->mode == KMC_INJECT_REGION)
    if (int rc = host_positions(c)) return rc;
  std::vector<int32_t> inject;
  std::vector<int32_t> warp_film;
  int64_t slot = 0, total = 0;
  c->n_exc.assign(c->n_films, 0);
  for (int32_t i = 0; i < c->n_films; ++i) {
    FilmDev& fd = c->films[i];
    int64_t ne = inj->n_excitons[i];
    if (ne < 0) FAIL(c, KMC_ERR_ARG, "kmc_init_excitons: negative exciton count");
    fd.mode = inj->mode;
    fd.seed = inj->seeds[i];
    fd.inj0 = (int64_t)inject.size();
    if (inj->mode == KMC_INJECT_REGION) {
      // injection_region / get_removal_domain, monte_carlo.cpp:203-251
      const auto& d = c->domains[i];
      std::vector<double> g[3];
      for (int k = 0; k < 3; ++k) {
        double step = (d[3 + k] - d[k]) / double(nsec);
        for (int q = 0; q <= nsec; ++q) g[k].push_back(double(q) * step + d[k]);
      }
      for (int64_t s = fd.site0; s < fd.site0 + fd.n_sites; ++s) {
        const double* p = &c->pos[3 * s];
        if (g[0][nsec / 2] <= p[0] && p[0] <= g[0][nsec / 2 + 1] && g[1][nsec / 2] <= p[1] && p[1] <= g[1][nsec / 2 + 1] &&
            g[2][nsec / 2] <= p[2] && p[2] <= g[2][nsec / 2 + 1])
          inject.push_back((int32_t)s);
      }
      for (int k = 0; k < 3; ++k) {
        fd.rmin[k] = g[k][1];
        fd.rmax[k] = g[k][nsec - 1];
      }
      fd.n_inj = (int64_t)inject.size() - fd.inj0;
    } else {
      fd.n_inj = fd.n_sites;
    }
    if (ne > 0 && fd.n_inj == 0) FAIL(c, KMC_ERR_ARG, "kmc_init_excitons: film %d has no injection site", i);
    if (fd.n_inj >= (1LL << 31)) FAIL(c, KMC_ERR_ARG, "kmc_init_excitons: too many injection sites");
    // every exciton holds ~80 bytes of state on the device: 2^31 slots (~170 GB) is past what
    // one GPU holds, and the bound keeps the slot arithmetic below far from overflow
    if (ne > (1LL << 31) - slot) FAIL(c, KMC_ERR_ARG, "kmc_init_excitons: more than 2^31 excitons");
    fd.slot0 = slot;
    fd.n_exc = ne;
    int64_t padded = (ne + 31) / 32 * 32;
    for (int64_t w = 0; w < padded / 32; ++w) warp_film.push_back(i);
    slot += padded;
    total += ne;
    c->n_exc[i] = ne;
  }
  if (slot == 0) FAIL(c, KMC_ERR_ARG, "kmc_init_excitons: no excitons");
  c->n_slots = slot;
  c->n_exc_total = total;
  CK(c, cudaMemcpyAsync(c->d_films.p, c->films.data(), c->films.size() * sizeof(FilmDev), cudaMemcpyHostToDevice, c->stream));
  CK(c, upload(c->d_inject, inject.data(), inject.size(), c->stream));
  CK(c, kmc::ids_to_slots(c->d_inject.p, (int64_t)inject.size(), c->d_rank.p, c->stream));
  CK(c, upload(c->d_warp_film, warp_film.data(), warp_film.size(), c->stream));
  CK(c, c->d_e_site.alloc(slot));
  CK(c, c->d_e_flags.alloc(slot));
  CK(c, c->d_e_pos.alloc(3 * slot));
  CK(c, c->d_e_delta.alloc(3 * slot));
  CK(c, c->d_e_ff.alloc(slot));
  CK(c, c->d_e_draws.alloc(slot));
  CK(c, c->d_e_hops.alloc(slot));
  if (c->n_trace > 0) {
    CK(c, c->d_trace.alloc((size_t)(c->n_trace * c->trace_cap)));
    CK(c, c->d_trace_cnt.alloc(c->n_trace));
    CK(c, cudaMemsetAsync(c->d_trace_cnt.p, 0, c->n_trace * sizeof(int64_t), c->stream));
  }
  c->steps_done = 0;
  c->msd_cap = 0;
  c->d_msd.release();
  CK(c, cudaMemsetAsync(c->d_counters.p, 0, 4 * sizeof(unsigned long long), c->stream));
  kmc::HopArgs a{};
  a.pos4 = c->d_pos4i.p;
  a.rank = c->d_rank.p;
  a.inv_total = c->d_inv_total.p;
  a.films = c->d_films.p;
  a.warp_film = c->d_warp_film.p;
  a.inject = c->d_inject.p;
  a.e_site = c->d_e_site.p;
  a.e_flags = c->d_e_flags.p;
  a.e_pos = c->d_e_pos.p;
  a.e_delta = c->d_e_delta.p;
  a.e_ff = c->d_e_ff.p;
  a.e_draws = c->d_e_draws.p;
  a.e_hops = c->d_e_hops.p;
  a.n_slots = slot;
  a.logtab = c->d_logtab.p;
  CK(c, kmc::launch_init_excitons(a, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  c->stats = kmc_run_stats{};
  c->contacts = false;
  c->inited = true;
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_init_excitons");
}

static int ensure_msd(kmc_ctx* c, int64_t need) {
  if (need <= c->msd_cap) return KMC_OK;
  int64_t cap = std::max<int64_t>(need, std::max<int64_t>(64, 2 * c->msd_cap));
  const size_t row = (size_t)c->msd_batches * 3;  // doubles per (film, step)
  DevBuf<double> nb;
  CK(c, nb.alloc((size_t)c->n_films * cap * row));
  CK(c, cudaMemsetAsync(nb.p, 0, (size_t)c->n_films * cap * row * sizeof(double), c->stream));
  if (c->msd_cap > 0 && c->steps_done > 0)
    CK(c, cudaMemcpy2DAsync(nb.p, cap * row * sizeof(double), c->d_msd.p, c->msd_cap * row * sizeof(double),
                            c->steps_done * row * sizeof(double), c->n_films, cudaMemcpyDeviceToDevice, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  c->d_msd.release();
  c->d_msd = std::move(nb);
  c->msd_cap = cap;
  return KMC_OK;
}

static kmc::HopArgs hop_args(kmc_ctx* c, double dt, double v) {
  kmc::HopArgs a{};
  a.pos4 = c->d_pos4i.p;
  a.left = c->d_left_i.p;
  a.right = c->d_right_i.p;
  a.rank = c->d_rank.p;
  a.rowptr = c->d_rowptr.p;
  a.blkptr = c->d_blkptr.p;
  a.total = c->d_total.p;
  a.inv_total = c->d_inv_total.p;
  a.rec = c->d_rec.p;
  a.blocks = c->d_blocks.p;
  a.blast = c->d_blast.p;
  a.cump = c->d_cump.p;
  a.lt64 = c->d_lt64.p;
  a.ulink = c->d_ulink.p;
  a.n_sites = c->n_sites;
  a.n_blocks = c->nblk;
  a.films = c->d_films.p;
  a.warp_film = c->d_warp_film.p;
  a.inject = c->d_inject.p;
  a.e_site = c->d_e_site.p;
  a.e_flags = c->d_e_flags.p;
  a.e_pos = c->d_e_pos.p;
  a.e_delta = c->d_e_delta.p;
  a.e_ff = c->d_e_ff.p;
  a.e_draws = c->d_e_draws.p;
  a.e_hops = c->d_e_hops.p;
  a.n_slots = c->n_slots;
  a.msd = c->d_msd.p;
  a.msd_cap = c->msd_cap;
  a.msd_batches = c->msd_batches;
  a.trace = c->d_trace.p;
  a.trace_cnt = c->d_trace_cnt.p;
  a.n_trace = c->n_trace;
  a.trace_cap = c->trace_cap;
  a.logtab = c->d_logtab.p;
  a.counters = c->d_counters.p;
  a.err = c->d_err.p;
  a.hop_cap = c->hop_cap;
  a.dt = dt;
  a.v = v;
  a.hold_short = c->short_steps ? 1 : 0;
  return a;
}

// Hops per exciton-step of a run decide whether the next runs batch step ends (short steps).
constexpr double kShortStepHops = 64.0;
static void note_step_length(kmc_ctx* c, double hops, double exciton_steps) {
  if (exciton_steps > 0) c->short_steps = hops < kShortStepHops * exciton_steps;
}

// Whether the mixed kernel takes the excitons in spatial order: on request, or (auto) when there
// are several excitons per resident lane, so that the lanes of an SM work on neighbouring sites
// (L1 and L2 reuse; on large films also TLB reach) and the per-launch sort is cheap against the
// launch.
static bool order_in_effect(const kmc_ctx* c) {
  if (c->work_order == KMC_ORDER_SLOTS || !c->built || c->n_slots >= (int64_t)INT32_MAX) return false;
  if (c->work_order == KMC_ORDER_SPATIAL) return true;
  return c->n_slots > (int64_t)c->n_sms * 2048;
}

static int ensure_order_buffers(kmc_ctx* c) {
  const int64_t nb = (c->n_sites + kmc::kOrderSpan - 1) / kmc::kOrderSpan;
  if (c->d_order.p && c->d_order.n == (size_t)c->n_slots && nb == c->n_obuckets) return KMC_OK;
  CK(c, c->d_obucket.alloc(c->n_slots));
  CK(c, c->d_ocount.alloc(nb + 1));
  CK(c, c->d_oscan.alloc(kmc::scan_scratch_len(nb + 1)));
  CK(c, c->d_order.alloc(c->n_slots));
  c->n_obuckets = nb;
  return KMC_OK;
}

// What a hop launch needs besides its arguments: exact link times for the velocity (mixed), the
// work-order buffers, the grid of the persistent mixed kernel.
struct HopPlan {
  bool ordered = false;
  int single_film = 0;
  int grid_blocks = 0;
};

static int prepare_hops(kmc_ctx* c, double v, int32_t precision, int variant, int64_t steps_per_launch, HopPlan* p) {
  if (precision == KMC_PREC_MIXED && c->lt_v != v) {
    CK(c, kmc::launch_link_times(c->d_pos4i.p, c->d_left_i.p, c->d_right_i.p, c->d_rec.p, c->d_lt64.p, c->d_ulink.p,
                                 c->n_sites, v,
                                 c->stream));
    c->lt_v = v;
  }
  p->ordered = precision == KMC_PREC_MIXED && order_in_effect(c);
  if (p->ordered) {
    int rc = ensure_order_buffers(c);
    if (rc) return rc;
  }
  p->single_film = (c->n_films == 1 && c->msd_batches == 1) ? 1 : 0;
  p->grid_blocks = c->n_sms * kmc::hop_mixed_blocks_per_sm(variant, steps_per_launch, p->single_film);
  return KMC_OK;
}

// The launches of n_steps steps (step indices step0.. in a.msd), spl steps per launch, with the
// work-order rebuild before each mixed launch; *nl += kernels launched.
static cudaError_t enqueue_hops(kmc_ctx* c, kmc::HopArgs a, int64_t n_steps, int64_t step0, int32_t precision,
                                int variant, int spl, const HopPlan& p, int* nl) {
  cudaError_t e = cudaSuccess;
  for (int64_t s = 0; s < n_steps && e == cudaSuccess; s += spl) {
    int64_t k = std::min<int64_t>(spl, n_steps - s);
    a.step0 = step0 + s;
    a.order = nullptr;
    if (precision == KMC_PREC_FP64) {
      e = kmc::launch_hop_fp64(a, k, c->block, c->stream);
    } else {
      if (p.ordered) {
        e = kmc::build_work_order(a, c->n_obuckets, c->d_obucket.p, c->d_ocount.p, c->d_oscan.p, (int64_t)c->d_oscan.n,
                                  c->d_order.p, c->stream);
        a.order = c->d_order.p;
        *nl += 2 + kmc::scan_kernel_count(c->n_obuckets + 1);
      }
      if (e == cudaSuccess)
        e = kmc::launch_hop_mixed(a, k, variant, p.grid_blocks, p.single_film, c->d_queue.p, c->stream);
    }
    ++*nl;
  }
  return e;
}

// Capture what enqueue() puts on the context's stream into *exec (updated in place when the
// topology of the previous capture matches, else re-instantiated).
static int capture_graph(kmc_ctx* c, cudaGraphExec_t* exec, const std::function<cudaError_t()>& enqueue) {
  cudaGraph_t g = nullptr;
  CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
  cudaError_t e = enqueue();
  cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    CK(c, e != cudaSuccess ? e : e2);
  }
  bool updated = false;
  if (*exec) {
    cudaGraphExecUpdateResultInfo info;
    updated = cudaGraphExecUpdate(*exec, g, &info) == cudaSuccess;
    if (!updated) {
      cudaGetLastError();  // clear the update's error state
      cudaGraphExecDestroy(*exec);
      *exec = nullptr;
    }
  }
  if (!updated) {
    e = cudaGraphInstantiate(exec, g, 0);
    if (e != cudaSuccess) {
      *exec = nullptr;
      cudaGraphDestroy(g);
      CK(c, e);
    }
  }
  cudaGraphDestroy(g);
  return KMC_OK;
}

// Device error word after a run: the failure it records, or KMC_OK.
static int check_device_error(kmc_ctx* c, const char* who) {
  int32_t herr = 0;
  CK(c, cudaMemcpy(&herr, c->d_err.p, sizeof herr, cudaMemcpyDeviceToHost));
  if (herr & KMC_ERR_CHECK_CODE)
    FAIL(c, KMC_ERR_CHECK, "%s: a device bounds check failed (site, row block, MSD bin or Philox counter)", who);
  if (herr & KMC_ERR_HOP_CAP_CODE)
    FAIL(c, KMC_ERR_HOP_CAP, "%s: an exciton exceeded %lld hops in one step", who, (long long)c->hop_cap);
  if (herr & KMC_ERR_CAPACITY_CODE)
    FAIL(c, KMC_ERR_CAPACITY, "%s: more excitons than the %lld slots of the contacts set-up", who, (long long)c->n_slots);
  if (herr) FAIL(c, KMC_ERR_ARG, "%s: a free flight crossed more than 2^22 links (zero-length tube links?)", who);
  return KMC_OK;
}

constexpr int64_t kMaxGraphLaunches = 256;

// Launch n_steps steps (step indices step0.. in a.msd) with the given shape; device time in *ms.
// The launches (and the work-order rebuild before each mixed launch) are captured into a CUDA
// graph; the graph of the previous run is updated in place when its topology matches.
static int run_steps(kmc_ctx* c, kmc::HopArgs a, int64_t n_steps, int64_t step0, int32_t precision, int variant,
                     int spl, float* ms, int* launches) {
  kmc::NvtxRange phase("run: plan");
  HopPlan plan;
  int rc = prepare_hops(c, a.v, precision, variant, std::min<int64_t>(spl, n_steps), &plan);
  if (rc) return rc;
  int nl = 0;
  auto enqueue = [&]() -> cudaError_t {
    cudaError_t e = cudaMemsetAsync(c->d_err.p, 0, sizeof(int32_t), c->stream);
    if (e == cudaSuccess) e = enqueue_hops(c, a, n_steps, step0, precision, variant, spl, plan, &nl);
    return e;
  };
  // runs of many launches (a caller asking for 10^5 steps in one call) are launched directly:
  // their graph would only add instantiation time
  const bool graph = c->use_graph && (n_steps + spl - 1) / spl <= kMaxGraphLaunches;
  if (graph) {
    phase.next("run: graph capture");
    rc = capture_graph(c, &c->gexec, enqueue);
    if (rc) return rc;
    phase.next("run: launch");
    CK(c, cudaEventRecord(c->ev0, c->stream));
    CK(c, cudaGraphLaunch(c->gexec, c->stream));
  } else {
    phase.next("run: launch");
    CK(c, cudaEventRecord(c->ev0, c->stream));
    CK(c, enqueue());
  }
  CK(c, cudaEventRecord(c->ev1, c->stream));
  phase.next("run: hop kernels (wait)");
  CK(c, cudaStreamSynchronize(c->stream));
  CK(c, cudaEventElapsedTime(ms, c->ev0, c->ev1));
  *launches = nl;
  return check_device_error(c, "kmc_run");
}

int kmc_run(kmc_ctx* c, int64_t n_steps, double dt, double v, int32_t precision) try {
  if (!c) return KMC_ERR_ARG;
  if (!c->inited) FAIL(c, KMC_ERR_STATE, "kmc_run: create the excitons first");
  if (c->contacts) FAIL(c, KMC_ERR_STATE, "kmc_run: the excitons are in contacts mode (kmc_contacts_run)");
  if (n_steps < 0 || !(dt >= 0) || !(v > 0)) FAIL(c, KMC_ERR_ARG, "kmc_run: bad step count, time step or velocity");
  if (precision != KMC_PREC_FP64 && precision != KMC_PREC_MIXED) FAIL(c, KMC_ERR_ARG, "kmc_run: bad precision");
  CK(c, cudaSetDevice(c->device));
  if (n_steps == 0) return KMC_OK;
  kmc::NvtxRange nv("kmc_run");
  dt = dt + 0.0;  // a zero time step is +0 (the kernels compare non-negative doubles bitwise)
  int rc = ensure_msd(c, c->steps_done + n_steps);
  if (rc) return rc;
  kmc::HopArgs a = hop_args(c, dt, v);
  float ms = 0;
  int launches = 0;
  rc = run_steps(c, a, n_steps, c->steps_done, precision, c->mixed_variant, c->steps_per_launch, &ms, &launches);
  unsigned long long after[4];
  CK(c, cudaMemcpy(after, c->d_counters.p, sizeof after, cudaMemcpyDeviceToHost));
  note_step_length(c, (double)(after[0] - (unsigned long long)c->stats.hops), (double)c->n_exc_total * n_steps);
  c->steps_done += n_steps;
  c->stats.hops = (int64_t)after[0];
  c->stats.crossings = (int64_t)after[1];
  c->stats.exact_resolves = (int64_t)after[2];
  c->stats.steps_done = c->steps_done;
  c->stats.last_run_ms = ms;
  c->stats.last_launches = launches;
  return rc;
} catch (...) {
  return kmc::abi_fail(c, "kmc_run");
}

// ---------------------------------------------------------------- contacts mode
int kmc_contacts_init(kmc_ctx* c, const kmc_contacts* cfg, kmc_contacts_info* info, double* area, int64_t* stat_pop) try {
  if (!c) return KMC_ERR_ARG;
  if (!c->built) FAIL(c, KMC_ERR_STATE, "kmc_contacts_init: build the neighbour lists first");
  if (!cfg) FAIL(c, KMC_ERR_ARG, "kmc_contacts_init: missing configuration");
  if (c->n_films != 1) FAIL(c, KMC_ERR_ARG, "kmc_contacts_init: contacts mode runs one film");
  const int32_t n_seg = cfg->n_segments;
  if (n_seg < 2 || n_seg > 4096) FAIL(c, KMC_ERR_ARG, "kmc_contacts_init: number of segments must be in [2, 4096]");
  for (int k = 0; k < 2; ++k)
    if (cfg->contact_pop[k] < 0 || cfg->contact_pop[k] > INT32_MAX)
      FAIL(c, KMC_ERR_ARG, "kmc_contacts_init: contact population out of range");
  CK(c, cudaSetDevice(c->device));
  kmc::NvtxRange nv("kmc_contacts_init");
  if (int rc = host_positions(c)) return rc;
  const int64_t n = c->n_sites;
  const auto& dom = c->domains[0];
  const double ymin = dom[1], ymax = dom[4];
  const double dy = (ymax - ymin) / double(n_seg);
  std::vector<int32_t> rank(n);
  for (int64_t k = 0; k < n; ++k) rank[c->h_perm[k]] = (int32_t)k;
  auto y_of = [&](int64_t k) { return c->pos[3 * k + 1]; };
  // get_area (monte_carlo.h:646-688): per slab the x and z extents, starting from the opposite
  // domain bounds; the else-if leaves a maximum unset while the minimum moves
  std::vector<double> xmn(n_seg, dom[3]), xmx(n_seg, dom[0]), zmn(n_seg, dom[5]), zmx(n_seg, dom[2]);
  for (int64_t k = 0; k < n; ++k) {
    const double* q = &c->pos[3 * k];
    int i = (int)((q[1] - ymin) / dy);
    i = i < 0 ? 0 : (i < n_seg ? i : n_seg - 1);
    if (xmn[i] > q[0])
      xmn[i] = q[0];
    else if (xmx[i] < q[0])
      xmx[i] = q[0];
    if (zmn[i] > q[2])
      zmn[i] = q[2];
    else if (zmx[i] < q[2])
      zmx[i] = q[2];
  }
  if (area)
    for (int i = 0; i < n_seg; ++i) area[i] = (zmx[i] - zmn[i]) * (xmx[i] - xmn[i]);
  // get_scatterer_statistics (:691-719)
  if (stat_pop) {
    std::fill(stat_pop, stat_pop + n_seg, 0);
    for (int64_t k = 0; k < n; ++k) stat_pop[(int)(std::fabs(y_of(k) - ymin) / dy) % n_seg]++;
  }
  // contact_scats(1) and contact_scats(n_seg) (:494-517), in site order
  std::vector<int32_t> clist;
  int64_t cn[2];
  for (int k = 0; k < 2; ++k) {
    const int i = k == 0 ? 1 : n_seg;
    const double y1 = ymin + double(i - 1) * dy, y2 = ymin + double(i) * dy;
    const size_t before = clist.size();
    for (int64_t q = 0; q < n; ++q)
      if (y_of(q) >= y1 && y_of(q) <= y2) clist.push_back(rank[q]);
    cn[k] = (int64_t)(clist.size() - before);
    if (cfg->contact_pop[k] > 0 && cn[k] == 0)
      FAIL(c, KMC_ERR_ARG, "kmc_contacts_init: contact %d has no site to place excitons at", k == 0 ? 1 : n_seg);
  }
  // create_particles (:274-316): slab i gets round(pop1 + i dp) excitons at its sites
  // [y1, y1 + dy), in site order
  // the slab lists in one pass over the sites: a site can only be in the slab (y - ymin) / dy
  // points at or in a neighbour of it (the rounded bounds can leave a site in two slabs or in
  // none); each candidate is tested with the reference's bounds, in site order
  std::vector<std::vector<int32_t>> seg_list((size_t)n_seg);
  for (int64_t q = 0; q < n; ++q) {
    const double y = y_of(q);
    const double f = (y - ymin) / dy;
    if (!(f > -2.0 && f < double(n_seg) + 2.0)) continue;
    const int i0 = (int)std::floor(f);
    for (int i = std::max(0, i0 - 1); i <= std::min(n_seg - 1, i0 + 1); ++i) {
      const double y1 = ymin + double(i) * dy;
      const double y2 = y1 + dy;
      if (y1 <= y && y < y2) seg_list[(size_t)i].push_back(rank[q]);
    }
  }
  std::vector<int32_t> seg_sites;
  std::vector<int64_t> seg_off(1, 0), part_first(1, 0);
  const double dp = double(cfg->contact_pop[1] - cfg->contact_pop[0]) / (double(n_seg) - 1);
  for (int i = 0; i < n_seg; ++i) {
    const int n_particle = (int)std::round(double(cfg->contact_pop[0]) + double(i) * dp);
    seg_sites.insert(seg_sites.end(), seg_list[(size_t)i].begin(), seg_list[(size_t)i].end());
    seg_off.push_back((int64_t)seg_sites.size());
    const int64_t np = std::max(n_particle, 0);
    if (np > 0 && seg_off[i + 1] == seg_off[i])
      FAIL(c, KMC_ERR_ARG, "kmc_contacts_init: segment %d has no site for its %lld excitons", i, (long long)np);
    part_first.push_back(part_first.back() + np);
  }
  const int64_t n_initial = part_first.back();
  int64_t cap = cfg->capacity > 0 ? cfg->capacity
                                  : std::max<int64_t>(1024, 2 * (n_initial + cfg->contact_pop[0] + cfg->contact_pop[1]));
  cap = (cap + 31) / 32 * 32;
  if (cap < n_initial) FAIL(c, KMC_ERR_CAPACITY, "kmc_contacts_init: %lld slots for %lld initial excitons", (long long)cap,
                            (long long)n_initial);
  if (cap >= (1LL << 31)) FAIL(c, KMC_ERR_ARG, "kmc_contacts_init: capacity too large");
  // slots and film
  FilmDev& fd = c->films[0];
  fd.mode = 2;  // no Green-Kubo removal
  fd.seed = cfg->seed;
  fd.slot0 = 0;
  fd.n_exc = cap;
  fd.inj0 = 0;
  fd.n_inj = 0;
  c->n_exc.assign(1, cap);
  c->n_slots = cap;
  c->n_exc_total = cap;
  std::vector<int32_t> warp_film((size_t)(cap / 32), 0);
  CK(c, cudaMemcpyAsync(c->d_films.p, c->films.data(), sizeof(FilmDev), cudaMemcpyHostToDevice, c->stream));
  CK(c, upload(c->d_warp_film, warp_film.data(), warp_film.size(), c->stream));
  CK(c, c->d_e_site.alloc(cap));
  CK(c, c->d_e_flags.alloc(cap));
  CK(c, c->d_e_pos.alloc(3 * cap));
  CK(c, c->d_e_delta.alloc(3 * cap));
  CK(c, c->d_e_ff.alloc(cap));
  CK(c, c->d_e_draws.alloc(cap));
  CK(c, c->d_e_hops.alloc(cap));
  CK(c, c->d_y_old.alloc(cap));
  CK(c, upload(c->d_c_list, clist.data(), clist.size(), c->stream));
  std::vector<double> yif(n_seg - 1);
  for (int i = 1; i < n_seg; ++i) yif[i - 1] = ymin + dy * double(i);  // save_currents :595-597
  CK(c, upload(c->d_c_yif, yif.data(), yif.size(), c->stream));
  const int64_t nb = kmc::contacts_blocks(cap);
  CK(c, c->d_c_blk_a.alloc(nb + 1));
  CK(c, c->d_c_blk_b.alloc(nb + 1));
  CK(c, c->d_c_scan.alloc(kmc::scan_scratch_len(nb + 1)));
  CK(c, c->d_c_step.alloc(1));
  c->cgkey_valid = false;  // buffers and slots change: the next run captures its step afresh
  c->d_c_pop.release();  // sized by the number of slabs: reallocated by the next run
  c->d_c_diff.release();
  c->d_c_live.release();
  if (c->n_trace > 0) {
    CK(c, c->d_trace.alloc((size_t)(c->n_trace * c->trace_cap)));
    CK(c, c->d_trace_cnt.alloc(c->n_trace));
    CK(c, cudaMemsetAsync(c->d_trace_cnt.p, 0, c->n_trace * sizeof(int64_t), c->stream));
  }
  kmc::ContactArgs& a = c->cargs;
  a = kmc::ContactArgs{};
  a.e_site = c->d_e_site.p;
  a.e_flags = c->d_e_flags.p;
  a.e_pos = c->d_e_pos.p;
  a.e_delta = c->d_e_delta.p;
  a.e_ff = c->d_e_ff.p;
  a.e_draws = c->d_e_draws.p;
  a.e_hops = c->d_e_hops.p;
  a.y_old = c->d_y_old.p;
  a.n_slots = cap;
  a.pos4 = c->d_pos4i.p;
  a.inv_total = c->d_inv_total.p;
  a.logtab = c->d_logtab.p;
  a.seed = cfg->seed;
  a.n_seg = n_seg;
  a.ymin = ymin;
  a.dy = dy;
  a.y_if = c->d_c_yif.p;
  // repopulate_contacts (:443-455): slab 1 = [ymin, ymin + dy], slab n = [ymin + (n-1) dy, ymax]
  a.rem_y1[0] = ymin;
  a.rem_y2[0] = ymin + dy;
  a.rem_y1[1] = ymin + double(n_seg - 1) * dy;
  a.rem_y2[1] = ymax;
  a.c_list[0] = c->d_c_list.p;
  a.c_list[1] = c->d_c_list.p + cn[0];
  for (int k = 0; k < 2; ++k) {
    a.c_n[k] = cn[k];
    a.c_pop[k] = cfg->contact_pop[k];
  }
  a.blk_a = c->d_c_blk_a.p;
  a.blk_b = c->d_c_blk_b.p;
  a.step = c->d_c_step.p;
  a.err = c->d_err.p;
  {
    DevBuf<int32_t> d_seg;
    DevBuf<int64_t> d_off, d_first;
    CK(c, upload(d_seg, seg_sites.data(), seg_sites.size(), c->stream));
    CK(c, upload(d_off, seg_off.data(), seg_off.size(), c->stream));
    CK(c, upload(d_first, part_first.data(), part_first.size(), c->stream));
    CK(c, kmc::launch_contacts_init(a, d_seg.p, d_off.p, d_first.p, n_initial, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
  }
  c->steps_done = 0;
  c->msd_cap = 0;
  c->d_msd.release();
  CK(c, cudaMemsetAsync(c->d_counters.p, 0, 4 * sizeof(unsigned long long), c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  c->stats = kmc_run_stats{};
  c->c_steps = 0;
  c->contacts = true;
  c->inited = true;
  if (info) {
    info->ymin = ymin;
    info->ymax = ymax;
    info->dy = dy;
    info->n_initial = n_initial;
    info->n_contact[0] = cn[0];
    info->n_contact[1] = cn[1];
    info->capacity = cap;
  }
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_contacts_init");
}

int kmc_contacts_run(kmc_ctx* c, int64_t n_steps, double dt, double v, int32_t precision, int64_t* population,
                     int64_t* current, int64_t* n_live) try {
  if (!c) return KMC_ERR_ARG;
  if (!c->contacts || !c->built || !c->inited)
    FAIL(c, KMC_ERR_STATE, "kmc_contacts_run: set up contacts mode first (kmc_contacts_init)");
  if (n_steps < 0 || !(dt >= 0) || !(v > 0)) FAIL(c, KMC_ERR_ARG, "kmc_contacts_run: bad step count, time step or velocity");
  if (precision != KMC_PREC_FP64 && precision != KMC_PREC_MIXED) FAIL(c, KMC_ERR_ARG, "kmc_contacts_run: bad precision");
  CK(c, cudaSetDevice(c->device));
  kmc::NvtxRange nv("kmc_contacts_run");
  if (n_steps == 0) return KMC_OK;
  dt = dt + 0.0;
  int rc = ensure_msd(c, 1);  // the hop kernels' MSD sums land in one scratch row
  if (rc) return rc;
  const int32_t n_seg = c->cargs.n_seg;
  // per-step outputs, kept between calls (a caller stepping one step at a time reuses them and
  // the captured graph is updated in place)
  if (c->d_c_live.n < (size_t)n_steps) {
    CK(c, c->d_c_pop.alloc((size_t)n_steps * n_seg));
    CK(c, c->d_c_diff.alloc((size_t)n_steps * n_seg));
    CK(c, c->d_c_live.alloc((size_t)n_steps));
  }
  CK(c, cudaMemsetAsync(c->d_c_pop.p, 0, (size_t)n_steps * n_seg * 8, c->stream));
  CK(c, cudaMemsetAsync(c->d_c_diff.p, 0, (size_t)n_steps * n_seg * 8, c->stream));
  CK(c, cudaMemsetAsync(c->d_c_live.p, 0, (size_t)n_steps * 8, c->stream));
  CK(c, cudaMemsetAsync(c->d_c_step.p, 0, sizeof(int64_t), c->stream));
  CK(c, cudaMemsetAsync(c->d_err.p, 0, sizeof(int32_t), c->stream));
  kmc::ContactArgs ca = c->cargs;
  ca.pop = c->d_c_pop.p;
  ca.diff = c->d_c_diff.p;
  ca.steps_cap = (int64_t)c->d_c_live.n;
  ca.n_live = c->d_c_live.p;
  kmc::HopArgs a = hop_args(c, dt, v);
  HopPlan plan;
  rc = prepare_hops(c, v, precision, c->mixed_variant, 1, &plan);
  if (rc) return rc;
  int nl = 0;
  auto enqueue = [&]() -> cudaError_t {
    nl = 0;
    cudaError_t e = enqueue_hops(c, a, 1, 0, precision, c->mixed_variant, 1, plan, &nl);
    if (e == cudaSuccess) e = kmc::enqueue_contacts_step(ca, c->d_c_scan.p, (int64_t)c->d_c_scan.n, c->stream);
    nl += kmc::contacts_kernel_count(c->n_slots);
    return e;
  };
  if (c->use_graph) {
    kmc_ctx::ContactsGraphKey key{};
    key.dt = dt;
    key.v = v;
    key.precision = precision;
    key.variant = c->mixed_variant;
    key.ordered = plan.ordered ? 1 : 0;
    key.grid_blocks = plan.grid_blocks;
    key.single_film = plan.single_film;
    key.hold_short = a.hold_short;
    key.hop_cap = c->hop_cap;
    key.n_trace = c->n_trace;
    key.n_slots = c->n_slots;
    key.pop = ca.pop;
    key.diff = ca.diff;
    key.live = ca.n_live;
    key.msd = a.msd;
    key.order = c->d_order.p;
    key.cargs_step = ca.step;
    if (!(c->cgexec && c->cgkey_valid && std::memcmp(&key, &c->cgkey, sizeof key) == 0)) {
      c->cgkey_valid = false;
      rc = capture_graph(c, &c->cgexec, enqueue);
      if (rc) return rc;
      c->cgkey = key;
      c->cgkey_valid = true;
      c->c_launches = nl;
    }
    nl = c->c_launches;
    CK(c, cudaEventRecord(c->ev0, c->stream));
    for (int64_t s = 0; s < n_steps; ++s) CK(c, cudaGraphLaunch(c->cgexec, c->stream));
  } else {
    CK(c, cudaEventRecord(c->ev0, c->stream));
    for (int64_t s = 0; s < n_steps; ++s) CK(c, enqueue());
  }
  CK(c, cudaEventRecord(c->ev1, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  float ms = 0;
  CK(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  rc = check_device_error(c, "kmc_contacts_run");
  unsigned long long after[4];
  CK(c, cudaMemcpy(after, c->d_counters.p, sizeof after, cudaMemcpyDeviceToHost));
  const unsigned long long hops_before = (unsigned long long)c->stats.hops;
  c->c_steps += n_steps;
  c->stats.hops = (int64_t)after[0];
  c->stats.crossings = (int64_t)after[1];
  c->stats.exact_resolves = (int64_t)after[2];
  c->stats.steps_done = c->c_steps;
  c->stats.last_run_ms = ms;
  c->stats.last_launches = (int32_t)(nl * n_steps);
  if (rc) return rc;
  std::vector<unsigned long long> hp((size_t)n_steps * n_seg), hd((size_t)n_steps * n_seg), hl((size_t)n_steps);
  CK(c, cudaMemcpy(hp.data(), c->d_c_pop.p, hp.size() * 8, cudaMemcpyDeviceToHost));
  CK(c, cudaMemcpy(hd.data(), c->d_c_diff.p, hd.size() * 8, cudaMemcpyDeviceToHost));
  CK(c, cudaMemcpy(hl.data(), c->d_c_live.p, hl.size() * 8, cudaMemcpyDeviceToHost));
  for (int64_t s = 0; s < n_steps; ++s) {
    long long run = 0;
    for (int32_t i = 0; i < n_seg; ++i) {
      if (population) population[s * n_seg + i] = (int64_t)hp[s * n_seg + i];
      if (i < n_seg - 1) {
        run += (long long)hd[s * n_seg + i];
        if (current) current[s * (n_seg - 1) + i] = run;
      }
    }
    if (n_live) n_live[s] = (int64_t)hl[s];
  }
  double live_steps = 0;
  for (int64_t s = 0; s < n_steps; ++s) live_steps += (double)hl[s];
  note_step_length(c, (double)(after[0] - hops_before), live_steps);
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_contacts_run");
}

int kmc_contacts_track(kmc_ctx* c, int64_t first, int32_t n_tracks, double dt, double v, int64_t max_steps,
                       double* path, int64_t* len, int32_t* arrived) try {
  if (!c) return KMC_ERR_ARG;
  if (!c->contacts || !c->built || !c->inited)
    FAIL(c, KMC_ERR_STATE, "kmc_contacts_track: set up contacts mode first (kmc_contacts_init)");
  if (first < 0 || n_tracks < 0 || max_steps < 0 || !(dt >= 0) || !(v > 0) || (n_tracks > 0 && (!path || !len || !arrived)))
    FAIL(c, KMC_ERR_ARG, "kmc_contacts_track: bad arguments");
  if (c->cargs.c_n[0] == 0) FAIL(c, KMC_ERR_ARG, "kmc_contacts_track: contact 1 has no site");
  if ((double)n_tracks * (double)max_steps * 3.0 > (double)(1LL << 31))
    FAIL(c, KMC_ERR_ARG, "kmc_contacts_track: n_tracks x max_steps too large");
  if (n_tracks == 0) return KMC_OK;
  CK(c, cudaSetDevice(c->device));
  kmc::NvtxRange nv("kmc_contacts_track");
  dt = dt + 0.0;
  const size_t np = (size_t)n_tracks * (size_t)max_steps * 3;
  DevBuf<double> d_path;
  DevBuf<int64_t> d_len;
  DevBuf<int32_t> d_arr;
  CK(c, d_path.alloc(np));
  CK(c, d_len.alloc(n_tracks));
  CK(c, d_arr.alloc(n_tracks));
  CK(c, cudaMemsetAsync(c->d_err.p, 0, sizeof(int32_t), c->stream));
  kmc::HopArgs h = hop_args(c, dt, v);
  CK(c, kmc::launch_contacts_track(h, c->cargs, first, n_tracks, max_steps, d_path.p, d_len.p, d_arr.p, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  int rc = check_device_error(c, "kmc_contacts_track");
  if (rc) return rc;
  if (np) CK(c, cudaMemcpy(path, d_path.p, np * sizeof(double), cudaMemcpyDeviceToHost));
  CK(c, cudaMemcpy(len, d_len.p, n_tracks * sizeof(int64_t), cudaMemcpyDeviceToHost));
  CK(c, cudaMemcpy(arrived, d_arr.p, n_tracks * sizeof(int32_t), cudaMemcpyDeviceToHost));
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_contacts_track");
}

int kmc_set_work_order(kmc_ctx* c, int32_t mode) try {
  if (!c) return KMC_ERR_ARG;
  if (mode != KMC_ORDER_AUTO && mode != KMC_ORDER_SLOTS && mode != KMC_ORDER_SPATIAL)
    FAIL(c, KMC_ERR_ARG, "kmc_set_work_order: mode must be KMC_ORDER_AUTO, _SLOTS or _SPATIAL");
  c->work_order = mode;
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_set_work_order");
}

int kmc_get_work_order(kmc_ctx* c, int32_t* in_effect) try {
  if (!c || !in_effect) return KMC_ERR_ARG;
  *in_effect = order_in_effect(c) ? KMC_ORDER_SPATIAL : KMC_ORDER_SLOTS;
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_get_work_order");
}

int kmc_set_graph(kmc_ctx* c, int32_t on) try {
  if (!c) return KMC_ERR_ARG;
  c->use_graph = on != 0;
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_set_graph");
}

int kmc_set_mixed_variant(kmc_ctx* c, int32_t variant) try {
  if (!c) return KMC_ERR_ARG;
  if (variant < 0 || variant >= kmc::kMixedVariants) FAIL(c, KMC_ERR_ARG, "kmc_set_mixed_variant: 0..%d", kmc::kMixedVariants - 1);
  c->mixed_variant = variant;
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_set_mixed_variant");
}

int kmc_autotune(kmc_ctx* c, double dt, double v, int64_t trial_steps, kmc_tune_result* out) try {
  if (!c) return KMC_ERR_ARG;
  if (!c->inited) FAIL(c, KMC_ERR_STATE, "kmc_autotune: create the excitons first");
  if (trial_steps < 1 || !(dt >= 0) || !(v > 0)) FAIL(c, KMC_ERR_ARG, "kmc_autotune: bad arguments");
  CK(c, cudaSetDevice(c->device));
  kmc::NvtxRange nv("kmc_autotune");
  dt = dt + 0.0;
  const int64_t ns = c->n_slots;
  // save the exciton state and counters; trials run into a scratch MSD buffer
  DevBuf<int32_t> b_site;
  DevBuf<uint32_t> b_flags;
  DevBuf<double> b_pos, b_delta, b_ff, t_msd;
  DevBuf<uint64_t> b_draws, b_hops;
  CK(c, b_site.alloc(ns));
  CK(c, b_flags.alloc(ns));
  CK(c, b_pos.alloc(3 * ns));
  CK(c, b_delta.alloc(3 * ns));
  CK(c, b_ff.alloc(ns));
  CK(c, b_draws.alloc(ns));
  CK(c, b_hops.alloc(ns));
  CK(c, t_msd.alloc((size_t)c->n_films * trial_steps * c->msd_batches * 3));
  auto copy_state = [&](bool save) -> cudaError_t {
    auto cp = [&](void* dst, const void* src, size_t bytes) {
      return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, c->stream);
    };
    cudaError_t e = cudaSuccess;
    if (save) {
      if ((e = cp(b_site.p, c->d_e_site.p, ns * 4)) || (e = cp(b_flags.p, c->d_e_flags.p, ns * 4)) ||
          (e = cp(b_pos.p, c->d_e_pos.p, 3 * ns * 8)) || (e = cp(b_delta.p, c->d_e_delta.p, 3 * ns * 8)) ||
          (e = cp(b_ff.p, c->d_e_ff.p, ns * 8)) || (e = cp(b_draws.p, c->d_e_draws.p, ns * 8)) ||
          (e = cp(b_hops.p, c->d_e_hops.p, ns * 8)))
        return e;
    } else {
      if ((e = cp(c->d_e_site.p, b_site.p, ns * 4)) || (e = cp(c->d_e_flags.p, b_flags.p, ns * 4)) ||
          (e = cp(c->d_e_pos.p, b_pos.p, 3 * ns * 8)) || (e = cp(c->d_e_delta.p, b_delta.p, 3 * ns * 8)) ||
          (e = cp(c->d_e_ff.p, b_ff.p, ns * 8)) || (e = cp(c->d_e_draws.p, b_draws.p, ns * 8)) ||
          (e = cp(c->d_e_hops.p, b_hops.p, ns * 8)))
        return e;
    }
    return cudaSuccess;
  };
  unsigned long long counters[4];
  CK(c, cudaMemcpy(counters, c->d_counters.p, sizeof counters, cudaMemcpyDeviceToHost));
  CK(c, copy_state(true));
  int64_t saved_trace = c->n_trace;
  c->n_trace = 0;  // trials record no trace
  kmc::HopArgs a = hop_args(c, dt, v);
  a.msd = t_msd.p;
  a.msd_cap = trial_steps;
  a.n_trace = 0;
  // one untimed trial measures the step length, so that the timed trials run the instantiation
  // (short-step batching or not) that the runs will use
  int rc = KMC_OK;
  {
    CK(c, copy_state(false));
    CK(c, cudaMemcpyAsync(c->d_counters.p, counters, sizeof counters, cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaMemsetAsync(t_msd.p, 0, t_msd.n * sizeof(double), c->stream));
    float ms = 0;
    int nl = 0;
    rc = run_steps(c, a, trial_steps, 0, KMC_PREC_MIXED, c->mixed_variant, 1, &ms, &nl);
    unsigned long long after[4];
    CK(c, cudaMemcpy(after, c->d_counters.p, sizeof after, cudaMemcpyDeviceToHost));
    int64_t live = 0;
    for (int64_t ne : c->n_exc) live += ne;
    if (c->contacts) {  // the slots' live count
      std::vector<uint32_t> fl(ns);
      CK(c, cudaMemcpy(fl.data(), c->d_e_flags.p, ns * 4, cudaMemcpyDeviceToHost));
      live = 0;
      for (uint32_t f : fl) live += (f & kmc::kExActive) ? 1 : 0;
    }
    if (rc == KMC_OK) note_step_length(c, (double)(after[0] - counters[0]), (double)live * trial_steps);
    a.hold_short = c->short_steps ? 1 : 0;
  }
  const int spl_options[3] = {1, 8, 32};
  double best = -1;
  int best_v = c->mixed_variant, best_spl = c->steps_per_launch;
  for (int variant = 0; variant < kmc::kMixedVariants && rc == KMC_OK; ++variant)
    for (int spl : spl_options) {
      if (spl > trial_steps && spl != 1) continue;
      CK(c, copy_state(false));
      CK(c, cudaMemcpyAsync(c->d_counters.p, counters, sizeof counters, cudaMemcpyHostToDevice, c->stream));
      CK(c, cudaMemsetAsync(t_msd.p, 0, t_msd.n * sizeof(double), c->stream));
      float ms = 0;
      int nl = 0;
      rc = run_steps(c, a, trial_steps, 0, KMC_PREC_MIXED, variant, spl, &ms, &nl);
      if (rc) break;
      unsigned long long after[4];
      CK(c, cudaMemcpy(after, c->d_counters.p, sizeof after, cudaMemcpyDeviceToHost));
      double rate = (double)(after[0] - counters[0]) / (ms * 1e-3);
      if (rate > best) {
        best = rate;
        best_v = variant;
        best_spl = spl;
      }
    }
  c->n_trace = saved_trace;
  CK(c, copy_state(false));
  CK(c, cudaMemcpyAsync(c->d_counters.p, counters, sizeof counters, cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  b_site.release();
  b_flags.release();
  b_pos.release();
  b_delta.release();
  b_ff.release();
  b_draws.release();
  b_hops.release();
  t_msd.release();
  if (rc) return rc;
  c->mixed_variant = best_v;
  c->steps_per_launch = best_spl;
  if (out) {
    out->variant = best_v;
    out->steps_per_launch = best_spl;
    out->hops_per_s = best;
  }
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_autotune");
}

int kmc_get_msd_batches(kmc_ctx* c, int64_t first, int64_t count, double* out) try {
  if (!c) return KMC_ERR_ARG;
  if (!out || first < 0 || count < 0 || count > c->steps_done - first) FAIL(c, KMC_ERR_ARG, "kmc_get_msd: range outside the steps run");
  if (count == 0) return KMC_OK;
  CK(c, cudaSetDevice(c->device));
  kmc::NvtxRange nv("kmc_get_msd_batches");
  const size_t row = (size_t)c->msd_batches * 3;
  CK(c, cudaMemcpy2DAsync(out, count * row * sizeof(double), c->d_msd.p + first * row, c->msd_cap * row * sizeof(double),
                          count * row * sizeof(double), c->n_films, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_get_msd_batches");
}

int kmc_get_msd(kmc_ctx* c, int64_t first, int64_t count, double* out) try {
  if (!c) return KMC_ERR_ARG;
  if (c->msd_batches == 1) return kmc_get_msd_batches(c, first, count, out);
  if (!out || first < 0 || count < 0 || count > c->steps_done - first) FAIL(c, KMC_ERR_ARG, "kmc_get_msd: range outside the steps run");
  kmc::NvtxRange nv("kmc_get_msd: batch reduce");
  const int64_t B = c->msd_batches;
  std::vector<double> tmp((size_t)c->n_films * count * B * 3);
  int rc = kmc_get_msd_batches(c, first, count, tmp.data());
  if (rc) return rc;
  for (int64_t f = 0; f < c->n_films; ++f)
    for (int64_t s = 0; s < count; ++s)
      for (int k = 0; k < 3; ++k) {
        double acc = 0;  // batch order
        for (int64_t b = 0; b < B; ++b) acc += tmp[((f * count + s) * B + b) * 3 + k];
        out[(f * count + s) * 3 + k] = acc;
      }
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_get_msd");
}

int kmc_set_msd_batches(kmc_ctx* c, int32_t batches) try {
  if (!c) return KMC_ERR_ARG;
  if (batches < 1 || batches > 4096) FAIL(c, KMC_ERR_ARG, "kmc_set_msd_batches: 1..4096 batches");
  c->msd_batches = batches;
  drop_excitons(c);
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_set_msd_batches");
}

int64_t kmc_num_excitons(const kmc_ctx* c) { return c && c->inited ? c->n_exc_total : 0; }

int kmc_get_excitons(kmc_ctx* c, int32_t* site, double* pos, double* delta, double* ff, int32_t* heading,
                     uint64_t* draws, int64_t* hops) try {
  if (!c) return KMC_ERR_ARG;
  if (!c->inited) FAIL(c, KMC_ERR_STATE, "kmc_get_excitons: no excitons");
  CK(c, cudaSetDevice(c->device));
  kmc::NvtxRange nv("kmc_get_excitons");
  const int64_t ns = c->n_slots;
  std::vector<int32_t> hs(ns);
  std::vector<uint32_t> hf(ns);
  std::vector<double> hp(3 * ns), hd(3 * ns), hff(ns);
  std::vector<uint64_t> hdr(ns), hh(ns);
  CK(c, cudaMemcpyAsync(hs.data(), c->d_e_site.p, ns * 4, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaMemcpyAsync(hf.data(), c->d_e_flags.p, ns * 4, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaMemcpyAsync(hp.data(), c->d_e_pos.p, 3 * ns * 8, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaMemcpyAsync(hd.data(), c->d_e_delta.p, 3 * ns * 8, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaMemcpyAsync(hff.data(), c->d_e_ff.p, ns * 8, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaMemcpyAsync(hdr.data(), c->d_e_draws.p, ns * 8, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaMemcpyAsync(hh.data(), c->d_e_hops.p, ns * 8, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  int64_t o = 0;
  for (int32_t f = 0; f < c->n_films; ++f) {
    const FilmDev& fd = c->films[f];
    for (int64_t i = 0; i < fd.n_exc; ++i, ++o) {
      int64_t s = fd.slot0 + i;
      if (site) site[o] = hs[s] < 0 ? -1 : (int32_t)(c->h_perm[hs[s]] - fd.site0);
      for (int k = 0; k < 3; ++k) {
        if (pos) pos[3 * o + k] = hp[k * ns + s];
        if (delta) delta[3 * o + k] = hd[k * ns + s];
      }
      if (ff) ff[o] = hff[s];
      if (heading) heading[o] = (hf[s] & kmc::kExHeading) ? 1 : 0;
      if (draws) draws[o] = hdr[s];
      if (hops) hops[o] = (int64_t)hh[s];
    }
  }
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_get_excitons");
}

// The inverse of kmc_get_excitons on the set kmc_init_excitons laid out (same films, counts,
// seeds and injection mode): every field is checked on the host first, then written to the
// slots.  The Philox stream of exciton i of a film is (film seed, i) at counter draws[i], so a
// run resumed from a saved state draws the numbers the uninterrupted run would have drawn.
// kExAtSite (the mixed kernel's "position is the site's" shortcut) is set where the position
// equals the site's bit for bit; the shortcut and the general path give the same doubles there.
int kmc_set_excitons(kmc_ctx* c, const int32_t* site, const double* pos, const double* delta, const double* ff,
                     const int32_t* heading, const uint64_t* draws, const int64_t* hops) try {
  if (!c) return KMC_ERR_ARG;
  if (!c->inited) FAIL(c, KMC_ERR_STATE, "kmc_set_excitons: lay the excitons out with kmc_init_excitons first");
  if (c->contacts) FAIL(c, KMC_ERR_STATE, "kmc_set_excitons: contacts mode keeps its own particle state");
  if (!site || !pos || !delta || !ff || !heading || !draws || !hops) FAIL(c, KMC_ERR_ARG, "kmc_set_excitons: missing arrays");
  CK(c, cudaSetDevice(c->device));
  kmc::NvtxRange nv("kmc_set_excitons");
  if (int rc = host_positions(c)) return rc;
  const int64_t ns = c->n_slots, n = c->n_sites;
  std::vector<int32_t> rank(n);
  for (int64_t k = 0; k < n; ++k) rank[c->h_perm[k]] = (int32_t)k;
  std::vector<int32_t> hs(ns, -1);
  std::vector<uint32_t> hf(ns, 0);
  std::vector<double> hp(3 * ns, 0.0), hd(3 * ns, 0.0), hff(ns, 0.0);
  std::vector<uint64_t> hdr(ns, 0), hh(ns, 0);
  int64_t o = 0;
  for (int32_t f = 0; f < c->n_films; ++f) {
    const FilmDev& fd = c->films[f];
    for (int64_t i = 0; i < fd.n_exc; ++i, ++o) {
      const int64_t s = fd.slot0 + i;
      if (site[o] < 0 || site[o] >= fd.n_sites) FAIL(c, KMC_ERR_ARG, "kmc_set_excitons: exciton %lld: site out of range", (long long)o);
      if (heading[o] != 0 && heading[o] != 1) FAIL(c, KMC_ERR_ARG, "kmc_set_excitons: exciton %lld: heading is 0 or 1", (long long)o);
      if (hops[o] < 0) FAIL(c, KMC_ERR_ARG, "kmc_set_excitons: exciton %lld: negative hop count", (long long)o);
      bool finite = std::isfinite(ff[o]) && ff[o] >= 0;
      for (int k = 0; k < 3; ++k) finite = finite && std::isfinite(pos[3 * o + k]) && std::isfinite(delta[3 * o + k]);
      if (!finite) FAIL(c, KMC_ERR_ARG, "kmc_set_excitons: exciton %lld: non-finite state", (long long)o);
      const int64_t gid = fd.site0 + site[o];
      const double* q = &c->pos[3 * gid];
      bool at = true;
      for (int k = 0; k < 3; ++k) {
        hp[k * ns + s] = pos[3 * o + k];
        hd[k * ns + s] = delta[3 * o + k];
        at = at && std::memcmp(&q[k], &pos[3 * o + k], sizeof(double)) == 0;
      }
      hs[s] = rank[gid];
      hf[s] = kmc::kExActive | (heading[o] ? kmc::kExHeading : 0u) | (at ? kmc::kExAtSite : 0u);
      hff[s] = ff[o];
      hdr[s] = draws[o];
      hh[s] = (uint64_t)hops[o];
    }
  }
  CK(c, cudaMemcpyAsync(c->d_e_site.p, hs.data(), ns * 4, cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaMemcpyAsync(c->d_e_flags.p, hf.data(), ns * 4, cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaMemcpyAsync(c->d_e_pos.p, hp.data(), 3 * ns * 8, cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaMemcpyAsync(c->d_e_delta.p, hd.data(), 3 * ns * 8, cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaMemcpyAsync(c->d_e_ff.p, hff.data(), ns * 8, cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaMemcpyAsync(c->d_e_draws.p, hdr.data(), ns * 8, cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaMemcpyAsync(c->d_e_hops.p, hh.data(), ns * 8, cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaMemsetAsync(c->d_counters.p, 0, 4 * sizeof(unsigned long long), c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  c->steps_done = 0;  // the resumed run's MSD bins and statistics start at its first step
  c->stats = kmc_run_stats{};
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_set_excitons");
}

int kmc_get_run_stats(kmc_ctx* c, kmc_run_stats* st) try {
  if (!c || !st) return KMC_ERR_ARG;
  *st = c->stats;
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_get_run_stats");
}

int kmc_get_neighbors(kmc_ctx* c, int64_t* rowptr, int32_t* col, double* cum, double* total) try {
  if (!c) return KMC_ERR_ARG;
  if (!c->built) FAIL(c, KMC_ERR_STATE, "kmc_get_neighbors: not built");
  CK(c, cudaSetDevice(c->device));
  const int64_t n = c->n_sites;
  std::vector<int64_t> rp(n + 1), bp(n + 1);
  CK(c, cudaMemcpy(rp.data(), c->d_rowptr.p, (n + 1) * 8, cudaMemcpyDeviceToHost));
  if (rowptr) std::copy(rp.begin(), rp.end(), rowptr);
  if (total) {  // stored per slot
    std::vector<double> t(n);
    CK(c, cudaMemcpy(t.data(), c->d_total.p, n * 8, cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < n; ++i) total[c->h_perm[i]] = t[i];
  }
  if (!col && !cum) return KMC_OK;
  CK(c, cudaMemcpy(bp.data(), c->d_blkptr.p, (n + 1) * 8, cudaMemcpyDeviceToHost));
  // rows are stored per slot in 8-entry blocks, with neighbours as slots; gather them back into
  // the reference's CSR layout and ids
  std::vector<kmc::RowBlock> blocks(c->nblk);
  std::vector<double> cump(c->nblk * 8);
  CK(c, cudaMemcpy(blocks.data(), c->d_blocks.p, c->nblk * sizeof(kmc::RowBlock), cudaMemcpyDeviceToHost));
  CK(c, cudaMemcpy(cump.data(), c->d_cump.p, c->nblk * 8 * sizeof(double), cudaMemcpyDeviceToHost));
  for (int32_t f = 0; f < c->n_films; ++f) {
    const FilmDev& fd = c->films[f];
    for (int64_t i = fd.site0; i < fd.site0 + fd.n_sites; ++i) {
      const int64_t s = c->h_perm[i];
      for (int64_t k = 0; k < rp[s + 1] - rp[s]; ++k) {
        if (col) col[rp[s] + k] = c->h_perm[blocks[bp[i] + (k >> 3)].col[k & 7]] - (int32_t)fd.site0;
        if (cum) cum[rp[s] + k] = cump[bp[i] * 8 + k];
      }
    }
  }
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_get_neighbors");
}

int64_t kmc_get_trace(kmc_ctx* c, int64_t e, int32_t* out, int64_t cap) try {
  if (!c || !c->inited || e < 0 || e >= c->n_trace || !out) return KMC_ERR_ARG;
  if (cudaSetDevice(c->device) != cudaSuccess) return KMC_ERR_CUDA;
  int64_t cnt = 0;
  if (cudaMemcpy(&cnt, c->d_trace_cnt.p + e, 8, cudaMemcpyDeviceToHost) != cudaSuccess) return KMC_ERR_CUDA;
  int64_t k = std::min(std::min(cnt, c->trace_cap), cap);
  if (k > 0 && cudaMemcpy(out, c->d_trace.p + e * c->trace_cap, k * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return KMC_ERR_CUDA;
  // storage slots back to site ids: v (hop), -1 - v (link crossing); INT32_MIN marks a reinjection
  for (int64_t j = 0; j < k; ++j) {
    const int32_t v = out[j];
    if (v >= 0) out[j] = c->h_perm[v];
    else if (v != INT32_MIN) out[j] = -1 - c->h_perm[-1 - v];
  }
  return cnt;
} catch (...) {
  return (int64_t)kmc::abi_fail(c, "kmc_get_trace");
}

int kmc_selftest_uniform(kmc_ctx* c, uint32_t r0, uint64_t count, uint64_t* mismatches) try {
  if (!c || !mismatches) return KMC_ERR_ARG;
  CK(c, cudaSetDevice(c->device));
  DevBuf<unsigned long long> m;
  CK(c, m.alloc(1));
  CK(c, cudaMemsetAsync(m.p, 0, 8, c->stream));
  CK(c, kmc::launch_u_check(r0, count, m.p, c->d_logtab.p, c->stream));
  unsigned long long h = 0;
  CK(c, cudaMemcpyAsync(&h, m.p, 8, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  m.release();
  *mismatches = h;
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_selftest_uniform");
}

int kmc_probe_l2(kmc_ctx* c, int64_t bytes, int32_t reps, double* gbs) try {
  if (!c || !gbs) return KMC_ERR_ARG;
  if (bytes < (1 << 20) || bytes % 16 || reps < 1) FAIL(c, KMC_ERR_ARG, "kmc_probe_l2: bytes >= 1 MiB, a multiple of 16; reps >= 1");
  CK(c, cudaSetDevice(c->device));
  DevBuf<unsigned char> buf;
  DevBuf<unsigned long long> sink;
  CK(c, buf.alloc((size_t)bytes));
  CK(c, sink.alloc(1));
  CK(c, cudaMemsetAsync(buf.p, 1, (size_t)bytes, c->stream));
  CK(c, kmc::launch_l2_probe(buf.p, bytes, 2, c->n_sms, sink.p, c->stream));  // bring the buffer into L2
  CK(c, cudaEventRecord(c->ev0, c->stream));
  CK(c, kmc::launch_l2_probe(buf.p, bytes, reps, c->n_sms, sink.p, c->stream));
  CK(c, cudaEventRecord(c->ev1, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  float ms = 0;
  CK(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  *gbs = (double)bytes * reps / (ms * 1e-3) / 1e9;
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_probe_l2");
}

int kmc_math_probe(kmc_ctx* c, const double* x, int64_t n, double* log_out, double* acos_out) try {
  if (!c || !x || !log_out || !acos_out || n < 0) return KMC_ERR_ARG;
  if (n == 0) return KMC_OK;
  CK(c, cudaSetDevice(c->device));
  DevBuf<double> dx, dl, da;
  CK(c, upload(dx, x, n, c->stream));
  CK(c, dl.alloc(n));
  CK(c, da.alloc(n));
  CK(c, kmc::launch_math_probe(dx.p, dl.p, da.p, n, c->d_logtab.p, c->stream));
  CK(c, cudaMemcpyAsync(log_out, dl.p, n * 8, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaMemcpyAsync(acos_out, da.p, n * 8, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  dx.release();
  dl.release();
  da.release();
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_math_probe");
}

// ---- learned pair-rate surrogate ----

static kmc::MlpDev mlp_dev(const kmc_ctx* c) {
  kmc::MlpDev m{};
  m.n_species = c->mlp_shape.n_species;
  m.n_params = c->mlp_np;
  m.d_min = c->mlp_shape.d_min;
  m.inv_span = 2.0 / std::log(c->mlp_shape.d_max / c->mlp_shape.d_min);
  m.log_mean = c->mlp_shape.log_mean;
  m.log_scale = c->mlp_shape.log_scale;
  m.master = c->d_mlp_master.p;
  m.wbf = c->d_mlp_wbf.p;
  m.image = c->d_mlp_image.p;
  return m;
}

// SplitMix64 (Steele, Lea & Flood, "Fast splittable pseudorandom number generators", 2014)
static uint64_t splitmix64(uint64_t& x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// master parameters from the host, BF16 copies, Adam moments cleared
static int mlp_upload_params(kmc_ctx* c, const float* params) {
  const size_t np = (size_t)c->mlp_np;
  CK(c, cudaMemcpyAsync(c->d_mlp_master.p, params, np * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaMemsetAsync(c->d_mlp_m1.p, 0, np * sizeof(float), c->stream));
  CK(c, cudaMemsetAsync(c->d_mlp_m2.p, 0, np * sizeof(float), c->stream));
  CK(c, kmc::launch_mlp_bf16(c->d_mlp_master.p, c->d_mlp_wbf.p, c->mlp_np, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  c->mlp_adam_t = 0;
  c->mlp_ready = true;
  return KMC_OK;
}

// gradient-kernel grid: one block per SM at most, no more blocks than 128-sample chunks
static int mlp_grid(const kmc_ctx* c, int64_t count) {
  const int64_t chunks = (count + kmc::kMlpChunk - 1) / kmc::kMlpChunk;
  return (int)std::min<int64_t>(chunks, c->n_sms);
}

int kmc_mlp_init(kmc_ctx* c, const kmc_mlp_shape* sh, uint64_t seed) try {
  if (!c) return KMC_ERR_ARG;
  if (!sh || sh->n_species < 1 || sh->n_species > KMC_MAX_SPECIES || !(sh->d_min > 0) || !(sh->d_max > sh->d_min) ||
      !(sh->log_scale > 0) || !std::isfinite(sh->log_mean) || !std::isfinite(sh->d_max) || !std::isfinite(sh->log_scale))
    FAIL(c, KMC_ERR_ARG, "kmc_mlp_init: need 1 <= n_species <= %d, 0 < d_min < d_max, log_scale > 0", KMC_MAX_SPECIES);
  CK(c, cudaSetDevice(c->device));
  const int32_t np = KMC_MLP_PARAMS(sh->n_species);
  c->mlp_ready = false;
  c->mlp_n_samples = 0;
  CK(c, c->d_mlp_master.alloc(np));
  CK(c, c->d_mlp_m1.alloc(np));
  CK(c, c->d_mlp_m2.alloc(np));
  CK(c, c->d_mlp_grad.alloc(np));
  CK(c, c->d_mlp_wbf.alloc(np));
  CK(c, c->d_mlp_part.alloc((size_t)c->n_sms * np));
  CK(c, c->d_mlp_image.alloc(kmc::kMlpImageFloats));
  CK(c, cudaMemsetAsync(c->d_mlp_image.p, 0, kmc::kMlpImageFloats * sizeof(float), c->stream));
  // partial entries no thread owns (the padding after b3) stay zero
  CK(c, cudaMemsetAsync(c->d_mlp_part.p, 0, (size_t)c->n_sms * np * sizeof(float), c->stream));
  CK(c, c->d_mlp_ploss.alloc(c->n_sms));
  CK(c, c->d_mlp_loss.alloc(2));
  c->mlp_shape = *sh;
  c->mlp_np = np;
  std::vector<float> p(np, 0.f);
  uint64_t x = seed;
  auto uni = [&](double bound) { return (float)(bound * (2.0 * std::ldexp((double)(splitmix64(x) >> 11), -53) - 1.0)); };
  for (int i = kmc::kMlpOffW1; i < kmc::kMlpOffW2; ++i) p[i] = uni(0.5);    // W1, b1: fan-in 4
  for (int i = kmc::kMlpOffW2; i < kmc::kMlpOffB3; ++i) p[i] = uni(0.125);  // W2, b2, W3: fan-in 64
  for (int i = kmc::kMlpOffE; i < np; ++i) p[i] = uni(1.0);                 // embedding
  return mlp_upload_params(c, p.data());
} catch (...) {
  return kmc::abi_fail(c, "kmc_mlp_init");
}

int kmc_mlp_set_params(kmc_ctx* c, const float* params, int64_t n) try {
  if (!c) return KMC_ERR_ARG;
  if (c->mlp_np == 0) FAIL(c, KMC_ERR_STATE, "kmc_mlp_set_params: call kmc_mlp_init first");
  if (!params || n != c->mlp_np) FAIL(c, KMC_ERR_ARG, "kmc_mlp_set_params: need %d parameters", c->mlp_np);
  for (int64_t i = 0; i < n; ++i)
    if (!std::isfinite(params[i])) FAIL(c, KMC_ERR_ARG, "kmc_mlp_set_params: parameter %lld is not finite", (long long)i);
  CK(c, cudaSetDevice(c->device));
  return mlp_upload_params(c, params);
} catch (...) {
  return kmc::abi_fail(c, "kmc_mlp_set_params");
}

int kmc_mlp_get_params(kmc_ctx* c, float* params, int64_t n) try {
  if (!c) return KMC_ERR_ARG;
  if (!c->mlp_ready) FAIL(c, KMC_ERR_STATE, "kmc_mlp_get_params: call kmc_mlp_init first");
  if (!params || n != c->mlp_np) FAIL(c, KMC_ERR_ARG, "kmc_mlp_get_params: need room for %d parameters", c->mlp_np);
  CK(c, cudaSetDevice(c->device));
  CK(c, cudaMemcpyAsync(params, c->d_mlp_master.p, n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_mlp_get_params");
}

// checks the pair inputs shared by set_samples and predict
static int mlp_check_pairs(kmc_ctx* c, const char* who, int64_t n, const double* dist, const double* theta,
                           const int32_t* pair) {
  const int32_t np2 = c->mlp_shape.n_species * c->mlp_shape.n_species;
  for (int64_t i = 0; i < n; ++i) {
    if (!(dist[i] > 0) || !std::isfinite(dist[i]) || !std::isfinite(theta[i]))
      FAIL(c, KMC_ERR_ARG, "%s: sample %lld has distance %g, angle %g", who, (long long)i, dist[i], theta[i]);
    if (pair[i] < 0 || pair[i] >= np2) FAIL(c, KMC_ERR_ARG, "%s: sample %lld has pair %d", who, (long long)i, pair[i]);
  }
  return KMC_OK;
}

int kmc_mlp_set_samples(kmc_ctx* c, int64_t n, const double* dist, const double* theta, const int32_t* pair,
                        const double* log_rate) try {
  if (!c) return KMC_ERR_ARG;
  if (!c->mlp_ready) FAIL(c, KMC_ERR_STATE, "kmc_mlp_set_samples: call kmc_mlp_init first");
  if (n < 1 || n > (1LL << 31) || !dist || !theta || !pair || !log_rate)
    FAIL(c, KMC_ERR_ARG, "kmc_mlp_set_samples: need 1 <= n <= 2^31 and four arrays");
  if (int rc = mlp_check_pairs(c, "kmc_mlp_set_samples", n, dist, theta, pair)) return rc;
  for (int64_t i = 0; i < n; ++i)
    if (!std::isfinite(log_rate[i])) FAIL(c, KMC_ERR_ARG, "kmc_mlp_set_samples: label %lld is not finite", (long long)i);
  CK(c, cudaSetDevice(c->device));
  DevBuf<double> dd, dt, dl;
  DevBuf<int32_t> dp;
  CK(c, upload(dd, dist, n, c->stream));
  CK(c, upload(dt, theta, n, c->stream));
  CK(c, upload(dp, pair, n, c->stream));
  CK(c, upload(dl, log_rate, n, c->stream));
  CK(c, c->d_mlp_samples.alloc(n));
  CK(c, kmc::launch_mlp_samples(mlp_dev(c), dd.p, dt.p, dp.p, dl.p, n, c->d_mlp_samples.p, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  c->mlp_n_samples = n;
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_mlp_set_samples");
}

int kmc_mlp_gradient(kmc_ctx* c, int64_t first, int64_t count, float* grad, double* loss) try {
  if (!c) return KMC_ERR_ARG;
  if (!c->mlp_ready || c->mlp_n_samples == 0) FAIL(c, KMC_ERR_STATE, "kmc_mlp_gradient: set parameters and samples first");
  if (first < 0 || count < 1 || count > c->mlp_n_samples - first || !grad)
    FAIL(c, KMC_ERR_ARG, "kmc_mlp_gradient: samples [%lld, +%lld) outside [0, %lld)", (long long)first, (long long)count,
         (long long)c->mlp_n_samples);
  CK(c, cudaSetDevice(c->device));
  const kmc::MlpDev m = mlp_dev(c);
  const int grid = mlp_grid(c, count);
  CK(c, kmc::launch_mlp_image(m, c->stream));
  kmc::MlpStep st{};
  st.inv_count = 1.0 / (double)count;
  CK(c, kmc::launch_mlp_grad(m, c->d_mlp_samples.p, first, count, c->d_mlp_part.p, c->d_mlp_ploss.p, grid, c->stream));
  CK(c, kmc::launch_mlp_update(m, c->d_mlp_master.p, c->d_mlp_wbf.p, c->d_mlp_m1.p, c->d_mlp_m2.p, c->d_mlp_part.p,
                               c->d_mlp_ploss.p, grid, st, c->d_mlp_grad.p, c->d_mlp_loss.p, c->stream));
  CK(c, cudaMemcpyAsync(grad, c->d_mlp_grad.p, c->mlp_np * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  double l = 0;
  CK(c, cudaMemcpyAsync(&l, c->d_mlp_loss.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  if (loss) *loss = l;
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_mlp_gradient");
}

int kmc_mlp_train(kmc_ctx* c, const kmc_mlp_train_cfg* cfg, kmc_mlp_train_stats* stats) try {
  if (!c) return KMC_ERR_ARG;
  if (!c->mlp_ready || c->mlp_n_samples == 0) FAIL(c, KMC_ERR_STATE, "kmc_mlp_train: set parameters and samples first");
  if (!cfg || cfg->epochs < 1 || cfg->batch < kmc::kMlpChunk || cfg->batch % kmc::kMlpChunk || cfg->batch > c->mlp_n_samples ||
      !(cfg->lr > 0) || !(cfg->lr_final >= 0) || !(cfg->beta1 >= 0 && cfg->beta1 < 1) || !(cfg->beta2 >= 0 && cfg->beta2 < 1) ||
      !(cfg->eps > 0))
    FAIL(c, KMC_ERR_ARG, "kmc_mlp_train: need epochs >= 1, batch a multiple of 128 within the samples, lr > 0, "
                         "lr_final >= 0, betas in [0, 1), eps > 0");
  CK(c, cudaSetDevice(c->device));
  kmc::NvtxRange nv("kmc_mlp_train");
  const kmc::MlpDev m = mlp_dev(c);
  CK(c, kmc::launch_mlp_image(m, c->stream));
  const int64_t per_epoch = c->mlp_n_samples / cfg->batch;
  const int64_t total = per_epoch * cfg->epochs;
  const int grid = mlp_grid(c, cfg->batch);
  // the whole schedule (cosine learning rate, Adam bias corrections, where the loss is kept) on
  // the device; each gradient launch advances a device counter that its update launch reads, so
  // one epoch of launches with fixed arguments is captured once and replayed every epoch
  std::vector<kmc::MlpStep> sched((size_t)total);
  for (int64_t k = 0; k < total; ++k) {
    const int64_t t = c->mlp_adam_t + k + 1;
    kmc::MlpStep& st = sched[(size_t)k];
    const double cosine = 0.5 * (1.0 + std::cos(3.141592653589793 * (double)k / (double)total));
    st.lr = (float)(cfg->lr_final + (cfg->lr - cfg->lr_final) * cosine);
    st.beta1 = (float)cfg->beta1;
    st.beta2 = (float)cfg->beta2;
    st.eps = (float)cfg->eps;
    st.c1 = (float)(1.0 / (1.0 - std::pow(cfg->beta1, (double)t)));
    st.c2 = (float)(1.0 / (1.0 - std::pow(cfg->beta2, (double)t)));
    st.inv_count = 1.0 / (double)cfg->batch;
    st.update = 1;
    st.loss_slot = k == 0 ? 0 : (k == total - 1 ? 1 : -1);
  }
  c->mlp_adam_t += total;
  DevBuf<kmc::MlpStep> d_sched;
  DevBuf<unsigned long long> d_ctr;
  CK(c, upload(d_sched, sched.data(), sched.size(), c->stream));
  CK(c, d_ctr.alloc(1));
  CK(c, cudaMemsetAsync(d_ctr.p, 0, sizeof(unsigned long long), c->stream));
  auto epoch = [&]() -> cudaError_t {
    for (int64_t k = 0; k < per_epoch; ++k) {
      cudaError_t e = kmc::launch_mlp_grad(m, c->d_mlp_samples.p, k * cfg->batch, cfg->batch, c->d_mlp_part.p,
                                           c->d_mlp_ploss.p, grid, c->stream, d_ctr.p);
      if (e == cudaSuccess)
        e = kmc::launch_mlp_update(m, c->d_mlp_master.p, c->d_mlp_wbf.p, c->d_mlp_m1.p, c->d_mlp_m2.p,
                                   c->d_mlp_part.p, c->d_mlp_ploss.p, grid, kmc::MlpStep{}, nullptr, c->d_mlp_loss.p,
                                   c->stream, d_sched.p, d_ctr.p);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  };
  cudaGraphExec_t exec = nullptr;
  const bool graph = c->use_graph && per_epoch <= 1024 && cfg->epochs > 1;
  if (graph) {
    int rc = capture_graph(c, &exec, epoch);
    if (rc) return rc;
  }
  CK(c, cudaEventRecord(c->ev0, c->stream));
  for (int64_t e = 0; e < cfg->epochs; ++e) {
    cudaError_t err = graph ? cudaGraphLaunch(exec, c->stream) : epoch();
    if (err != cudaSuccess) {
      if (exec) cudaGraphExecDestroy(exec);
      CK(c, err);
    }
  }
  CK(c, cudaEventRecord(c->ev1, c->stream));
  double l[2] = {0, 0};
  CK(c, cudaMemcpyAsync(l, c->d_mlp_loss.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  float ms = 0;
  CK(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  if (exec) cudaGraphExecDestroy(exec);
  if (stats) {
    stats->steps = total;
    stats->first_loss = l[0];
    stats->last_loss = total > 1 ? l[1] : l[0];
    stats->seconds = ms * 1e-3;
  }
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_mlp_train");
}

int kmc_mlp_predict(kmc_ctx* c, int64_t n, const double* dist, const double* theta, const int32_t* pair,
                    double* log_rate) try {
  if (!c) return KMC_ERR_ARG;
  if (!c->mlp_ready) FAIL(c, KMC_ERR_STATE, "kmc_mlp_predict: call kmc_mlp_init first");
  if (n < 0 || (n > 0 && (!dist || !theta || !pair || !log_rate))) FAIL(c, KMC_ERR_ARG, "kmc_mlp_predict: bad arrays");
  if (n == 0) return KMC_OK;
  if (int rc = mlp_check_pairs(c, "kmc_mlp_predict", n, dist, theta, pair)) return rc;
  CK(c, cudaSetDevice(c->device));
  DevBuf<double> dd, dt, out;
  DevBuf<int32_t> dp;
  CK(c, upload(dd, dist, n, c->stream));
  CK(c, upload(dt, theta, n, c->stream));
  CK(c, upload(dp, pair, n, c->stream));
  CK(c, out.alloc(n));
  CK(c, kmc::launch_mlp_predict(mlp_dev(c), dd.p, dt.p, dp.p, n, out.p, c->stream));
  CK(c, cudaMemcpyAsync(log_rate, out.p, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_mlp_predict");
}

int kmc_mlp_rate_table(kmc_ctx* c, int32_t nd, const double* dist, int32_t nt, const double* theta, double* rate) try {
  if (!c) return KMC_ERR_ARG;
  if (!c->mlp_ready) FAIL(c, KMC_ERR_STATE, "kmc_mlp_rate_table: call kmc_mlp_init first");
  if (nd < 1 || nt < 1 || !dist || !theta || !rate) FAIL(c, KMC_ERR_ARG, "kmc_mlp_rate_table: empty grid");
  if ((int64_t)nd * nt > (int64_t(1) << 34) / ((int64_t)c->mlp_shape.n_species * c->mlp_shape.n_species))
    FAIL(c, KMC_ERR_ARG, "kmc_mlp_rate_table: more than 2^34 rates");
  for (int32_t i = 0; i < nd; ++i)
    if (!(dist[i] > 0) || !std::isfinite(dist[i])) FAIL(c, KMC_ERR_ARG, "kmc_mlp_rate_table: distance %d is %g", i, dist[i]);
  for (int32_t i = 0; i < nt; ++i)
    if (!std::isfinite(theta[i])) FAIL(c, KMC_ERR_ARG, "kmc_mlp_rate_table: angle %d is not finite", i);
  CK(c, cudaSetDevice(c->device));
  kmc::NvtxRange nv("kmc_mlp_rate_table");
  const int64_t S = c->mlp_shape.n_species;
  const int64_t n = S * S * nd * nt;
  DevBuf<double> dd, dt, out;
  CK(c, upload(dd, dist, nd, c->stream));
  CK(c, upload(dt, theta, nt, c->stream));
  CK(c, out.alloc(n));
  CK(c, kmc::launch_mlp_table(mlp_dev(c), dd.p, nd, dt.p, nt, out.p, c->stream));
  CK(c, cudaMemcpyAsync(rate, out.p, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_mlp_rate_table");
}

int kmc_set_launch_config(kmc_ctx* c, int32_t block, int32_t steps_per_launch) try {
  if (!c) return KMC_ERR_ARG;
  if (block < 32 || block > 256 || block % 32 || steps_per_launch < 1 || steps_per_launch > 1024) FAIL(c, KMC_ERR_ARG, "kmc_set_launch_config: bad values");
  c->block = block;
  c->steps_per_launch = steps_per_launch;
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(c, "kmc_set_launch_config");
}

}  // extern "C"
