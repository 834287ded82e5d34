// kmc_noalloc.cu -- kmc_build_neighbors_noalloc: the neighbour/rate CSR of one film written into
// caller-provided device buffers without allocating any device memory.
//
// Who needs it: callers whose device memory is owned by someone else -- an application that
// hands out all device memory from its own pool or pre-reserved arena, a host framework that
// forbids cudaMalloc/cudaFree once it is running (they synchronise the device and can fail
// mid-run) -- can still build neighbour lists.  They pass inputs and outputs in their own
// device buffers; the build's intermediate storage (cell ids, cell members, cell offsets and
// the domain reduction) lives in one file-scope __device__ array of fixed size, which every
// GPU that loads this library holds until the process exits.
//
// Limits: at most KMC_NOALLOC_MAX_SITES sites and KMC_NOALLOC_MAX_CELLS cells (cells of side
// max_hopping_radius over the film's bounding box); larger inputs are rejected with
// KMC_ERR_ARG and a message.  The first call on a device looks up the array's device address
// (cudaGetSymbolAddress) with that device current; make that first call before any stream
// capture.  The address is kept for the life of the process, so the entry point must not be
// called again on a device after cudaDeviceReset (the library's module, and the array with it,
// is reloaded at a new address).  All calls share the one array, and each call clears what must
// start at zero; calls whose GPU work overlaps (different streams or host threads on the same
// device) race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/cntkmc.h"
#include "kmc_abi_guard.h"
#include "kmc_internal.h"
#include "kmc_pair.cuh"

namespace {

using namespace kmc;

struct NoAllocScratch {
  int32_t cell_of[KMC_NOALLOC_MAX_SITES];
  int32_t members[KMC_NOALLOC_MAX_SITES];
  int32_t sorted[KMC_NOALLOC_MAX_SITES];  // members of a cell in site order, before the copy back
  int32_t cell_start[KMC_NOALLOC_MAX_CELLS + 1];
  int32_t cursor[KMC_NOALLOC_MAX_CELLS];
  unsigned long long dom[6];  // order-preserving keys of min x,y,z and max x,y,z
  int32_t err;
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

constexpr int kMaxDevices = 64;
std::mutex g_lock;
NoAllocScratch* g_scratch_ptr[kMaxDevices] = {nullptr};

// order-preserving map of doubles to unsigned keys (for atomicMin / atomicMax)
__device__ __forceinline__ unsigned long long dkey(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ __forceinline__ double dkey_inv(unsigned long long k) {
  unsigned long long b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
  double x;
  memcpy(&x, &b, 8);
  return x;
}

__global__ void k_na_reset(NoAllocScratch* sc, int32_t n_cells) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i <= n_cells) sc->cell_start[i] = 0;
  if (i < n_cells) sc->cursor[i] = 0;
  if (i == 0) sc->err = 0;
}

__global__ void k_na_domain_init(NoAllocScratch* sc) {
  if (threadIdx.x < 3) sc->dom[threadIdx.x] = ~0ull;
  else if (threadIdx.x < 6) sc->dom[threadIdx.x] = 0ull;
}

// find_simulation_domain (monte_carlo.h:328-340): exact min/max, order independent
__global__ void k_na_domain(const double* __restrict__ pos, int64_t n, NoAllocScratch* sc) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  for (int c = 0; c < 3; ++c) {
    unsigned long long k = dkey(pos[3 * s + c]);
    atomicMin(&sc->dom[c], k);
    atomicMax(&sc->dom[3 + c], k);
  }
}

struct NaGrid {
  double mn[3];
  double r;
  int32_t nx, ny, nz, n_cells;
};

// cell of each site (monte_carlo.h:389-395; the conversion to int truncates)
__global__ void k_na_cells(const double* __restrict__ pos, int64_t n, NaGrid g, NoAllocScratch* sc) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  int ix = (int)((pos[3 * s] - g.mn[0]) / g.r);
  int iy = (int)((pos[3 * s + 1] - g.mn[1]) / g.r);
  int iz = (int)((pos[3 * s + 2] - g.mn[2]) / g.r);
  if (ix < 0 || iy < 0 || iz < 0 || ix >= g.nx || iy >= g.ny || iz >= g.nz) {
    atomicOr(&sc->err, 1);
    ix = min(max(ix, 0), g.nx - 1);
    iy = min(max(iy, 0), g.ny - 1);
    iz = min(max(iz, 0), g.nz - 1);
  }
  int32_t c = ix + iy * g.nx + iz * g.nx * g.ny;
  sc->cell_of[s] = c;
  atomicAdd(&sc->cell_start[c], 1);
}

// exclusive scan of n <= 65537 values with one block of 1024 threads
template <typename T>
__global__ void k_na_scan(T* data, int64_t n) {
  __shared__ T part[1024];
  const int t = threadIdx.x;
  const int64_t per = (n + 1023) / 1024;
  const int64_t b = t * per, e = min(b + per, n);
  T sum = 0;
  for (int64_t i = b; i < e; ++i) sum += data[i];
  part[t] = sum;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    T v = t >= o ? part[t - o] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  T run = part[t] - sum;
  for (int64_t i = b; i < e; ++i) {
    T v = data[i];
    data[i] = run;
    run += v;
  }
}

__global__ void k_na_scatter(int64_t n, NoAllocScratch* sc) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  int32_t c = sc->cell_of[s];
  int32_t k = atomicAdd(&sc->cursor[c], 1);
  sc->members[sc->cell_start[c] + k] = (int32_t)s;
}

// Members back into site order (push_back order of monte_carlo.h:389-395): one block per cell.
// Site ids are distinct, so a member's place is the number of members with a smaller id; each
// thread counts that for its members against the cell's members staged through shared memory,
// tile by tile, and writes them to `sorted`, which the block then copies back.  m members cost
// m^2 / blockDim comparisons per thread from shared memory (a whole 65,536-site film in one cell:
// ~17 M per thread), against m^2 dependent global accesses for a per-cell insertion sort.
constexpr int kNaSortThreads = 256;
constexpr int kNaSortTile = 2048;
__global__ void __launch_bounds__(kNaSortThreads) k_na_sort(NoAllocScratch* sc) {
  __shared__ int32_t tile[kNaSortTile];
  const int32_t c = blockIdx.x;
  const int32_t b = sc->cell_start[c], m = sc->cell_start[c + 1] - b;
  if (m < 2) return;  // uniform over the block
  for (int32_t i0 = 0; i0 < m; i0 += kNaSortThreads) {
    const int32_t i = i0 + (int32_t)threadIdx.x;
    const int32_t v = i < m ? sc->members[b + i] : 0;
    int32_t rank = 0;
    for (int32_t t0 = 0; t0 < m; t0 += kNaSortTile) {
      const int32_t nt = min(kNaSortTile, m - t0);
      __syncthreads();
      for (int32_t j = threadIdx.x; j < nt; j += kNaSortThreads) tile[j] = sc->members[b + t0 + j];
      __syncthreads();
      if (i < m)
        for (int32_t j = 0; j < nt; ++j) rank += tile[j] < v ? 1 : 0;
    }
    if (i < m) sc->sorted[b + rank] = v;
  }
  __syncthreads();  // the block's writes to `sorted` are visible to the whole block
  for (int32_t i = threadIdx.x; i < m; i += kNaSortThreads) sc->members[b + i] = sc->sorted[b + i];
}

// neighbours of site s in find_neighbors order (scatterer.cpp:34-83; cells x-outer, y, z-inner)
template <typename F>
__device__ __forceinline__ void na_for_each(const double* __restrict__ pos, int64_t s, const NaGrid& g,
                                            double r_max, const NoAllocScratch* sc, F fn) {
  double4_32a p1 = make_double4_32a(pos[3 * s], pos[3 * s + 1], pos[3 * s + 2], 0.0);
  int32_t c0 = sc->cell_of[s];
  int ix = c0 % g.nx, iy = (c0 / g.nx) % g.ny, iz = c0 / (g.nx * g.ny);
  for (int i = ix - 1; i <= ix + 1; ++i) {
    if (i < 0 || i >= g.nx) continue;
    for (int j = iy - 1; j <= iy + 1; ++j) {
      if (j < 0 || j >= g.ny) continue;
      for (int k = iz - 1; k <= iz + 1; ++k) {
        if (k < 0 || k >= g.nz) continue;
        int32_t c = i + j * g.nx + k * g.nx * g.ny;
        for (int32_t m = sc->cell_start[c], e = sc->cell_start[c + 1]; m < e; ++m) {
          int32_t q = sc->members[m];
          double4_32a p2 = make_double4_32a(pos[3 * q], pos[3 * q + 1], pos[3 * q + 2], 0.0);
          double dR0 = p1.x - p2.x, dR1 = p1.y - p2.y, dR2 = p1.z - p2.z;
          double distance = norm3(dR0, dR1, dR2);
          if ((distance < r_max) && (distance > kMinHopDist)) fn(q, p1, p2, dR0, dR1, dR2, distance);
        }
      }
    }
  }
}

__global__ void k_na_count(const double* __restrict__ pos, int64_t n, NaGrid g, double r_max,
                           const NoAllocScratch* sc, int64_t* rowptr) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s > n) return;
  if (s == n) {
    rowptr[n] = 0;
    return;
  }
  int64_t cnt = 0;
  na_for_each(pos, s, g, r_max, sc,
              [&](int32_t, const double4_32a&, const double4_32a&, double, double, double, double) { ++cnt; });
  rowptr[s] = cnt;
}

__global__ void k_na_fill(const double* __restrict__ pos, const double* __restrict__ orient, int64_t n, NaGrid g,
                          double r_max, TableDev table, const NoAllocScratch* sc, const int64_t* rowptr, int32_t* col,
                          double* cum, double* total) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  double a1v[3] = {orient[3 * s], orient[3 * s + 1], orient[3 * s + 2]};
  int64_t b = rowptr[s], k = 0;
  double run = 0.0;
  na_for_each(pos, s, g, r_max, sc,
              [&](int32_t q, const double4_32a& p1, const double4_32a& p2, double dR0, double dR1, double dR2,
                  double distance) {
                double a2v[3] = {orient[3 * (int64_t)q], orient[3 * (int64_t)q + 1], orient[3 * (int64_t)q + 2]};
                double rate = pair_rate(table, p1, a1v, p2, a2v, dR0, dR1, dR2, distance);
                run = (k == 0) ? rate : run + rate;  // inclusive prefix sum, scatterer.cpp:78-80
                col[b + k] = q;
                cum[b + k] = run;
                ++k;
              });
  total[s] = k > 0 ? run : 0.0;
}

int fail(char* err, int64_t err_len, int code, const char* msg) {
  if (err && err_len > 0) {
    std::strncpy(err, msg, (size_t)err_len - 1);
    err[err_len - 1] = 0;
  }
  return code;
}

}  // namespace

extern "C" int kmc_build_neighbors_noalloc(const double* pos, const double* orient, int64_t n_sites,
                                           const kmc_table* table, double max_hopping_radius, int64_t* rowptr,
                                           int32_t* col, double* cum, double* total, int64_t capacity,
                                           int64_t* nnz, void* stream, char* err, int64_t err_len) try {
  char msg[256];
  if (!pos || !orient || !table || !rowptr || !total || !nnz || capacity < 0)
    return fail(err, err_len, KMC_ERR_ARG, "kmc_build_neighbors_noalloc: missing argument");
  if (n_sites < 1 || n_sites > KMC_NOALLOC_MAX_SITES) {
    std::snprintf(msg, sizeof msg, "kmc_build_neighbors_noalloc: %lld sites; this entry point takes 1..%d",
                  (long long)n_sites, KMC_NOALLOC_MAX_SITES);
    return fail(err, err_len, KMC_ERR_ARG, msg);
  }
  if (!(max_hopping_radius > 0)) return fail(err, err_len, KMC_ERR_ARG, "kmc_build_neighbors_noalloc: radius must be positive");
  if (table->kind != KMC_TABLE_4D && table->kind != KMC_TABLE_2D)
    return fail(err, err_len, KMC_ERR_ARG, "kmc_build_neighbors_noalloc: table kind must be 4 or 2");
  TableDev td{};
  td.kind = table->kind;
  for (int d = 0; d < (table->kind == KMC_TABLE_4D ? 4 : 2); ++d) {
    if (table->n[d] < 1 || !table->grid[d]) return fail(err, err_len, KMC_ERR_ARG, "kmc_build_neighbors_noalloc: empty grid");
    td.n[d] = table->n[d];
    td.grid[d] = table->grid[d];
  }
  if (!table->rate) return fail(err, err_len, KMC_ERR_ARG, "kmc_build_neighbors_noalloc: missing rates");
  td.rate = table->rate;
  cudaStream_t st = (cudaStream_t)stream;
  kmc::NvtxRange nv("kmc_build_neighbors_noalloc");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(err, err_len, KMC_ERR_NO_DEVICE, "kmc_build_neighbors_noalloc: no current CUDA device");
  NoAllocScratch* sc = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_lock);
    if (!g_scratch_ptr[dev]) {  // once per device, with that device current
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) {
        std::snprintf(msg, sizeof msg, "kmc_build_neighbors_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        return fail(err, err_len, KMC_ERR_CUDA, msg);
      }
      g_scratch_ptr[dev] = static_cast<NoAllocScratch*>(p);
    }
    sc = g_scratch_ptr[dev];
  }
#define NA_CK(call)                                                                                         \
  do {                                                                                                      \
    cudaError_t _e = (call);                                                                                \
    if (_e != cudaSuccess) {                                                                                \
      std::snprintf(msg, sizeof msg, "kmc_build_neighbors_noalloc: %s: %s", #call, cudaGetErrorString(_e)); \
      return fail(err, err_len, KMC_ERR_CUDA, msg);                                                         \
    }                                                                                                       \
  } while (0)
  const unsigned nb = (unsigned)((n_sites + 255) / 256);
  // domain
  k_na_domain_init<<<1, 32, 0, st>>>(sc);
  k_na_domain<<<nb, 256, 0, st>>>(pos, n_sites, sc);
  NA_CK(cudaGetLastError());
  unsigned long long hk[6];
  NA_CK(cudaMemcpyAsync(hk, sc->dom, sizeof hk, cudaMemcpyDeviceToHost, st));
  NA_CK(cudaStreamSynchronize(st));
  NaGrid g;
  double mx[3];
  for (int c = 0; c < 3; ++c) {
    g.mn[c] = dkey_inv(hk[c]);
    mx[c] = dkey_inv(hk[3 + c]);
  }
  // cell grid, monte_carlo.h:375-387
  double nd[3];
  for (int c = 0; c < 3; ++c) nd[c] = std::ceil((mx[c] - g.mn[c]) / max_hopping_radius) + 1;
  if (!(nd[0] * nd[1] * nd[2] <= (double)KMC_NOALLOC_MAX_CELLS)) {
    std::snprintf(msg, sizeof msg,
                  "kmc_build_neighbors_noalloc: the film needs %.0f cells of side %g m; this entry point takes at most %d",
                  nd[0] * nd[1] * nd[2], max_hopping_radius, KMC_NOALLOC_MAX_CELLS);
    return fail(err, err_len, KMC_ERR_ARG, msg);
  }
  g.nx = (int32_t)nd[0];
  g.ny = (int32_t)nd[1];
  g.nz = (int32_t)nd[2];
  g.n_cells = g.nx * g.ny * g.nz;
  g.r = max_hopping_radius;
  // cells: counts, offsets, members in site order (the shared array keeps the previous call's
  // contents, so every counter used below is cleared first)
  k_na_reset<<<(unsigned)((g.n_cells + 1 + 255) / 256), 256, 0, st>>>(sc, g.n_cells);
  k_na_cells<<<nb, 256, 0, st>>>(pos, n_sites, g, sc);
  k_na_scan<int32_t><<<1, 1024, 0, st>>>(sc->cell_start, (int64_t)g.n_cells + 1);
  k_na_scatter<<<nb, 256, 0, st>>>(n_sites, sc);
  k_na_sort<<<(unsigned)g.n_cells, kNaSortThreads, 0, st>>>(sc);
  // row lengths -> row pointers (caller's buffer)
  k_na_count<<<(unsigned)((n_sites + 1 + 127) / 128), 128, 0, st>>>(pos, n_sites, g, max_hopping_radius, sc, rowptr);
  k_na_scan<int64_t><<<1, 1024, 0, st>>>(rowptr, n_sites + 1);
  NA_CK(cudaGetLastError());
  int64_t need = 0;
  int32_t herr = 0;
  NA_CK(cudaMemcpyAsync(&need, rowptr + n_sites, sizeof need, cudaMemcpyDeviceToHost, st));
  NA_CK(cudaMemcpyAsync(&herr, &sc->err, sizeof herr, cudaMemcpyDeviceToHost, st));
  NA_CK(cudaStreamSynchronize(st));
  *nnz = need;
  if (herr) return fail(err, err_len, KMC_ERR_ARG, "kmc_build_neighbors_noalloc: a site lies outside the cell grid (non-finite position?)");
  if (need > capacity) {
    std::snprintf(msg, sizeof msg, "kmc_build_neighbors_noalloc: %lld neighbour entries do not fit the capacity %lld",
                  (long long)need, (long long)capacity);
    return fail(err, err_len, KMC_ERR_ARG, msg);
  }
  if (need > 0 && (!col || !cum)) return fail(err, err_len, KMC_ERR_ARG, "kmc_build_neighbors_noalloc: missing col/cum");
  k_na_fill<<<(unsigned)((n_sites + 127) / 128), 128, 0, st>>>(pos, orient, n_sites, g, max_hopping_radius, td, sc,
                                                               rowptr, col, cum, total);
  NA_CK(cudaGetLastError());
  NA_CK(cudaStreamSynchronize(st));
#undef NA_CK
  return KMC_OK;
} catch (...) {
  const char* what = nullptr;
  const int code = kmc::abi_status(&what);
  return fail(err, err_len, code, what);
}
