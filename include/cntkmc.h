/* cntkmc.h -- C ABI of the GB300 exciton-hopping kinetic Monte Carlo engine.
 *
 * The reference (amirhosseindavoody/cnt_film_monte_carlo) has no plugin or FFI layer; its
 * boundary is the C++ class mc::monte_carlo driven by src/main.cpp:62-76.  Each entry point
 * below names the reference code it replaces.  Conventions:
 *   - every call returns int: KMC_OK (0) or a negative KMC_ERR_* code; kmc_last_error()
 *     gives the message of the last failure on that context; nothing throws across the ABI
 *     (a host allocation that fails inside a call is KMC_ERR_NOMEM, any other C++ exception
 *     KMC_ERR_ARG with its message);
 *   - plain pointers and sizes only; host buffers are copied in (the caller keeps them),
 *     device memory belongs to the context;
 *   - SI units (m, s, 1/s); positions [n][3] row-major;
 *   - one context per host thread; calls on one context are not reentrant.
 */
#ifndef CNTKMC_H
#define CNTKMC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KMC_OK 0
#define KMC_ERR_ARG (-1)       /* invalid argument or size */
#define KMC_ERR_CUDA (-2)      /* CUDA runtime failure (message has the CUDA error) */
#define KMC_ERR_STATE (-3)     /* call out of order (e.g. run before build) */
#define KMC_ERR_IO (-4)        /* file missing or malformed */
#define KMC_ERR_HOP_CAP (-5)   /* an exciton exceeded the per-step hop cap (device error word) */
#define KMC_ERR_NOMEM (-6)     /* device or host allocation failed */
#define KMC_ERR_NO_DEVICE (-7) /* no CUDA device / wrong architecture */
#define KMC_ERR_CAPACITY (-8)  /* contacts mode: more excitons than slots */
#define KMC_ERR_CHECK (-9)     /* libcntkmc_check.so only: a device bounds check failed (index or counter) */

#define KMC_TABLE_4D 4 /* rate(theta)(z_shift, axis_shift_1, axis_shift_2), nearest grid point */
#define KMC_TABLE_2D 2 /* rate(centre distance, folded angle in [0, pi/2]), nearest grid point */
#define KMC_TABLE_2D_SPECIES 3 /* one 2-D table per (donor, acceptor) chirality pair of the sites */
#define KMC_MAX_SPECIES 8      /* chiralities of a mixed film */

#define KMC_INJECT_REGION 0  /* reference Green-Kubo set-up: central cell of an n^3 split, removal slab */
#define KMC_INJECT_UNIFORM 1 /* every site is an injection site, nothing is removed */

#define KMC_PREC_FP64 0  /* plain FP64 hop kernel */
#define KMC_PREC_MIXED 1 /* FP32 cumulative rates with exact FP64 re-resolve; same hop sequence */

#define KMC_ORDER_AUTO (-1)  /* spatial order when there are several excitons per resident lane */
#define KMC_ORDER_SLOTS 0    /* excitons taken in slot order */
#define KMC_ORDER_SPATIAL 1  /* excitons taken in spatial order of their current site */

typedef struct kmc_ctx kmc_ctx;

/* One or more films (batched).  Sites of film f are [film_site_offsets[f], [f+1]); left/right
 * are film-local site indices or -1. */
typedef struct {
  int32_t n_films;
  const int64_t* film_site_offsets; /* [n_films + 1] */
  const double* pos;                /* [n_sites][3], metres */
  const double* orient;             /* [n_sites][3], unit tube axes */
  const int32_t* left;              /* [n_sites] */
  const int32_t* right;             /* [n_sites] */
} kmc_film;

/* Rate table (scattering_struct, src/monte_carlo/scattering_struct.h:21-52).  grid[d] has n[d]
 * points; rate is row-major [n0][n1][n2][n3] (4-D) or [n0][n1] (2-D).  KMC_TABLE_2D_SPECIES:
 * grids 0 and 1 as 2-D, n[2] = number of chiralities S, rate [S][S][n0][n1] (donor, acceptor,
 * distance, angle); the sites' chiralities come from kmc_set_site_species. */
typedef struct {
  int32_t kind;
  int32_t n[4];
  const double* grid[4];
  const double* rate;
} kmc_table;

typedef struct {
  int32_t mode;               /* KMC_INJECT_* */
  int32_t n_sections;         /* KMC_INJECT_REGION: odd n > 1 ("number of sections for injection region") */
  const int64_t* n_excitons;  /* [n_films] */
  const uint64_t* seeds;      /* [n_films] Philox key per film; exciton i of a film uses stream i */
} kmc_inject;

typedef struct {
  int64_t n_sites;
  int64_t nnz;           /* neighbour entries */
  double k_mean;         /* nnz / n_sites */
  int32_t k_max;
  int64_t n_cells;
  int64_t isolated;      /* sites with an empty neighbour list */
  int64_t exact_only;    /* sites whose row the mixed kernel always resolves in FP64 */
  double build_ms;       /* device time of cell binning + neighbour/rate build */
} kmc_nbr_stats;

typedef struct {
  int64_t hops;          /* update_state calls (dwell draws + cumulative-rate selections) */
  int64_t crossings;     /* moves onto the next segment by free flight along the tube */
  int64_t exact_resolves;/* mixed kernel: selections/comparisons re-resolved in FP64 */
  int64_t steps_done;    /* global time steps run so far */
  double last_run_ms;    /* device time of the last kmc_run (CUDA events) */
  int32_t last_launches; /* kernels launched by the last kmc_run */
} kmc_run_stats;

/* Context on CUDA device `device` (replaces mc::monte_carlo's constructor,
 * src/monte_carlo/monte_carlo.h:116-136, minus file-system work). status may be NULL. */
kmc_ctx* kmc_create(int device, int* status);
void kmc_destroy(kmc_ctx* ctx);
const char* kmc_last_error(const kmc_ctx* ctx);

/* Copy the film(s) to the device (replaces create_scatterers, monte_carlo.h:199-271, after
 * trim_scats :722-782, which the host applies with kmc_trim_sites). */
int kmc_load_film(kmc_ctx* ctx, const kmc_film* film);

/* Copy a rate table to the device (replaces set_scat_table, monte_carlo.h:419-423).  Reads
 * n[0] x n[1] (x n[2] x n[3] for kind 4; x S^2 for kind 3) rates; KMC_ERR_ARG for an empty grid
 * or more than 2^34 rates. */
int kmc_set_rate_table(kmc_ctx* ctx, const kmc_table* table);

/* Chirality index of every loaded site, species[n_sites] in [0, n_species) (no counterpart in
 * the reference, whose films hold one chirality).  A KMC_TABLE_2D_SPECIES table reads the pair
 * (species[donor], species[acceptor]).  Cleared by kmc_load_film. */
int kmc_set_site_species(kmc_ctx* ctx, const int32_t* species, int32_t n_species);

/* Cell binning and the per-site neighbour/rate CSR, built once on the device (replaces
 * create_scatterer_buckets monte_carlo.h:368-416, set_max_rate :426-440, and the per-hop
 * find_neighbors scatterer.cpp:34-83).  Neighbour order, rates and cumulative sums are those of
 * find_neighbors.  stats may be NULL. */
int kmc_build_neighbors(kmc_ctx* ctx, double max_hopping_radius, kmc_nbr_stats* stats);

/* Create the excitons (replaces injection_region / get_removal_domain / kubo_create_particles,
 * monte_carlo.cpp:203-251,308-316, and the particle constructor particle.h:48-52).  At most
 * 2^31 excitons over all films. */
int kmc_init_excitons(kmc_ctx* ctx, const kmc_inject* inject);

/* n_steps calls of kubo_step(dt) (monte_carlo.cpp:319-342; particle::step particle.cpp:57-80;
 * update_state scatterer.cpp:9-31; fly particle.cpp:9-54), velocity in m/s.  After each step the
 * sums sum_i dx_i^2, dy_i^2, dz_i^2 of every film are recorded (the numerators of
 * kubo_save_avg_dispalcement_squared, monte_carlo.cpp:382-409). */
int kmc_run(kmc_ctx* ctx, int64_t n_steps, double dt, double velocity, int32_t precision);

/* MSD sums of steps [first, first + count) for every film: out[f][s][3]. */
int kmc_get_msd(kmc_ctx* ctx, int64_t first, int64_t count, double* out);

/* MSD sums per exciton batch (no counterpart in the reference; used for the confidence interval
 * of D).  Exciton i of a film belongs to batch (i / 32) mod batches.  Set before
 * kmc_init_excitons (default 1).  out[f][s][batch][3]. */
int kmc_set_msd_batches(kmc_ctx* ctx, int32_t batches);
int kmc_get_msd_batches(kmc_ctx* ctx, int64_t first, int64_t count, double* out);

/* Diffusion coefficient from batch MSD curves (the reference plots MSD/t,
 * visualization/monte_carlo_results.py:478-500, and reports no fit): per batch and axis the
 * least-squares slope of <dx^2>(t) over the last `fit_fraction` of the steps, D = slope/2;
 * D[axis] = mean over batches, ci95[axis] = t(0.975, B-1) sd / sqrt(B).  msd is
 * [n_steps][batches][3] sums, counts[batch] the excitons per batch, times[n_steps] the step
 * end times.  Host-only. */
int kmc_fit_diffusion(const double* msd, const int64_t* counts, const double* times, int64_t n_steps,
                      int32_t batches, double fit_fraction, double D[3], double ci95[3]);

/* ---- contacts (steady-state flux) mode: the reference's second driver, src/main.cpp:85-106 ----
 * init (monte_carlo.h:157-195) up to the particles: y split into n_segments slabs; get_area
 * (:646-688); get_scatterer_statistics (:691-719); contact_scats of slab 1 and slab n (:494-517);
 * create_particles (:274-316), a linear profile from contact_pop[0] to contact_pop[1] excitons
 * per slab at random sites of the slab.  Then each step is step (:343-354: particle::step of
 * every exciton, nothing removed), save_metrics (:519-643: excitons per slab, net crossings of
 * every slab interface) and repopulate_contacts (:443-491: the excitons inside slab 1 are removed
 * and contact_pop[0] new ones placed at random contact-1 sites; then the same for slab n).
 * Excitons live in slots: slot k draws from Philox stream k (key `seed`) and keeps its draw
 * counter when its exciton is removed; the initial excitons take slots 0.. in create_particles
 * order and the new excitons of a contact the lowest empty slots, in order.  One film only;
 * kmc_get_excitons then reads every slot (site -1: empty). */
typedef struct {
  int32_t n_segments;     /* "number of segments" (2..4096) */
  int64_t contact_pop[2]; /* excitons kept in contact 1 / contact n (the reference: 1100, 0) */
  uint64_t seed;          /* Philox key */
  int64_t capacity;       /* exciton slots (0: 2 (initial + contact_pop[0] + contact_pop[1]), >= 1024) */
} kmc_contacts;

typedef struct {
  double ymin, ymax, dy;  /* domain in y and the slab width */
  int64_t n_initial;      /* excitons placed by create_particles */
  int64_t n_contact[2];   /* sites of contact 1 / contact n */
  int64_t capacity;       /* slots (a multiple of 32) */
} kmc_contacts_info;

/* Set up contacts mode after kmc_build_neighbors (replaces kmc_init_excitons).  info, area
 * [n_segments] (get_area) and stat_pop [n_segments] (sites per slab, get_scatterer_statistics)
 * may be NULL.  KMC_ERR_ARG when a slab or contact that must receive excitons has no site (the
 * reference divides by zero there). */
int kmc_contacts_init(kmc_ctx* ctx, const kmc_contacts* cfg, kmc_contacts_info* info, double* area, int64_t* stat_pop);

/* n_steps of step(dt) + save_metrics + repopulate_contacts, velocity in m/s.  population
 * [n_steps][n_segments]: excitons per slab after the step (the population file holds
 * count / (area dy)); current [n_steps][n_segments - 1]: net crossings of interface k
 * (y = ymin + dy (k + 1)) in +y during the step (the current file holds count / (interface area
 * dt)); n_live [n_steps]: excitons after repopulation.  Any output may be NULL. */
int kmc_contacts_run(kmc_ctx* ctx, int64_t n_steps, double dt, double velocity, int32_t precision,
                     int64_t* population, int64_t* current, int64_t* n_live);

/* track_particle (monte_carlo.h:786-818) for tracks first .. first + n_tracks - 1: one exciton
 * placed at a random contact-1 site and stepped (particle::step, plain FP64) until its y reaches
 * the last slab (y >= ymin + (n_segments - 1) dy), its position recorded after every step.  Track
 * k draws from Philox stream 2^32 + k (key: the contacts seed); the exciton slots are untouched.
 * The reference loops until the exciton arrives; here at most max_steps steps: len[t] = steps
 * recorded, arrived[t] = 1 when it reached the slab.  path [n_tracks][max_steps][3]. */
int kmc_contacts_track(kmc_ctx* ctx, int64_t first, int32_t n_tracks, double dt, double velocity, int64_t max_steps,
                       double* path, int64_t* len, int32_t* arrived);

/* Exciton state (film-major, exciton order).  Any pointer may be NULL.  pos/delta are [n][3]. */
int kmc_get_excitons(kmc_ctx* ctx, int32_t* site, double* pos, double* delta, double* ff, int32_t* heading,
                     uint64_t* draws, int64_t* hops);
/* Checkpoint/resume (no counterpart in the reference, whose runs are not resumable): writes the
 * state kmc_get_excitons returned back into the set kmc_init_excitons laid out with the same films,
 * exciton counts, seeds and injection mode.  site is film-local; heading 0/1; pos, delta finite;
 * ff finite and >= 0; hops >= 0; every array required.  draws is each exciton's Philox counter, so
 * the resumed run continues every random stream where the saved one stopped: k steps, save,
 * restore into a fresh context, n - k steps gives the state of n steps bit for bit.  The MSD bins
 * and run statistics start again at zero.  KMC_ERR_STATE before kmc_init_excitons or in contacts
 * mode; KMC_ERR_ARG on a bad field (nothing written). */
int kmc_set_excitons(kmc_ctx* ctx, const int32_t* site, const double* pos, const double* delta, const double* ff,
                     const int32_t* heading, const uint64_t* draws, const int64_t* hops);
int64_t kmc_num_excitons(const kmc_ctx* ctx);
int kmc_get_run_stats(kmc_ctx* ctx, kmc_run_stats* stats);

/* Device CSR copied out for inspection: rowptr [n_sites+1] (film-global), col (film-local site),
 * cum (FP64 cumulative rate), total [n_sites].  Any pointer may be NULL. */
int kmc_get_neighbors(kmc_ctx* ctx, int64_t* rowptr, int32_t* col, double* cum, double* total);

/* Hop trace of excitons [0, n_trace) of film 0, cap entries each (must be set before
 * kmc_init_excitons): update_state result -> site; free-flight crossing -> -1 - site;
 * reinjection -> INT32_MIN then the new site.  get returns the number of events recorded.
 * KMC_ERR_ARG for negative sizes or n_trace x cap above 2^36 entries. */
int kmc_set_trace(kmc_ctx* ctx, int64_t n_trace, int64_t cap);
int64_t kmc_get_trace(kmc_ctx* ctx, int64_t exciton, int32_t* out, int64_t cap);

/* Per-step hop cap per exciton (default 1e8); exceeding it makes kmc_run return KMC_ERR_HOP_CAP. */
int kmc_set_hop_cap(kmc_ctx* ctx, int64_t cap);

/* ---- host-side reference algorithms (no device needed) ---- */

/* trim_scats (monte_carlo.h:722-782): remove sites outside lim = {xmin,xmax,ymin,ymax,zmin,zmax}
 * by swapping them to the end and repairing tube links; arrays are permuted in place and
 * *n_out gets the number kept.  KMC_ERR_ARG (nothing changed) when n > 2^31 - 1 or a link is
 * neither -1 nor a site index below n. */
int kmc_trim_sites(int64_t n, double* pos, double* orient, int32_t* left, int32_t* right, const double lim[6],
                   int64_t* n_out);

/* Domain of a site set (find_simulation_domain, monte_carlo.h:328-340): mn[3], mx[3]. */
int kmc_domain(int64_t n, const double* pos, double mn[3], double mx[3]);

/* The 2-D (centre distance, folded angle) Förster-form table of the benchmark films (no counterpart
 * in the reference, which tabulates 4-D): the formula of create_forster_scatt_table
 * (monte_carlo.cpp:174-187) at zero axis shifts, gamma_0 cos^2(theta) (1 nm / d)^6, on
 * arma::linspace grids {start, end, n} (distance in m, theta in degrees scaled by 3.141592/180).
 * Outputs: dist[nd], theta[nt], rate[nd][nt].  The C++ and Python drivers both use it.
 * KMC_ERR_ARG unless each n is a number in [1, 2^31 - 1]. */
int kmc_forster2d_table(double gamma_0, const double distance[3], const double theta_deg[3], double* dist,
                        double* theta, double* rate);

/* create_forster_scatt_table (monte_carlo.cpp:156-200) on arma::linspace grids {start, end, n};
 * the theta grid is in degrees and scaled by pi/180 with pi = 3.141592 (helper/constants.h:10).
 * Outputs: grids theta[nt], zsh[nz], ash1[n1], ash2[n2]; rate[nt][nz][n1][n2].
 * KMC_ERR_ARG unless each n is a number in [1, 2^31 - 1]. */
int kmc_forster_table(double gamma_0, const double theta_deg[3], const double zshift[3], const double ash1[3],
                      const double ash2[3], double* theta, double* zsh, double* a1, double* a2, double* rate);

/* Mesh directory (single_cnt.{pos,orient}.{x,y,z}.dat, monte_carlo.h:199-271): first call with
 * NULL arrays returns *n_tubes and *n_points; second call fills pos/orient [n][3] (pos in m)
 * and left/right.  KMC_ERR_IO when a file is missing, holds a token that is not a number, has
 * rows of different lengths or a shape unlike the others, or holds more than 2^31 - 1 points. */
int kmc_read_mesh(const char* dir, int64_t* n_tubes, int64_t* n_points, double* pos, double* orient,
                  int32_t* left, int32_t* right);

/* ---- diagnostics and tuning (no counterpart in the reference) ---- */

/* Check the division-free dwell uniform RN(r / RAND_MAX) of the mixed kernel against IEEE
 * division, and its dwell-time log (specialised to these uniforms) against the general device
 * log, on the device for r in [r0, r0 + count); *mismatches gets the number of differences. */
int kmc_selftest_uniform(kmc_ctx* ctx, uint32_t r0, uint64_t count, uint64_t* mismatches);

/* L2 read bandwidth of this GPU (no counterpart in the reference; the denominator of the L2
 * roofline of films whose rows stay in L2): 16-byte L2-only loads streamed over an L2-resident
 * buffer of `bytes` (>= 1 MiB, a multiple of 16), reps passes timed with CUDA events; GB/s. */
int kmc_probe_l2(kmc_ctx* ctx, int64_t bytes, int32_t reps, double* gbs);

/* Evaluate the engine's device log and acos on x[n] (for accuracy tests). */
int kmc_math_probe(kmc_ctx* ctx, const double* x, int64_t n, double* log_out, double* acos_out);

/* Hop-kernel launch shape: threads per block (multiple of 32, <= 256) and Green-Kubo steps per
 * launch (the kernel keeps excitons in registers across the steps of one launch). */
int kmc_set_launch_config(kmc_ctx* ctx, int32_t block, int32_t steps_per_launch);

/* Mixed kernel variant (threads per block x resident blocks per SM the kernel's registers are
 * budgeted for): 0 = 128 x 4, 1 = 128 x 6, 2 = 128 x 8, 3 = 256 x 3, 4 = 768 x 1,
 * 5 = 1024 x 1.  Larger blocks stage the log table fewer times per SM and leave more L1 cache. */
int kmc_set_mixed_variant(kmc_ctx* ctx, int32_t variant);

/* Order in which the mixed kernel takes excitons (no counterpart in the reference, whose OpenMP
 * loop runs the particles in index order): KMC_ORDER_AUTO (default), _SLOTS or _SPATIAL.  In
 * spatial order the slots are re-sorted before every launch by the storage slot of their current
 * site (sites are stored in tiles of 16 x 16 cell columns, z innermost, film by film), so the
 * excitons in flight together hop over a compact region whose rows stay in L1/L2.  Results never
 * depend on it. */
int kmc_set_work_order(kmc_ctx* ctx, int32_t mode);
/* The order the next mixed run will use: KMC_ORDER_SLOTS or KMC_ORDER_SPATIAL. */
int kmc_get_work_order(kmc_ctx* ctx, int32_t* in_effect);

/* Capture each kmc_run's launch sequence into a CUDA graph and replay it (default on; the graph
 * of the previous run is updated in place when its shape matches).  on = 0 launches directly. */
int kmc_set_graph(kmc_ctx* ctx, int32_t on);

typedef struct {
  int32_t variant;
  int32_t steps_per_launch;
  double hops_per_s;
} kmc_tune_result;

/* Time every mixed-kernel variant with 1, 8 and 32 steps per launch for trial_steps steps of dt
 * on the current excitons (their state is saved and restored; no MSD step is recorded) and keep
 * the fastest.  Results never depend on the choice. */
int kmc_autotune(kmc_ctx* ctx, double dt, double velocity, int64_t trial_steps, kmc_tune_result* out);

/* ---- neighbour lists without device allocation (no counterpart in the reference) ----
 *
 * For callers that cannot call cudaMalloc: applications whose device memory is handed out by
 * their own pool or a pre-reserved arena, or hosts that forbid allocation (which synchronises
 * the device) while they run.  Builds the neighbour/rate CSR of ONE film exactly as
 * kmc_build_neighbors does (same order, rates and FP64 cumulative sums), into the caller's
 * device buffers, and allocates nothing: no cudaMalloc/cudaFree, no allocating library call.
 *   inputs  (device): pos [n][3] in m, orient [n][3]; table->grid[d] and table->rate are device
 *                     pointers (same layout as kmc_table);
 *   outputs (device): rowptr [n+1], col [capacity] (site ids), cum [capacity], total [n];
 *   *nnz (host) receives the number of neighbour entries; if it exceeds `capacity` the call
 *   returns KMC_ERR_ARG after writing rowptr, so a caller can size col/cum and call again.
 *   stream: a cudaStream_t (NULL: the default stream); the call returns after the stream has
 *   finished its work.  err/err_len: optional buffer for a message.
 * Limits: n_sites <= KMC_NOALLOC_MAX_SITES and the film's cell grid (cells of side
 * max_hopping_radius) <= KMC_NOALLOC_MAX_CELLS; larger inputs are rejected with KMC_ERR_ARG.
 * Intermediate storage is one fixed device array (about 1.3 MB) that every GPU loading this
 * library keeps until exit.  The first call on a device looks up that array's address with the
 * device current; make it before any stream capture, and do not call again on a device after
 * cudaDeviceReset (the address is kept for the process).  All calls share the array (each
 * clears what must start at zero); calls that overlap on the GPU race and must be serialised. */
#define KMC_NOALLOC_MAX_SITES 65536
#define KMC_NOALLOC_MAX_CELLS 65536
int kmc_build_neighbors_noalloc(const double* pos, const double* orient, int64_t n_sites, const kmc_table* table,
                                double max_hopping_radius, int64_t* rowptr, int32_t* col, double* cum, double* total,
                                int64_t capacity, int64_t* nnz, void* stream, char* err, int64_t err_len);

/* ---- learned pair-rate surrogate (no counterpart in the reference) ----
 *
 * Rates of mixed-chirality films come from a small network instead of one exciton_transfer table
 * per chirality pair (exciton_transfer.cpp:380-441 computes one pair's table).  The network maps
 * (centre distance d, folded angle theta, chirality pair) to the normalised log-rate
 * y = (ln rate - log_mean) / log_scale: 4 inputs (2 ln(d / d_min) / ln(d_max / d_min) - 1,
 * 2 theta / (pi/2) - 1, and a learned 2-wide embedding of the ordered pair donor * S + acceptor),
 * two hidden layers of 64 with GELU (tanh form), one output.  The three weight matrices are held
 * in BF16 (with FP32 master copies for training); biases and the embedding are FP32; every sum is
 * FP32.  Parameters form one FP32 vector of KMC_MLP_PARAMS(S) values: W1[64][4] at 0, b1[64] at
 * 256, W2[64][64] (row = output unit) at 320, b2[64] at 4416, W3[64] at 4480, b3 at 4544, three
 * unused, E[S*S][2] at 4548.  Training is deterministic: same samples, parameters and
 * configuration give the same weights on the same GPU model. */
#define KMC_MLP_HIDDEN 64
#define KMC_MLP_PARAMS(S) (4548 + 2 * (S) * (S))

typedef struct {
  int32_t n_species;           /* S, 1..KMC_MAX_SPECIES */
  double d_min, d_max;         /* m: distance range of the log-distance input */
  double log_mean, log_scale;  /* output scaling of ln(rate) */
} kmc_mlp_shape;

/* A closed-form chirality labeller, much cheaper than exciton_transfer's first-order rate
 * (kmc_exciton_rates, which labels the surrogate for mixed films): the Förster formula of
 * create_forster_scatt_table (monte_carlo.cpp:174-187) at zero axis shifts, extended by chirality:
 *   rate = gamma_0 s_ab (cos^2 theta + floor) (1 nm / sqrt(d^2 + near_field^2))^6,
 *   s_ab = (D_a D_b / D_ref^2) exp(-dE^2 / (2 width^2)) min(1, exp(-dE / kT)), dE = E_b - E_a,
 * for donor a and acceptor b.  Equal energies and diameters with floor = near_field = 0 give
 * kmc_forster2d_table's values bit for bit. */
typedef struct {
  int32_t n_species;       /* S */
  double gamma_0;          /* 1/s */
  const double* energy;    /* [S] exciton energies, eV */
  const double* diameter;  /* [S] tube diameters, m */
  double diameter_ref;     /* m */
  double width;            /* eV */
  double kT;               /* eV */
  double floor;            /* added to cos^2(theta) */
  double near_field;       /* m */
} kmc_species_model;

/* Host labeller: rate[i] for donor[i] -> acceptor[i] at dist[i] (m) and theta[i] (rad). */
int kmc_species_rates(const kmc_species_model* model, int64_t n, const double* dist, const double* theta,
                      const int32_t* donor, const int32_t* acceptor, double* rate);

/* The network of a context: shape and parameters drawn uniformly in +-1/sqrt(fan-in) (the
 * embedding in +-1, b3 = 0) from a SplitMix64 stream of `seed`; training state reset. */
int kmc_mlp_init(kmc_ctx* ctx, const kmc_mlp_shape* shape, uint64_t seed);
/* Replace / read the FP32 master parameters (n = KMC_MLP_PARAMS(S)); set also resets Adam. */
int kmc_mlp_set_params(kmc_ctx* ctx, const float* params, int64_t n);
int kmc_mlp_get_params(kmc_ctx* ctx, float* params, int64_t n);

/* Labelled samples kept on the device: dist (m), folded theta (rad), pair = donor * S + acceptor,
 * log_rate = ln(rate). */
int kmc_mlp_set_samples(kmc_ctx* ctx, int64_t n, const double* dist, const double* theta, const int32_t* pair,
                        const double* log_rate);

/* Mean squared error of y against the normalised labels of samples [first, first + count) and its
 * gradient grad[KMC_MLP_PARAMS(S)] with respect to the parameters (BF16 weights' gradient);
 * parameters are not changed. */
int kmc_mlp_gradient(kmc_ctx* ctx, int64_t first, int64_t count, float* grad, double* loss);

typedef struct {
  int32_t epochs;
  int32_t batch;            /* samples per step, a multiple of 128, <= number of samples */
  double lr, lr_final;      /* Adam step size, cosine schedule from lr to lr_final */
  double beta1, beta2, eps; /* Adam moments */
} kmc_mlp_train_cfg;

typedef struct {
  int64_t steps;
  double first_loss, last_loss; /* mean squared error of the first and the last step's batch */
  double seconds;               /* device time of the whole training (CUDA events) */
} kmc_mlp_train_stats;

/* Adam training over the samples: epochs x floor(n / batch) steps, batch k of an epoch being
 * samples [k batch, (k + 1) batch).  Continues from the current parameters and Adam moments. */
int kmc_mlp_train(kmc_ctx* ctx, const kmc_mlp_train_cfg* cfg, kmc_mlp_train_stats* stats);

/* Predicted ln(rate) for n pairs. */
int kmc_mlp_predict(kmc_ctx* ctx, int64_t n, const double* dist, const double* theta, const int32_t* pair,
                    double* log_rate);

/* A KMC_TABLE_2D_SPECIES rate table from the network: rate[S][S][nd][nt] = exp(predicted ln rate)
 * on the grids dist[nd] (m) and theta[nt] (rad); at most 2^34 rates. */
int kmc_mlp_rate_table(kmc_ctx* ctx, int32_t nd, const double* dist, int32_t nt, const double* theta, double* rate);

/* Library version string. */
const char* kmc_version(void);

/* ---- exciton-transfer physics: the labeller of pair transfer rates ----
 *
 * The reference computes pair rates from a tight-binding / Bethe-Salpeter exciton model of each
 * tube (src/exciton_transfer/cnt.cpp) and the first-order (Foerster-like) transfer rate between
 * two tubes (src/exciton_transfer/exciton_transfer.cpp); its "davoody" rate table fills the 4-D
 * scattering table with that rate (src/monte_carlo/monte_carlo.cpp:64-153).  Here the sums run on
 * the GPU: vq, the polarisation, the Bethe-Salpeter kernels and their eigen-decompositions when a
 * tube is created, and the Coulomb sum J of every matched state pair at every geometry.
 * A geometry is (z_shift [m], axis shift 1 [m], axis shift 2 [m], theta [rad]) as in
 * exciton_transfer::first_order: the donor along y shifted by axis shift 1, the acceptor shifted
 * by axis shift 2 along its own axis and by z_shift in z, then rotated by theta about z. */
typedef struct kmc_cnt kmc_cnt;

#define KMC_CNT_MAX_RELEVANT 64 /* relevant states per valley (1 eV window): tubes up to ~80 nm */

typedef struct {
  int32_t n, m, cells, Nu, M, Q, t1, t2; /* chirality, length in unit cells, cnt parameters */
  int32_t nk, n_mu;                      /* K2-extended grid */
  int32_t n_valley_pairs, n_relevant;    /* valley pairs; relevant states per valley */
  int32_t iq0, nq, mq0, nmq;             /* vq / PI / eps grid: iq in [iq0, iq0 + nq), mu likewise */
  int32_t ik_cm0, nk_cm;                 /* exciton centre-of-mass momenta */
  double radius, length, area_u;         /* m, m (cells x |T|), m^2 (graphene unit cell) */
} kmc_cnt_info;

/* What kmc_cnt_get_array copies out (doubles unless noted; complex as (re, im) pairs):
 * GEOMETRY [26]: a1, a2, b1, b2, aCC, ch, t_vec, K1, K2, dk_l (2 each), t_vec_3d (3), radius,
 *   |ch|, length; POS_U_3D [Nu][3]; BANDS [2][nk][n_mu] (valence, conduction); VALLEYS int32
 *   [n_valley_pairs][2][2] (ik, mu); RELEVANT int32 [2][n_relevant][2]; VQ complex
 *   [nq][nmq][4]; PI, EPS [nq][nmq]; A1, A2_TRIPLET, A2_SINGLET [nk_cm][n_relevant] (J);
 *   IK_IDX int32 [nk_cm][4][2 n_relevant]; Q_PARTIAL complex [nk_cm][n_relevant]. */
#define KMC_CNT_GEOMETRY 0
#define KMC_CNT_POS_U_3D 1
#define KMC_CNT_BANDS 2
#define KMC_CNT_VALLEYS 3
#define KMC_CNT_RELEVANT 4
#define KMC_CNT_VQ 5
#define KMC_CNT_PI 6
#define KMC_CNT_EPS 7
#define KMC_CNT_A1 8
#define KMC_CNT_A2_TRIPLET 9
#define KMC_CNT_A2_SINGLET 10
#define KMC_CNT_IK_IDX 11
#define KMC_CNT_Q_PARTIAL 12

typedef struct {
  double temperature;  /* K ("temperature", exciton_transfer.h:85-90; the table uses 300) */
  double broadening;   /* J, Lorentzian half width (exciton_transfer.h:93-97; the table uses 4 meV) */
  int32_t precision;   /* KMC_PREC_FP64: J in FP64; KMC_PREC_MIXED: FP32 positions and tile sums */
} kmc_transfer_cfg;

/* cnt(json) + cnt::calculate_exciton_dispersion (cnt.h:146-187, cnt.cpp:1056-1080): the exciton
 * model of an (n, m) tube of length_cells unit cells, computed on the context's GPU.  The model
 * lives in host memory; destroy it with kmc_cnt_destroy. */
int kmc_cnt_create(kmc_ctx* ctx, int32_t n, int32_t m, int32_t length_cells, kmc_cnt** out);
void kmc_cnt_destroy(kmc_cnt* tube);
int kmc_cnt_get_info(const kmc_cnt* tube, kmc_cnt_info* info);
/* Copy one of the model's arrays (KMC_CNT_*); count must equal its number of values. */
int kmc_cnt_get_array(const kmc_cnt* tube, int32_t which, void* out, int64_t count);
/* exciton_transfer::calculate_J (exciton_transfer.cpp:307-377) for n_pairs (donor ik_cm,
 * acceptor ik_cm) pairs at one geometry; j_out complex [n_pairs][2]. */
int kmc_exciton_j(kmc_ctx* ctx, const kmc_cnt* donor, const kmc_cnt* acceptor, int64_t n_pairs,
                  const int32_t* ik_cm_pairs, const double geometry[4], int32_t precision, double* j_out);
/* exciton_transfer::first_order (exciton_transfer.cpp:380-424) at n_geometries geometries
 * [n][4]; rate [n] in 1/s. */
int kmc_exciton_rates(kmc_ctx* ctx, const kmc_cnt* donor, const kmc_cnt* acceptor, const kmc_transfer_cfg* cfg,
                      int64_t n_geometries, const double* geometries, double* rate);
/* monte_carlo::create_davoody_scatt_table (monte_carlo.cpp:64-153): the first-order rate on the
 * 4-D grid theta (degrees, scaled by the reference's pi / 180) x z_shift x axis shift 1 x axis
 * shift 2 ({start, end, count} linspace each); outputs the grids and rate [nt][nz][n1][n2],
 * the layout of a KMC_TABLE_4D table.  KMC_ERR_ARG unless each count is a number in
 * [1, 2^31 - 1] and the table has at most 2^34 entries. */
int kmc_davoody_table(kmc_ctx* ctx, const kmc_cnt* donor, const kmc_cnt* acceptor, const kmc_transfer_cfg* cfg,
                      const double theta_deg[3], const double zshift[3], const double ash1[3], const double ash2[3],
                      double* theta, double* zsh, double* a1, double* a2, double* rate);

#ifdef __cplusplus
}
#endif

#endif /* CNTKMC_H */
