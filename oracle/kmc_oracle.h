/* kmc_oracle.h -- TEST INFRASTRUCTURE: CPU restatement of the reference's exciton-hopping
 * hot path (amirhosseindavoody/cnt_film_monte_carlo, src/monte_carlo/).
 *
 * It is what the tests compare the CUDA engine with, and the "port" CPU baseline of the benchmark.
 * Only tests/, __graft_entry__.smoke() and bench.py (its CPU-baseline and reference legs)
 * load it; the product never does.
 *
 * Vector arithmetic follows the operation order of the oracle's Armadillo shim
 * (oracle/shim/armadillo): 3-element dot products and norms use two accumulators,
 * (v0 w0 + v2 w2) + v1 w1, normalise divides by the norm (unless it is zero), and the
 * whole oracle is compiled with -ffp-contract=off.  std::log, std::acos and std::rand
 * are replaced by orc_log, orc_acos and the per-exciton Philox streams of kmc_math.h.
 */
#ifndef ORC_KMC_ORACLE_H
#define ORC_KMC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Rate table.  kind 4: rate(theta)(z_shift, axis_shift_1, axis_shift_2) of
 * src/monte_carlo/scattering_struct.h:38-52, stored [n0][n1][n2][n3] row-major.
 * kind 2: rate(distance, theta_folded), stored [n0][n1] row-major.
 * kind 3 (mixed-chirality films, no counterpart in the reference): one kind-2 table per
 * (donor, acceptor) chirality pair, n[2] = chiralities S, stored [S][S][n0][n1]; species[site]
 * gives each site's chirality (NULL for the other kinds). */
typedef struct {
  int kind;
  int n[4];
  const double* grid[4];
  const double* rate;
  const int32_t* species;
} orc_table;

typedef struct orc_sim orc_sim;

/* arma::linspace as the shim defines it (used by monte_carlo.cpp:66-75). */
void orc_linspace(double start, double end, int64_t num, double* out);

/* The benchmark films' 2-D table: the Förster formula of monte_carlo.cpp:174-187 at zero axis
 * shifts on a (distance [m], angle [deg]) grid; rate is [nd][nt], theta in radians. */
void orc_forster2d_table(double gamma_0, const double distance[3], const double th_deg[3], double* dist,
                         double* theta, double* rate);
/* create_forster_scatt_table, src/monte_carlo/monte_carlo.cpp:156-200.  rate is
 * [n_th][n_zsh][n_a1][n_a2]; theta grid in degrees is scaled by pi/180 with the reference's
 * pi = 3.141592 (src/helper/constants.h:10). */
void orc_forster_table(double gamma_0, const double th_deg[3], const double zsh[3], const double a1[3],
                       const double a2[3], double* theta, double* z_shift, double* ash1, double* ash2,
                       double* rate);

/* trim_scats, src/monte_carlo/monte_carlo.h:722-782 (swap-to-end with link repair).
 * pos/orient are [n][3].  lim = {xmin, xmax, ymin, ymax, zmin, zmax}.  Returns the new n. */
int64_t orc_trim(int64_t n, double* pos, double* orient, int32_t* left, int32_t* right, const double lim[6]);

/* Read a mesh directory (create_scatterers, monte_carlo.h:199-271): the six files
 * single_cnt.{pos,orient}.{x,y,z}.dat, tubes x points, positions in nm (scaled by 1e-9).
 * Returns n sites (and n_tubes, n_points) or -1; arrays are malloc'ed ([n][3] and [n]). */
int64_t orc_load_mesh(const char* dir, double** pos, double** orient, int32_t** left, int32_t** right,
                      int64_t* n_tubes, int64_t* n_points);
void orc_free(void* p);

/* Build the engine: domain (monte_carlo.h:328-340), cell buckets (:368-416) and the
 * per-site total rates (set_max_rate, scatterer.h:89-93).  Copies every input. */
orc_sim* orc_sim_create(int64_t n_sites, const double* pos, const double* orient, const int32_t* left,
                        const int32_t* right, const orc_table* table, double r_max, double velocity,
                        int n_threads);
void orc_sim_destroy(orc_sim* s);

/* Neighbour list of one site exactly as find_neighbors (scatterer.cpp:34-83) builds it:
 * cumulative rates and neighbour site ids in list order.  Returns the count (<= cap). */
int orc_find_neighbors(const orc_sim* s, int64_t site, double* cum, int32_t* col, int cap);

/* Precompute all neighbour lists once (CSR).  Steps then read the CSR instead of
 * recomputing the list on every hop as the reference does; results are identical. */
int64_t orc_sim_build_csr(orc_sim* s);
/* Copy the CSR out (rowptr[n+1], col[nnz], cum[nnz]) and the per-site totals. */
void orc_sim_get_csr(const orc_sim* s, int64_t* rowptr, int32_t* col, double* cum, double* total, double* inv_total);

void orc_sim_domain(const orc_sim* s, double mn[3], double mx[3], int32_t ncell[3]);

/* Exciton creation.  mode 0: reference Green-Kubo set-up with n_sections
 * (injection_region / get_removal_domain, monte_carlo.cpp:203-251; kubo_create_particles
 * :308-316 and the particle constructor particle.h:48-52).  mode 1: every site is an
 * injection site and nothing is removed.  Exciton i draws from stream stream_base + i. */
int orc_sim_create_excitons(orc_sim* s, int mode, int n_sections, int64_t n_exc, uint64_t seed,
                            uint64_t stream_base, int use_csr);
int64_t orc_sim_n_inject(const orc_sim* s);

/* Record every site change of the first n_trace excitons (cap entries each):
 * hop result (update_state, also when it stays) -> site; flight across a tube link -> -1 - site;
 * reinjection -> INT32_MIN followed by the new site. */
void orc_sim_set_trace(orc_sim* s, int64_t n_trace, int64_t cap);
int64_t orc_sim_get_trace(const orc_sim* s, int64_t e, int32_t* buf, int64_t cap);

/* n_steps calls of kubo_step(dt) (monte_carlo.cpp:319-342); after each, the sums
 * sum_i dx_i^2, dy^2, dz^2 in exciton order (kubo_save_avg_dispalcement_squared
 * :382-409 before its division) go to msd_sums[step][3]. */
int orc_sim_step(orc_sim* s, double dt, int64_t n_steps, double* msd_sums);
/* As orc_sim_step, with the sums split by exciton batch: exciton i adds to batch
 * (i / 32) % batches; out[step][batch][3], each batch summed in exciton order. */
int orc_sim_step_batches(orc_sim* s, double dt, int64_t n_steps, int batches, double* out);

/* Per-exciton state: site, pos[3], old_pos[3], delta[3], ff, heading, draws, hops. */
void orc_sim_get_excitons(const orc_sim* s, int32_t* site, double* pos, double* old_pos, double* delta, double* ff,
                          int32_t* heading, uint64_t* draws, int64_t* hops);
int64_t orc_sim_total_hops(const orc_sim* s);
int64_t orc_sim_total_crossings(const orc_sim* s);

/* Contacts (steady-state flux) mode: the reference's second driver, init (monte_carlo.h:157-195),
 * step (:343-354), save_metrics (:519-643), repopulate_contacts (:443-491).  Slot k of `capacity`
 * draws from Philox stream k (key seed) and keeps its draw counter when its exciton is removed;
 * the initial excitons take slots 0.. in create_particles order and the n new excitons of a
 * contact the n lowest empty slots.  area[n_seg] (get_area), stat_pop[n_seg]
 * (get_scatterer_statistics), n_contact[2] (contact site counts) may be NULL.  Returns 0, -1 (bad
 * argument), -3 (a segment or contact with excitons to place has no site) or -4 (capacity). */
int orc_contacts_init(orc_sim* s, int n_seg, int64_t pop1, int64_t pop2, uint64_t seed, int64_t capacity,
                      double* area, int64_t* stat_pop, int64_t* n_contact);
/* n_steps of step(dt), the counts behind save_metrics (pop[step][n_seg]: excitons per segment;
 * curr[step][n_seg-1]: net crossings of each interface in +y) and repopulate_contacts;
 * n_live[step] = excitons after repopulation.  orc_sim_get_excitons reads the slots (site -1:
 * empty). */
int orc_contacts_step(orc_sim* s, double dt, int64_t n_steps, int64_t* pop, int64_t* curr, int64_t* n_live);
/* Hops from the precomputed CSR (1, the default of contacts mode) or from a fresh neighbour search
 * on every hop as the reference does (0); the results are the same. */
void orc_sim_use_csr(orc_sim* s, int use_csr);
/* track_particle (monte_carlo.h:786-818) for tracks first..: path [n_tracks][max_steps][3],
 * len[n_tracks] steps recorded, arrived[n_tracks].  Track k draws from Philox stream 2^32 + k. */
int orc_contacts_track(orc_sim* s, int64_t first, int n_tracks, double dt, int64_t max_steps, double* path,
                       int64_t* len, int32_t* arrived);

/* Exposed pieces for known-answer tests. */
double orc_log_export(double x);
void orc_log_array(const double* x, double* out, int64_t n);
double orc_acos_export(double x);
void orc_philox_export(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
int orc_rand_export(uint64_t seed, uint64_t stream, uint64_t n);
/* update_state's bisection (scatterer.cpp:17-30) on a given cumulative row: the index chosen. */
int orc_select_export(const double* cum, int n, double dice);
/* index_min(abs(grid - x)) of scattering_struct.h:41-49. */
int orc_index_min_export(const double* grid, int n, double x);

#ifdef __cplusplus
}
#endif

#endif
