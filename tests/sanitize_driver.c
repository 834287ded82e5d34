/* sanitize_driver.c -- runs the oracle (oracle/kmc_oracle.c) and the library's host code
 * (cnt_film_monte_carlo_gb300/csrc/kmc_host.cpp) under AddressSanitizer and
 * UndefinedBehaviorSanitizer: tests/test_sanitizers.py compiles it with -fsanitize=address,
 * undefined and fails on any report.  Everything here is host code; no GPU is involved.
 *
 * A small synthetic film (straight tubes on a grid, every fourth tube tilted), then:
 *   oracle: trim, both table producers, neighbour lists, CSR, region and uniform injection,
 *           steps (plain and batched), the per-hop search path, contacts mode and tracks;
 *   library host code: trim, domain, both table producers, the closed-form labeller, the
 *           diffusion fit, and the mesh reader on a mesh written here.
 * Exit code 0 when every call returned success. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "cntkmc.h"
#include "kmc_oracle.h"

#define CHECK(c)                                                                     \
  do {                                                                               \
    if (!(c)) {                                                                      \
      fprintf(stderr, "sanitize_driver: check failed: %s (line %d)\n", #c, __LINE__); \
      abort();                                                                       \
    }                                                                                \
  } while (0)

enum { TUBES = 24, PTS = 30 };

static void film(double* pos, double* orient, int32_t* left, int32_t* right) {
  for (int t = 0; t < TUBES; ++t) {
    const double x0 = 3e-9 * (t % 6), y0 = 4e-9 * (t / 6), z0 = 0.5e-9 * (t % 3);
    const double a = (t % 4 == 0) ? 0.3 : 0.1; /* tilted in y, so that contacts mode finds every y slab */
    const double ox = cos(a), oy = sin(a), oz = 0.0;
    for (int j = 0; j < PTS; ++j) {
      const int s = t * PTS + j;
      pos[3 * s] = x0 + 1e-9 * j * ox;
      pos[3 * s + 1] = y0 + 1e-9 * j * oy;
      pos[3 * s + 2] = z0 + 1e-9 * j * oz;
      orient[3 * s] = ox;
      orient[3 * s + 1] = oy;
      orient[3 * s + 2] = oz;
      left[s] = j > 0 ? s - 1 : -1;
      right[s] = j + 1 < PTS ? s + 1 : -1;
    }
  }
}

static int write_mesh(const char* dir, const double* pos, const double* orient) {
  static const char* names[6] = {"single_cnt.pos.x.dat",    "single_cnt.pos.y.dat",    "single_cnt.pos.z.dat",
                                 "single_cnt.orient.x.dat", "single_cnt.orient.y.dat", "single_cnt.orient.z.dat"};
  char path[4096];
  for (int k = 0; k < 6; ++k) {
    snprintf(path, sizeof path, "%s/%s", dir, names[k]);
    FILE* f = fopen(path, "w");
    if (!f) return 1;
    for (int t = 0; t < TUBES; ++t) {
      for (int j = 0; j < PTS; ++j) {
        const int s = t * PTS + j;
        const double v = k < 3 ? pos[3 * s + k] * 1e9 : orient[3 * s + k - 3];
        fprintf(f, " %.17g", v);
      }
      fprintf(f, "\n");
    }
    fclose(f);
  }
  return 0;
}

int main(int argc, char** argv) {
  const int64_t n = TUBES * PTS;
  double* pos = malloc(sizeof(double) * 3 * n);
  double* orient = malloc(sizeof(double) * 3 * n);
  int32_t* left = malloc(sizeof(int32_t) * n);
  int32_t* right = malloc(sizeof(int32_t) * n);
  film(pos, orient, left, right);

  /* ---- oracle ---- */
  double d2[3] = {0.5e-9, 10e-9, 24}, th2[3] = {0, 90, 19};
  double *g0 = malloc(24 * sizeof(double)), *g1 = malloc(19 * sizeof(double)), *r2 = malloc(24 * 19 * sizeof(double));
  orc_forster2d_table(1e12, d2, th2, g0, g1, r2); /* slow rates: few hops on a dense film */
  double th4[3] = {0, 180, 7}, zs[3] = {1.5e-9, 10e-9, 5}, a1[3] = {-10e-9, 10e-9, 5}, a2[3] = {-10e-9, 10e-9, 5};
  double *h0 = malloc(7 * sizeof(double)), *h1 = malloc(5 * sizeof(double)), *h2 = malloc(5 * sizeof(double)),
         *h3 = malloc(5 * sizeof(double)), *r4 = malloc(7 * 5 * 5 * 5 * sizeof(double));
  orc_forster_table(1e12, th4, zs, a1, a2, h0, h1, h2, h3, r4);
  orc_table t2 = {2, {24, 19, 0, 0}, {g0, g1, NULL, NULL}, r2, NULL};
  orc_table t4 = {4, {7, 5, 5, 5}, {h0, h1, h2, h3}, r4, NULL};
  for (int pass = 0; pass < 2; ++pass) {
    orc_sim* s = orc_sim_create(n, pos, orient, left, right, pass ? &t4 : &t2, 10e-9, 2e5, 1);
    CHECK(s != NULL);
    CHECK(orc_sim_build_csr(s) > 0);
    double cum[4096];
    int32_t col[4096];
    CHECK(orc_find_neighbors(s, 5, cum, col, 4096) >= 0);
    orc_sim_set_trace(s, 4, 256); /* before the excitons: their trace buffers come with them */
    CHECK(orc_sim_create_excitons(s, pass ? 0 : 1, 3, 200, 7 + pass, 0, 1) == 0);
    double msd[3 * 4];
    CHECK(orc_sim_step(s, 2e-13, 4, msd) == 0);
    double bm[4 * 4 * 3];
    CHECK(orc_sim_step_batches(s, 2e-13, 4, 4, bm) == 0);
    orc_sim_use_csr(s, 0); /* the reference's per-hop neighbour search */
    CHECK(orc_sim_step(s, 1e-13, 2, msd) == 0);
    int32_t buf[256];
    CHECK(orc_sim_get_trace(s, 0, buf, 256) >= 0);
    int32_t site[200], heading[200];
    double ep[600], eo[600], ed[600], ff[200];
    uint64_t draws[200];
    int64_t hops[200];
    orc_sim_get_excitons(s, site, ep, eo, ed, ff, heading, draws, hops);
    CHECK(orc_sim_total_hops(s) > 0);
    orc_sim_destroy(s);
  }
  { /* contacts mode and tracks */
    orc_sim* s = orc_sim_create(n, pos, orient, left, right, &t2, 10e-9, 2e5, 1);
    CHECK(s != NULL);
    double area[4];
    int64_t stat[4], ncon[2];
    CHECK(orc_contacts_init(s, 4, 60, 10, 3, 4096, area, stat, ncon) == 0);
    int64_t pop[3 * 4], cur[3 * 3], live[3];
    CHECK(orc_contacts_step(s, 2e-13, 3, pop, cur, live) == 0);
    double path[2 * 50 * 3];
    int64_t len[2];
    int32_t arrived[2];
    CHECK(orc_contacts_track(s, 0, 2, 2e-13, 50, path, len, arrived) == 0);
    orc_sim_destroy(s);
  }
  { /* trim, in both implementations (each on its own copy: trim reorders in place) */
    double *p = malloc(sizeof(double) * 3 * n), *o = malloc(sizeof(double) * 3 * n);
    int32_t *l = malloc(sizeof(int32_t) * n), *r = malloc(sizeof(int32_t) * n);
    const double lim[6] = {-1e-6, 1e-6, 2e-9, 1e-6, -1e-6, 1e-6};
    for (int impl = 0; impl < 2; ++impl) {
      memcpy(p, pos, sizeof(double) * 3 * n);
      memcpy(o, orient, sizeof(double) * 3 * n);
      memcpy(l, left, sizeof(int32_t) * n);
      memcpy(r, right, sizeof(int32_t) * n);
      int64_t kept = 0;
      if (impl == 0)
        kept = orc_trim(n, p, o, l, r, lim);
      else
        CHECK(kmc_trim_sites(n, p, o, l, r, lim, &kept) == KMC_OK);
      CHECK(kept > 0 && kept < n);
    }
    free(p), free(o), free(l), free(r);
  }

  /* ---- library host code ---- */
  double mn[3], mx[3];
  CHECK(kmc_domain(n, pos, mn, mx) == KMC_OK);
  CHECK(kmc_forster2d_table(1e15, d2, th2, g0, g1, r2) == KMC_OK);
  CHECK(kmc_forster_table(1e15, th4, zs, a1, a2, h0, h1, h2, h3, r4) == KMC_OK);
  {
    double e[2] = {1.2, 1.3}, dia[2] = {0.8e-9, 0.9e-9};
    kmc_species_model m = {2, 1e15, e, dia, 0.85e-9, 0.1, 0.02585, 0.05, 0.3e-9};
    double dist[4] = {1e-9, 2e-9, 5e-9, 9e-9}, th[4] = {0, 0.4, 0.9, 1.5}, rate[4];
    int32_t da[4] = {0, 1, 0, 1}, ac[4] = {1, 0, 0, 1};
    CHECK(kmc_species_rates(&m, 4, dist, th, da, ac, rate) == KMC_OK);
  }
  {
    enum { ST = 20, B = 4 };
    double msd[ST * B * 3], times[ST], D[3], ci[3];
    int64_t counts[B] = {32, 32, 32, 30};
    for (int i = 0; i < ST; ++i) {
      times[i] = (i + 1) * 1e-12;
      for (int b = 0; b < B; ++b)
        for (int c = 0; c < 3; ++c) msd[(i * B + b) * 3 + c] = counts[b] * 2e-4 * times[i] * (1 + 0.01 * ((i + b + c) % 5));
    }
    CHECK(kmc_fit_diffusion(msd, counts, times, ST, B, 0.8, D, ci) == KMC_OK);
  }
  if (argc > 1) { /* mesh reader on a mesh written into argv[1] */
    CHECK(write_mesh(argv[1], pos, orient) == 0);
    int64_t nt = 0, np = 0;
    CHECK(kmc_read_mesh(argv[1], &nt, &np, NULL, NULL, NULL, NULL) == KMC_OK && nt == TUBES && np == PTS);
    double *p = malloc(sizeof(double) * 3 * nt * np), *o = malloc(sizeof(double) * 3 * nt * np);
    int32_t *l = malloc(sizeof(int32_t) * nt * np), *r = malloc(sizeof(int32_t) * nt * np);
    CHECK(kmc_read_mesh(argv[1], &nt, &np, p, o, l, r) == KMC_OK);
    free(p), free(o), free(l), free(r);
    /* a token that is not a number, appended to one file: refused, not read short */
    char path[4096];
    snprintf(path, sizeof path, "%s/single_cnt.pos.y.dat", argv[1]);
    FILE* f = fopen(path, "a");
    CHECK(f != NULL);
    fprintf(f, " 1 x\n");
    fclose(f);
    CHECK(kmc_read_mesh(argv[1], &nt, &np, NULL, NULL, NULL, NULL) == KMC_ERR_IO);
  }
  { /* refusals: nothing is read or written past the inputs */
    int32_t *l = malloc(sizeof(int32_t) * n), *l0 = malloc(sizeof(int32_t) * n);
    double *p = malloc(sizeof(double) * 3 * n), *o = malloc(sizeof(double) * 3 * n);
    int32_t* r = malloc(sizeof(int32_t) * n);
    memcpy(l, left, sizeof(int32_t) * n);
    memcpy(r, right, sizeof(int32_t) * n);
    memcpy(p, pos, sizeof(double) * 3 * n);
    memcpy(o, orient, sizeof(double) * 3 * n);
    l[3] = (int32_t)n + 5; /* a link past the film */
    memcpy(l0, l, sizeof(int32_t) * n);
    const double lim[6] = {-1e-6, 1e-6, 2e-9, 1e-6, -1e-6, 1e-6};
    int64_t kept = -1;
    CHECK(kmc_trim_sites(n, p, o, l, r, lim, &kept) == KMC_ERR_ARG && kept == -1);
    CHECK(memcmp(l, l0, sizeof(int32_t) * n) == 0 && memcmp(p, pos, sizeof(double) * 3 * n) == 0);
    free(l), free(l0), free(p), free(o), free(r);
    const double bad_counts[4] = {NAN, 0.5, -3.0, 1e300};
    for (int k = 0; k < 4; ++k) {
      const double dd[3] = {0.5e-9, 10e-9, bad_counts[k]};
      CHECK(kmc_forster2d_table(1e15, dd, th2, g0, g1, r2) == KMC_ERR_ARG);
      const double zz[3] = {1e-9, 2e-9, bad_counts[k]};
      CHECK(kmc_forster_table(1e15, th4, zz, a1, a2, h0, h1, h2, h3, r4) == KMC_ERR_ARG);
    }
  }
  free(g0), free(g1), free(r2), free(h0), free(h1), free(h2), free(h3), free(r4);
  free(pos), free(orient), free(left), free(right);
  printf("sanitize_driver: ok\n");
  return 0;
}
