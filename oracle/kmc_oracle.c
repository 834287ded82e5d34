/* kmc_oracle.c -- TEST INFRASTRUCTURE: CPU restatement of the reference's exciton-hopping
 * hot path.  See kmc_oracle.h for what it is and who may use it.  Every function names
 * the reference lines it restates (paths relative to the reference project). */
#include "kmc_oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "kmc_math.h"

#define ORC_REF_PI 3.141592 /* src/helper/constants.h:10 */
#define ORC_MIN_HOP_DIST 0.4e-9 /* scatterer.cpp:43 */

/* ---------------------------------------------------------------- vector helpers (shim order) */
static inline double v3_dot(const double* a, const double* b) {
  double acc1 = 0.0, acc2 = 0.0;
  acc1 += a[0] * b[0];
  acc2 += a[1] * b[1];
  acc1 += a[2] * b[2];
  return acc1 + acc2;
}
static inline double v3_norm(const double* a) { return sqrt(v3_dot(a, a)); }

/* ---------------------------------------------------------------- tables */
void orc_linspace(double start, double end, int64_t num, double* out) {
  if (num == 1) {
    out[0] = end;
    return;
  }
  if (num < 2) return;
  double delta = (end - start) / (double)(num - 1);
  for (int64_t i = 0; i < num - 1; ++i) out[i] = start + (double)i * delta;
  out[num - 1] = end;
}

int orc_index_min_export(const double* grid, int n, double x) {
  /* scattering_struct.h:41-49: tmp = abs(grid - x); tmp.index_min() (first minimum) */
  double best = INFINITY;
  int idx = 0;
  for (int i = 0; i < n; ++i) {
    double t = fabs(grid[i] - x);
    if (t < best) {
      best = t;
      idx = i;
    }
  }
  return idx;
}

void orc_forster_table(double gamma_0, const double th_deg[3], const double zsh[3], const double a1[3],
                       const double a2[3], double* theta, double* z_shift, double* ash1, double* ash2,
                       double* rate) {
  /* monte_carlo.cpp:157-167 */
  int64_t nz = (int64_t)zsh[2], n1 = (int64_t)a1[2], n2 = (int64_t)a2[2], nt = (int64_t)th_deg[2];
  orc_linspace(zsh[0], zsh[1], nz, z_shift);
  orc_linspace(a1[0], a1[1], n1, ash1);
  orc_linspace(a2[0], a2[1], n2, ash2);
  orc_linspace(th_deg[0], th_deg[1], nt, theta);
  double scale = ORC_REF_PI / 180;
  for (int64_t i = 0; i < nt; ++i) theta[i] = theta[i] * scale;
  /* monte_carlo.cpp:174-195 */
  for (int64_t it = 0; it < nt; ++it) {
    double th = theta[it];
    for (int64_t iz = 0; iz < nz; ++iz) {
      double z = z_shift[iz];
      for (int64_t i1 = 0; i1 < n1; ++i1) {
        double s1 = ash1[i1];
        for (int64_t i2 = 0; i2 < n2; ++i2) {
          double s2 = ash2[i2];
          double r1[3] = {s1, 0, 0};
          double r2[3] = {s2 * cos(th), s2 * sin(th), z};
          double dR[3] = {r1[0] - r2[0], r1[1] - r2[1], r1[2] - r2[2]};
          double n_r1 = v3_norm(r1), n_r2 = v3_norm(r2), n_dR = v3_norm(dR);
          double d_r1 = n_r1 != 0 ? n_r1 : 1.0, d_r2 = n_r2 != 0 ? n_r2 : 1.0, d_dR = n_dR != 0 ? n_dR : 1.0;
          double u1[3] = {r1[0] / d_r1, r1[1] / d_r1, r1[2] / d_r1};
          double u2[3] = {r2[0] / d_r2, r2[1] / d_r2, r2[2] / d_r2};
          double ud[3] = {dR[0] / d_dR, dR[1] / d_dR, dR[2] / d_dR};
          double af = cos(th) - 3 * v3_dot(u1, ud) * v3_dot(u2, ud);
          rate[((it * nz + iz) * n1 + i1) * n2 + i2] = gamma_0 * (af * af) * pow(1.e-9 / n_dR, 6);
        }
      }
    }
  }
}

/* The 2-D (centre distance, folded angle) table of the benchmark films: create_forster_scatt_table's
 * formula (monte_carlo.cpp:174-187) at zero axis shifts, gamma_0 cos^2(theta) (1 nm / d)^6, on
 * linspace grids of distance (m) and angle (degrees, scaled by the reference's pi, :167). */
void orc_forster2d_table(double gamma_0, const double distance[3], const double th_deg[3], double* dist,
                         double* theta, double* rate) {
  int64_t nd = (int64_t)distance[2], nt = (int64_t)th_deg[2];
  orc_linspace(distance[0], distance[1], nd, dist);
  orc_linspace(th_deg[0], th_deg[1], nt, theta);
  double scale = ORC_REF_PI / 180;
  for (int64_t i = 0; i < nt; ++i) theta[i] = theta[i] * scale;
  for (int64_t i = 0; i < nd; ++i)
    for (int64_t k = 0; k < nt; ++k) {
      double c = cos(theta[k]);
      rate[i * nt + k] = gamma_0 * (c * c) * pow(1.e-9 / dist[i], 6);
    }
}

/* get_rate, scattering_struct.h:38-52 (and the 2-D (distance, theta) extension) */
static inline double table_rate(const orc_table* t, double th, double zsh, double a1, double a2, double dist,
                                int64_t pair_off) {
  if (t->kind == 4) {
    int i0 = orc_index_min_export(t->grid[0], t->n[0], th);
    int i1 = orc_index_min_export(t->grid[1], t->n[1], zsh);
    int i2 = orc_index_min_export(t->grid[2], t->n[2], a1);
    int i3 = orc_index_min_export(t->grid[3], t->n[3], a2);
    return t->rate[(((int64_t)i0 * t->n[1] + i1) * t->n[2] + i2) * t->n[3] + i3];
  }
  int i0 = orc_index_min_export(t->grid[0], t->n[0], dist);
  int i1 = orc_index_min_export(t->grid[1], t->n[1], th);
  return t->rate[pair_off + (int64_t)i0 * t->n[1] + i1];
}

/* ---------------------------------------------------------------- trim */
int64_t orc_trim(int64_t n, double* pos, double* orient, int32_t* left, int32_t* right, const double lim[6]) {
  /* monte_carlo.h:730-750: swap two sites and repair the links that point at them */
#define SWAP_SITES(I, J)                                              \
  do {                                                                \
    int64_t si = (I), sj = (J);                                       \
    int32_t iL = left[si], iR = right[si], jL = left[sj], jR = right[sj]; \
    int32_t new_i = (int32_t)sj, new_j = (int32_t)si;                 \
    if (iL > -1) right[iL] = new_i;                                   \
    if (iR > -1) left[iR] = new_i;                                    \
    if (jL > -1) right[jL] = new_j;                                   \
    if (jR > -1) left[jR] = new_j;                                    \
    for (int c = 0; c < 3; ++c) {                                     \
      double t = pos[3 * si + c];                                     \
      pos[3 * si + c] = pos[3 * sj + c];                              \
      pos[3 * sj + c] = t;                                            \
      t = orient[3 * si + c];                                         \
      orient[3 * si + c] = orient[3 * sj + c];                        \
      orient[3 * sj + c] = t;                                         \
    }                                                                 \
    int32_t tl = left[si], tr = right[si];                            \
    left[si] = left[sj];                                              \
    right[si] = right[sj];                                            \
    left[sj] = tl;                                                    \
    right[sj] = tr;                                                   \
  } while (0)
  /* monte_carlo.h:752-771 */
  int64_t j = n;
  for (int64_t i = 0; i < j;) {
    const double* p = pos + 3 * i;
    if (p[0] < lim[0] || p[1] < lim[2] || p[2] < lim[4] || p[0] > lim[1] || p[1] > lim[3] || p[2] > lim[5]) {
      --j;
      SWAP_SITES(i, j);
      if (left[j] > -1) right[left[j]] = -1;
      if (right[j] > -1) left[right[j]] = -1;
    } else {
      ++i;
    }
  }
#undef SWAP_SITES
  return j;
}

/* ---------------------------------------------------------------- mesh reader */
static int read_matrix(const char* path, double** out, int64_t* rows, int64_t* cols) {
  FILE* f = fopen(path, "r");
  if (!f) return -1;
  size_t cap = 1024, n = 0;
  double* v = (double*)malloc(cap * sizeof(double));
  int64_t r = 0, c0 = -1;
  char* line = NULL;
  size_t lcap = 0;
  ssize_t len;
  while ((len = getline(&line, &lcap, f)) >= 0) {
    int64_t c = 0;
    char* s = line;
    for (;;) {
      while (*s == ' ' || *s == '\t' || *s == ',' || *s == '\r' || *s == '\n') ++s;
      if (!*s) break;
      char* e;
      double x = strtod(s, &e);
      if (e == s) break;
      if (n == cap) {
        cap *= 2;
        v = (double*)realloc(v, cap * sizeof(double));
      }
      v[n++] = x;
      ++c;
      s = e;
    }
    if (c == 0) continue;
    if (c0 < 0) c0 = c;
    if (c != c0) {
      free(v);
      free(line);
      fclose(f);
      return -2;
    }
    ++r;
  }
  free(line);
  fclose(f);
  *out = v;
  *rows = r;
  *cols = c0 < 0 ? 0 : c0;
  return 0;
}

int64_t orc_load_mesh(const char* dir, double** pos_out, double** orient_out, int32_t** left_out,
                      int32_t** right_out, int64_t* n_tubes, int64_t* n_points) {
  static const char* names[6] = {"single_cnt.pos.x.dat",    "single_cnt.pos.y.dat",    "single_cnt.pos.z.dat",
                                 "single_cnt.orient.x.dat", "single_cnt.orient.y.dat", "single_cnt.orient.z.dat"};
  double* m[6] = {0};
  int64_t rows = -1, cols = -1;
  for (int k = 0; k < 6; ++k) {
    char path[4096];
    snprintf(path, sizeof path, "%s/%s", dir, names[k]);
    int64_t r, c;
    if (read_matrix(path, &m[k], &r, &c) != 0 || (rows >= 0 && (r != rows || c != cols))) {
      for (int q = 0; q < 6; ++q) free(m[q]);
      return -1;
    }
    rows = r;
    cols = c;
  }
  int64_t n = rows * cols;
  double* pos = (double*)malloc(sizeof(double) * 3 * (n ? n : 1));
  double* orient = (double*)malloc(sizeof(double) * 3 * (n ? n : 1));
  int32_t* left = (int32_t*)malloc(sizeof(int32_t) * (n ? n : 1));
  int32_t* right = (int32_t*)malloc(sizeof(int32_t) * (n ? n : 1));
  /* monte_carlo.h:211,225,239 scale positions by 1e-9; :249-262 number and link the sites */
  for (int64_t i = 0; i < rows; ++i) {
    for (int64_t j = 0; j < cols; ++j) {
      int64_t s = i * cols + j;
      for (int c = 0; c < 3; ++c) {
        pos[3 * s + c] = m[c][s] * 1.e-9;
        orient[3 * s + c] = m[3 + c][s];
      }
      left[s] = j > 0 ? (int32_t)(s - 1) : -1;
      right[s] = j + 1 < cols ? (int32_t)(s + 1) : -1;
    }
  }
  for (int q = 0; q < 6; ++q) free(m[q]);
  *pos_out = pos;
  *orient_out = orient;
  *left_out = left;
  *right_out = right;
  *n_tubes = rows;
  *n_points = cols;
  return n;
}

void orc_free(void* p) { free(p); }

/* ---------------------------------------------------------------- engine */
typedef struct {
  int32_t site;
  int32_t heading;
  double pos[3], old[3], delta[3];
  double ff;
  orc_rng rng;
  int64_t hops, crossings;
  int32_t* trace;
  int64_t trace_n;
} orc_exc;

struct orc_sim {
  int64_t n;
  double *pos, *orient;
  int32_t *left, *right;
  orc_table tab;
  double* tab_store;
  int32_t* species_store; /* kind-3 tables: chirality of each site */
  double r_max, v;
  int n_threads;
  double mn[3], mx[3];
  int32_t nx, ny, nz;
  int64_t* cell_start; /* [ncell+1] */
  int32_t* cell_members;
  int32_t* close_cells; /* [n][27], -1 padded, in x-outer/y/z-inner order */
  double *total, *inv_total;
  int64_t* rowptr;
  int32_t* col;
  double* cum;
  int use_csr;
  /* green-kubo */
  int mode;
  int32_t* inject;
  int64_t n_inject;
  double rmin[3], rmax[3];
  orc_exc* exc;
  int64_t n_exc;
  int64_t n_trace, trace_cap;
  int max_list; /* longest neighbour list (scratch size for per-hop recompute) */
  /* contacts mode */
  int n_seg;
  int64_t c_pop[2];
  int32_t* c_list[2];
  int64_t c_n[2];
  uint64_t c_seed;
  uint8_t* live; /* [n_exc] */
};

static void domain_of(const orc_sim* s, double mn[3], double mx[3]) {
  /* monte_carlo.h:328-340 */
  for (int c = 0; c < 3; ++c) mn[c] = mx[c] = s->pos[c];
  for (int64_t i = 0; i < s->n; ++i)
    for (int c = 0; c < 3; ++c) {
      double p = s->pos[3 * i + c];
      mn[c] = mn[c] > p ? p : mn[c];
      mx[c] = mx[c] < p ? p : mx[c];
    }
}

static void build_buckets(orc_sim* s) {
  /* monte_carlo.h:375-412 */
  double r = s->r_max;
  s->nx = (int32_t)ceil((s->mx[0] - s->mn[0]) / r) + 1;
  s->ny = (int32_t)ceil((s->mx[1] - s->mn[1]) / r) + 1;
  s->nz = (int32_t)ceil((s->mx[2] - s->mn[2]) / r) + 1;
  int64_t ncell = (int64_t)s->nx * s->ny * s->nz;
  s->cell_start = (int64_t*)calloc(ncell + 1, sizeof(int64_t));
  int32_t* cid = (int32_t*)malloc(sizeof(int32_t) * (s->n ? s->n : 1));
  int32_t* ix3 = (int32_t*)malloc(sizeof(int32_t) * 3 * (s->n ? s->n : 1));
  for (int64_t i = 0; i < s->n; ++i) {
    int ix = (int)((s->pos[3 * i + 0] - s->mn[0]) / r);
    int iy = (int)((s->pos[3 * i + 1] - s->mn[1]) / r);
    int iz = (int)((s->pos[3 * i + 2] - s->mn[2]) / r);
    ix3[3 * i] = ix;
    ix3[3 * i + 1] = iy;
    ix3[3 * i + 2] = iz;
    cid[i] = ix + iy * s->nx + iz * s->nx * s->ny;
    s->cell_start[cid[i] + 1]++;
  }
  for (int64_t c = 0; c < ncell; ++c) s->cell_start[c + 1] += s->cell_start[c];
  s->cell_members = (int32_t*)malloc(sizeof(int32_t) * (s->n ? s->n : 1));
  int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (ncell ? ncell : 1));
  memcpy(fill, s->cell_start, sizeof(int64_t) * ncell);
  for (int64_t i = 0; i < s->n; ++i) s->cell_members[fill[cid[i]]++] = (int32_t)i; /* push_back in site order */
  free(fill);
  s->close_cells = (int32_t*)malloc(sizeof(int32_t) * 27 * (s->n ? s->n : 1));
  for (int64_t i = 0; i < s->n; ++i) {
    int q = 0;
    int ix = ix3[3 * i], iy = ix3[3 * i + 1], iz = ix3[3 * i + 2];
    for (int a = ix - 1; a <= ix + 1; ++a)
      for (int b = iy - 1; b <= iy + 1; ++b)
        for (int c = iz - 1; c <= iz + 1; ++c)
          if (a > -1 && a < s->nx && b > -1 && b < s->ny && c > -1 && c < s->nz)
            s->close_cells[27 * i + q++] = a + b * s->nx + c * s->nx * s->ny;
    for (; q < 27; ++q) s->close_cells[27 * i + q] = -1;
  }
  free(cid);
  free(ix3);
}

/* find_neighbors, scatterer.cpp:34-83 */
int orc_find_neighbors(const orc_sim* s, int64_t site, double* cum, int32_t* col, int cap) {
  const double* p1 = s->pos + 3 * site;
  const double* a1 = s->orient + 3 * site;
  int k = 0;
  for (int q = 0; q < 27; ++q) {
    int32_t c = s->close_cells[27 * site + q];
    if (c < 0) break;
    for (int64_t m = s->cell_start[c]; m < s->cell_start[c + 1]; ++m) {
      int32_t j = s->cell_members[m];
      const double* p2 = s->pos + 3 * (int64_t)j;
      double dR[3] = {p1[0] - p2[0], p1[1] - p2[1], p1[2] - p2[2]};
      double distance = v3_norm(dR);
      if ((distance < s->r_max) && (distance > ORC_MIN_HOP_DIST)) {
        const double* a2 = s->orient + 3 * (int64_t)j;
        double cosT = v3_dot(a1, a2);
        double theta, ash1, ash2, zsh;
        if (s->tab.kind != 4) { /* 2-D tables: folded angle */
          double ac = fabs(cosT);
          theta = ac >= 1.0 ? 0.0 : orc_acos(ac);
          ash1 = ash2 = zsh = 0;
        } else if (cosT == 1) {
          ash1 = 0;
          ash2 = v3_dot(dR, a1);
          theta = 0;
          double t = v3_dot(dR, a1);
          double w[3] = {dR[0] - t * a1[0], dR[1] - t * a1[1], dR[2] - t * a1[2]};
          zsh = v3_norm(w);
        } else {
          theta = orc_acos(cosT);
          double y1 = v3_dot(a1, dR);
          double y2 = v3_dot(a2, dR);
          double sin2 = 1 - cosT * cosT;
          ash1 = (y1 + y2 * cosT) / sin2;
          ash2 = (y2 + y1 * cosT) / sin2;
          double w[3];
          for (int c3 = 0; c3 < 3; ++c3) w[c3] = (ash1 * a1[c3] + p1[c3]) - (ash2 * a2[c3] + p2[c3]);
          zsh = v3_norm(w);
        }
        const int64_t pair_off =
            s->tab.kind == 3
                ? ((int64_t)s->tab.species[site] * s->tab.n[2] + s->tab.species[j]) * ((int64_t)s->tab.n[0] * s->tab.n[1])
                : 0;
        double rate = table_rate(&s->tab, theta, zsh, ash1, ash2, distance, pair_off);
        if (k < cap) {
          cum[k] = rate;
          col[k] = j;
        }
        ++k;
      }
    }
  }
  /* scatterer.cpp:78-80: inclusive prefix sum in list order */
  int kk = k < cap ? k : cap;
  for (int i = 1; i < kk; ++i) cum[i] += cum[i - 1];
  return k;
}

static int count_neighbors(const orc_sim* s, int64_t site) {
  /* no_of_neighbors, scatterer.cpp:85-104 */
  const double* p1 = s->pos + 3 * site;
  int k = 0;
  for (int q = 0; q < 27; ++q) {
    int32_t c = s->close_cells[27 * site + q];
    if (c < 0) break;
    for (int64_t m = s->cell_start[c]; m < s->cell_start[c + 1]; ++m) {
      const double* p2 = s->pos + 3 * (int64_t)s->cell_members[m];
      double dR[3] = {p1[0] - p2[0], p1[1] - p2[1], p1[2] - p2[2]};
      double d = v3_norm(dR);
      if (d < s->r_max && d > ORC_MIN_HOP_DIST) ++k;
    }
  }
  return k;
}

orc_sim* orc_sim_create(int64_t n_sites, const double* pos, const double* orient, const int32_t* left,
                        const int32_t* right, const orc_table* table, double r_max, double velocity,
                        int n_threads) {
  if (n_sites <= 0) return NULL;
  if (table->kind == 3) {
    if (!table->species || table->n[2] < 1) return NULL;
    for (int64_t i = 0; i < n_sites; ++i)
      if (table->species[i] < 0 || table->species[i] >= table->n[2]) return NULL;
  }
  orc_sim* s = (orc_sim*)calloc(1, sizeof(orc_sim));
  s->n = n_sites;
  s->pos = (double*)malloc(sizeof(double) * 3 * n_sites);
  s->orient = (double*)malloc(sizeof(double) * 3 * n_sites);
  s->left = (int32_t*)malloc(sizeof(int32_t) * n_sites);
  s->right = (int32_t*)malloc(sizeof(int32_t) * n_sites);
  memcpy(s->pos, pos, sizeof(double) * 3 * n_sites);
  memcpy(s->orient, orient, sizeof(double) * 3 * n_sites);
  memcpy(s->left, left, sizeof(int32_t) * n_sites);
  memcpy(s->right, right, sizeof(int32_t) * n_sites);
  s->r_max = r_max;
  s->v = velocity;
  s->n_threads = n_threads > 0 ? n_threads : 1;
  /* copy the table */
  s->tab = *table;
  int64_t nr = table->kind == 3 ? (int64_t)table->n[2] * table->n[2] : 1, ng = 0;
  int dims = table->kind == 4 ? 4 : 2;
  for (int d = 0; d < dims; ++d) {
    nr *= table->n[d];
    ng += table->n[d];
  }
  s->tab_store = (double*)malloc(sizeof(double) * (nr + ng));
  double* w = s->tab_store;
  for (int d = 0; d < dims; ++d) {
    memcpy(w, table->grid[d], sizeof(double) * table->n[d]);
    s->tab.grid[d] = w;
    w += table->n[d];
  }
  memcpy(w, table->rate, sizeof(double) * nr);
  s->tab.rate = w;
  s->species_store = NULL;
  s->tab.species = NULL;
  if (table->kind == 3) {
    s->species_store = (int32_t*)malloc(sizeof(int32_t) * n_sites);
    memcpy(s->species_store, table->species, sizeof(int32_t) * n_sites);
    s->tab.species = s->species_store;
  }
  domain_of(s, s->mn, s->mx);
  build_buckets(s);
  /* set_max_rate, monte_carlo.h:426-440 / scatterer.h:89-93.  An empty list is undefined
   * behaviour in the reference (back() of an empty vector); here total = 0, 1/total = inf. */
  s->total = (double*)malloc(sizeof(double) * n_sites);
  s->inv_total = (double*)malloc(sizeof(double) * n_sites);
  int max_list = 0;
#pragma omp parallel for schedule(dynamic, 256) num_threads(s->n_threads) reduction(max : max_list)
  for (int64_t i = 0; i < n_sites; ++i) {
    int k = count_neighbors(s, i);
    if (k > max_list) max_list = k;
  }
  s->max_list = max_list;
#pragma omp parallel num_threads(s->n_threads)
  {
    double* cum = (double*)malloc(sizeof(double) * (max_list + 1));
    int32_t* col = (int32_t*)malloc(sizeof(int32_t) * (max_list + 1));
#pragma omp for schedule(dynamic, 256)
    for (int64_t i = 0; i < n_sites; ++i) {
      int k = orc_find_neighbors(s, i, cum, col, max_list + 1);
      s->total[i] = k > 0 ? cum[k - 1] : 0.0;
      s->inv_total[i] = 1. / s->total[i];
    }
    free(cum);
    free(col);
  }
  return s;
}

void orc_sim_domain(const orc_sim* s, double mn[3], double mx[3], int32_t ncell[3]) {
  for (int c = 0; c < 3; ++c) {
    mn[c] = s->mn[c];
    mx[c] = s->mx[c];
  }
  ncell[0] = s->nx;
  ncell[1] = s->ny;
  ncell[2] = s->nz;
}

int64_t orc_sim_build_csr(orc_sim* s) {
  free(s->rowptr);
  free(s->col);
  free(s->cum);
  s->rowptr = (int64_t*)malloc(sizeof(int64_t) * (s->n + 1));
  s->rowptr[0] = 0;
  for (int64_t i = 0; i < s->n; ++i) s->rowptr[i + 1] = s->rowptr[i] + count_neighbors(s, i);
  int64_t nnz = s->rowptr[s->n];
  s->col = (int32_t*)malloc(sizeof(int32_t) * (nnz ? nnz : 1));
  s->cum = (double*)malloc(sizeof(double) * (nnz ? nnz : 1));
#pragma omp parallel for schedule(dynamic, 256) num_threads(s->n_threads)
  for (int64_t i = 0; i < s->n; ++i) {
    int64_t b = s->rowptr[i];
    orc_find_neighbors(s, i, s->cum + b, s->col + b, (int)(s->rowptr[i + 1] - b));
  }
  return nnz;
}

void orc_sim_get_csr(const orc_sim* s, int64_t* rowptr, int32_t* col, double* cum, double* total, double* inv_total) {
  if (!s->rowptr) return;
  int64_t nnz = s->rowptr[s->n];
  if (rowptr) memcpy(rowptr, s->rowptr, sizeof(int64_t) * (s->n + 1));
  if (col) memcpy(col, s->col, sizeof(int32_t) * nnz);
  if (cum) memcpy(cum, s->cum, sizeof(double) * nnz);
  if (total) memcpy(total, s->total, sizeof(double) * s->n);
  if (inv_total) memcpy(inv_total, s->inv_total, sizeof(double) * s->n);
}

/* bisection of update_state, scatterer.cpp:17-30 (unsigned arithmetic as written) */
static inline unsigned select_index(const double* cum, unsigned n, double dice) {
  unsigned left = (unsigned)-1;
  unsigned right = n - 1;
  while (left + 1 < right) {
    unsigned mid = (left + right) / 2;
    if (cum[mid] <= dice)
      left = mid;
    else
      right = mid;
  }
  return right;
}
int orc_select_export(const double* cum, int n, double dice) { return (int)select_index(cum, (unsigned)n, dice); }

static inline void trace_push(const orc_sim* s, orc_exc* p, int32_t v) {
  if (p->trace) {
    if (p->trace_n < s->trace_cap) p->trace[p->trace_n] = v;
    p->trace_n++;
  }
}

/* ff_time, scatterer.h:74-80 */
static inline double ff_time(const orc_sim* s, int32_t site, orc_rng* g) {
  int r;
  while ((r = orc_rand(g)) == 0) {
  }
  return -s->inv_total[site] * orc_log((double)r / (double)ORC_RAND_MAX);
}

/* update_state, scatterer.cpp:9-31 */
static inline int32_t update_state(const orc_sim* s, orc_exc* p, double* cum_buf, int32_t* col_buf) {
  int32_t site = p->site;
  const double* cum;
  const int32_t* col;
  int64_t n;
  if (s->use_csr) {
    int64_t b = s->rowptr[site];
    n = s->rowptr[site + 1] - b;
    cum = s->cum + b;
    col = s->col + b;
  } else {
    n = orc_find_neighbors(s, site, cum_buf, col_buf, s->max_list + 1);
    cum = cum_buf;
    col = col_buf;
  }
  if (n == 0) return site;
  double dice = cum[n - 1] * (double)orc_rand(&p->rng) / (double)ORC_RAND_MAX;
  return col[select_index(cum, (unsigned)n, dice)];
}

/* particle::fly, particle.cpp:9-54 */
static inline void fly(const orc_sim* s, orc_exc* p, double dt) {
  if (s->left[p->site] < 0 && s->right[p->site] < 0) return;
  for (;;) {
    int32_t l = s->left[p->site], r = s->right[p->site];
    int32_t next;
    if (p->heading)
      next = r > -1 ? r : l;
    else
      next = l > -1 ? l : r;
    p->heading = (next == r);
    const double* t = s->pos + 3 * (int64_t)next;
    double d[3] = {p->pos[0] - t[0], p->pos[1] - t[1], p->pos[2] - t[2]};
    double dist = v3_norm(d);
    if (dist / s->v < dt) {
      p->pos[0] = t[0];
      p->pos[1] = t[1];
      p->pos[2] = t[2];
      p->site = next;
      dt -= dist / s->v;
      p->crossings++;
      trace_push(s, p, -1 - next);
    } else {
      double e[3] = {t[0] - p->pos[0], t[1] - p->pos[1], t[2] - p->pos[2]};
      double nn = v3_norm(e);
      double den = nn != 0 ? nn : 1.0;
      double u[3] = {e[0] / den, e[1] / den, e[2] / den};
      double k = s->v * dt;
      for (int c = 0; c < 3; ++c) p->pos[c] = p->pos[c] + k * u[c];
      return;
    }
  }
}

/* particle::step, particle.cpp:57-80 */
static void step(const orc_sim* s, orc_exc* p, double dt, double* cum_buf, int32_t* col_buf) {
  for (int c = 0; c < 3; ++c) p->old[c] = p->pos[c];
  while (p->ff <= dt) {
    dt -= p->ff;
    fly(s, p, p->ff);
    int32_t ns = update_state(s, p, cum_buf, col_buf);
    p->hops++;
    trace_push(s, p, ns);
    if (ns != p->site) {
      p->site = ns;
      for (int c = 0; c < 3; ++c) p->pos[c] = s->pos[3 * (int64_t)ns + c];
    }
    p->ff = ff_time(s, p->site, &p->rng);
  }
  fly(s, p, dt);
  p->ff -= dt;
}

int64_t orc_sim_n_inject(const orc_sim* s) { return s->n_inject; }

int orc_sim_create_excitons(orc_sim* s, int mode, int n_sections, int64_t n_exc, uint64_t seed,
                            uint64_t stream_base, int use_csr) {
  s->mode = mode;
  s->use_csr = use_csr;
  if (use_csr && !s->rowptr) orc_sim_build_csr(s);
  free(s->inject);
  s->inject = (int32_t*)malloc(sizeof(int32_t) * s->n);
  s->n_inject = 0;
  if (mode == 0) {
    /* injection_region, monte_carlo.cpp:203-228 */
    int n = n_sections;
    if (!(n > 1 && n % 2 == 1)) return -1;
    double g[3][64];
    if (n + 1 > 64) return -1;
    for (int c = 0; c < 3; ++c) {
      double d = (s->mx[c] - s->mn[c]) / (double)n;
      for (int i = 0; i <= n; ++i) g[c][i] = (double)i * d + s->mn[c];
    }
    for (int64_t i = 0; i < s->n; ++i) {
      const double* p = s->pos + 3 * i;
      if (g[0][n / 2] <= p[0] && p[0] <= g[0][n / 2 + 1] && g[1][n / 2] <= p[1] && p[1] <= g[1][n / 2 + 1] &&
          g[2][n / 2] <= p[2] && p[2] <= g[2][n / 2 + 1])
        s->inject[s->n_inject++] = (int32_t)i;
    }
    /* get_removal_domain, monte_carlo.cpp:231-251 */
    for (int c = 0; c < 3; ++c) {
      s->rmin[c] = g[c][1];
      s->rmax[c] = g[c][n - 1];
    }
  } else {
    for (int64_t i = 0; i < s->n; ++i) s->inject[s->n_inject++] = (int32_t)i;
  }
  if (s->n_inject == 0) return -2;
  if (s->exc) {
    for (int64_t e = 0; e < s->n_exc; ++e) free(s->exc[e].trace);
    free(s->exc);
  }
  s->n_exc = n_exc;
  s->exc = (orc_exc*)calloc(n_exc > 0 ? n_exc : 1, sizeof(orc_exc));
  /* kubo_create_particles, monte_carlo.cpp:308-316, and particle(pos, s, v), particle.h:48-52 */
  for (int64_t e = 0; e < n_exc; ++e) {
    orc_exc* p = s->exc + e;
    orc_rng_init(&p->rng, seed, stream_base + (uint64_t)e, 0);
    int dice = orc_rand(&p->rng) % (int)s->n_inject;
    int32_t site = s->inject[dice];
    p->site = site;
    for (int c = 0; c < 3; ++c) p->pos[c] = p->old[c] = s->pos[3 * (int64_t)site + c];
    p->ff = ff_time(s, site, &p->rng);
    p->heading = orc_rand(&p->rng) % 2;
    if (e < s->n_trace) p->trace = (int32_t*)malloc(sizeof(int32_t) * (s->trace_cap ? s->trace_cap : 1));
  }
  return 0;
}

void orc_sim_set_trace(orc_sim* s, int64_t n_trace, int64_t cap) {
  s->n_trace = n_trace;
  s->trace_cap = cap;
}

int64_t orc_sim_get_trace(const orc_sim* s, int64_t e, int32_t* buf, int64_t cap) {
  if (e < 0 || e >= s->n_exc || !s->exc[e].trace) return -1;
  const orc_exc* p = s->exc + e;
  int64_t n = p->trace_n < s->trace_cap ? p->trace_n : s->trace_cap;
  if (n > cap) n = cap;
  memcpy(buf, p->trace, sizeof(int32_t) * n);
  return p->trace_n;
}

/* kubo_step, monte_carlo.cpp:319-342, then the sums of kubo_save_avg_dispalcement_squared :398-402 */
int orc_sim_step(orc_sim* s, double dt, int64_t n_steps, double* msd_sums) {
  return orc_sim_step_batches(s, dt, n_steps, 1, msd_sums);
}

int orc_sim_step_batches(orc_sim* s, double dt, int64_t n_steps, int batches, double* msd_sums) {
  if (batches < 1) return -1;
  for (int64_t st = 0; st < n_steps; ++st) {
#pragma omp parallel num_threads(s->n_threads)
    {
      double* cum = NULL;
      int32_t* col = NULL;
      if (!s->use_csr) {
        cum = (double*)malloc(sizeof(double) * (s->max_list + 1));
        col = (int32_t*)malloc(sizeof(int32_t) * (s->max_list + 1));
      }
#pragma omp for schedule(dynamic, 16)
      for (int64_t e = 0; e < s->n_exc; ++e) {
        orc_exc* p = s->exc + e;
        step(s, p, dt, cum, col);
        for (int c = 0; c < 3; ++c) p->delta[c] += p->pos[c] - p->old[c];
        if (s->mode == 0) {
          int out = 0;
          for (int c = 0; c < 3; ++c) out |= (p->pos[c] < s->rmin[c]) | (s->rmax[c] < p->pos[c]);
          if (out) {
            int dice = orc_rand(&p->rng) % (int)s->n_inject;
            int32_t site = s->inject[dice];
            for (int c = 0; c < 3; ++c) p->pos[c] = s->pos[3 * (int64_t)site + c];
            p->site = site;
            trace_push(s, p, INT32_MIN);
            trace_push(s, p, site);
          }
        }
      }
      free(cum);
      free(col);
    }
    if (msd_sums) {
      double* row = msd_sums + (size_t)st * batches * 3;
      for (int b = 0; b < 3 * batches; ++b) row[b] = 0.0;
      for (int64_t e = 0; e < s->n_exc; ++e) {
        const orc_exc* p = s->exc + e;
        double* m = row + 3 * ((e / 32) % batches);
        m[0] += p->delta[0] * p->delta[0];
        m[1] += p->delta[1] * p->delta[1];
        m[2] += p->delta[2] * p->delta[2];
      }
    }
  }
  return 0;
}

void orc_sim_get_excitons(const orc_sim* s, int32_t* site, double* pos, double* old_pos, double* delta, double* ff,
                          int32_t* heading, uint64_t* draws, int64_t* hops) {
  for (int64_t e = 0; e < s->n_exc; ++e) {
    const orc_exc* p = s->exc + e;
    if (site) site[e] = p->site;
    for (int c = 0; c < 3; ++c) {
      if (pos) pos[3 * e + c] = p->pos[c];
      if (old_pos) old_pos[3 * e + c] = p->old[c];
      if (delta) delta[3 * e + c] = p->delta[c];
    }
    if (ff) ff[e] = p->ff;
    if (heading) heading[e] = p->heading;
    if (draws) draws[e] = p->rng.n;
    if (hops) hops[e] = p->hops;
  }
}

int64_t orc_sim_total_hops(const orc_sim* s) {
  int64_t h = 0;
  for (int64_t e = 0; e < s->n_exc; ++e) h += s->exc[e].hops;
  return h;
}
int64_t orc_sim_total_crossings(const orc_sim* s) {
  int64_t h = 0;
  for (int64_t e = 0; e < s->n_exc; ++e) h += s->exc[e].crossings;
  return h;
}

void orc_sim_destroy(orc_sim* s) {
  if (!s) return;
  free(s->pos);
  free(s->orient);
  free(s->left);
  free(s->right);
  free(s->tab_store);
  free(s->species_store);
  free(s->cell_start);
  free(s->cell_members);
  free(s->close_cells);
  free(s->total);
  free(s->inv_total);
  free(s->rowptr);
  free(s->col);
  free(s->cum);
  free(s->inject);
  free(s->c_list[0]);
  free(s->c_list[1]);
  free(s->live);
  if (s->exc) {
    for (int64_t e = 0; e < s->n_exc; ++e) free(s->exc[e].trace);
    free(s->exc);
  }
  free(s);
}

/* ---------------------------------------------------------------- contacts mode
 * The second driver of mc::monte_carlo: init (monte_carlo.h:157-195), step (:343-354),
 * save_metrics (:519-643) and repopulate_contacts (:443-481), run as src/main.cpp:94-105 does.
 * Exciton slots replace the reference's particle vector: slot k draws from Philox stream k, and
 * its draw counter carries on when its exciton is removed and a new one takes the slot.  The
 * initial excitons take slots 0.. in create_particles order; the n new excitons of a contact take
 * the n lowest empty slots, in creation order. */

static void contact_bounds(const orc_sim* s, double* ymin, double* ymax, double* dy) {
  *ymin = s->mn[1];
  *ymax = s->mx[1];
  *dy = (*ymax - *ymin) / (double)s->n_seg;
}

/* particle(pos, s, v) at a drawn site of `list` (repopulate :478-488, create_particles :305-310,
 * particle.h:48-52), drawing from p's stream. */
static void place(const orc_sim* s, orc_exc* p, const int32_t* list, int64_t n_list) {
  int dice = (int)((uint32_t)orc_rand(&p->rng) % (uint64_t)n_list);
  int32_t site = list[dice];
  p->site = site;
  for (int c = 0; c < 3; ++c) {
    p->pos[c] = p->old[c] = s->pos[3 * (int64_t)site + c];
    p->delta[c] = 0.0;
  }
  p->ff = ff_time(s, site, &p->rng);
  p->heading = orc_rand(&p->rng) % 2;
}

/* into an empty slot, whose stream carries on */
static void create_at(orc_sim* s, int64_t slot, const int32_t* list, int64_t n_list) {
  place(s, s->exc + slot, list, n_list);
  s->live[slot] = 1;
}

int orc_contacts_init(orc_sim* s, int n_seg, int64_t pop1, int64_t pop2, uint64_t seed, int64_t capacity,
                      double* area, int64_t* stat_pop, int64_t* n_contact) {
  if (n_seg < 2 || pop1 < 0 || pop2 < 0 || capacity <= 0 || pop1 > INT32_MAX || pop2 > INT32_MAX) return -1;
  if (!s->rowptr) orc_sim_build_csr(s);
  s->use_csr = 1;
  s->mode = 2; /* particle::step only: no Green-Kubo removal */
  s->n_seg = n_seg;
  s->c_seed = seed;
  s->c_pop[0] = pop1;
  s->c_pop[1] = pop2;
  double ymin, ymax, dy;
  contact_bounds(s, &ymin, &ymax, &dy);
  /* get_area, monte_carlo.h:646-688 (the else-if leaves a maximum unset while the minimum moves) */
  double *xmn = malloc(sizeof(double) * n_seg), *xmx = malloc(sizeof(double) * n_seg);
  double *zmn = malloc(sizeof(double) * n_seg), *zmx = malloc(sizeof(double) * n_seg);
  for (int i = 0; i < n_seg; ++i) {
    xmx[i] = s->mn[0];
    xmn[i] = s->mx[0];
    zmx[i] = s->mn[2];
    zmn[i] = s->mx[2];
  }
  for (int64_t k = 0; k < s->n; ++k) {
    const double* q = s->pos + 3 * k;
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
  for (int i = 0; i < n_seg; ++i) {
    if (area) area[i] = (zmx[i] - zmn[i]) * (xmx[i] - xmn[i]);
    if (stat_pop) stat_pop[i] = 0;
  }
  free(xmn);
  free(xmx);
  free(zmn);
  free(zmx);
  /* get_scatterer_statistics, monte_carlo.h:691-719 */
  if (stat_pop)
    for (int64_t k = 0; k < s->n; ++k) stat_pop[(int)(fabs(s->pos[3 * k + 1] - ymin) / dy) % n_seg]++;
  /* contact_scats(1) and contact_scats(n_seg), monte_carlo.h:494-517 */
  for (int c = 0; c < 2; ++c) {
    int i = c == 0 ? 1 : n_seg;
    double y1 = ymin + (double)(i - 1) * dy, y2 = ymin + (double)i * dy;
    free(s->c_list[c]);
    s->c_list[c] = malloc(sizeof(int32_t) * (s->n ? s->n : 1));
    s->c_n[c] = 0;
    for (int64_t k = 0; k < s->n; ++k) {
      double y = s->pos[3 * k + 1];
      if (y >= y1 && y <= y2) s->c_list[c][s->c_n[c]++] = (int32_t)k;
    }
    if (n_contact) n_contact[c] = s->c_n[c];
  }
  /* slots */
  if (s->exc) {
    for (int64_t e = 0; e < s->n_exc; ++e) free(s->exc[e].trace);
    free(s->exc);
  }
  free(s->live);
  s->n_exc = capacity;
  s->exc = (orc_exc*)calloc(capacity, sizeof(orc_exc));
  s->live = (uint8_t*)calloc(capacity, 1);
  for (int64_t e = 0; e < capacity; ++e) {
    orc_rng_init(&s->exc[e].rng, seed, (uint64_t)e, 0);
    s->exc[e].site = -1;
  }
  /* create_particles(domain, n_seg, scats, c1_pop, c2_pop), monte_carlo.h:274-316 */
  int32_t* seg = malloc(sizeof(int32_t) * (s->n ? s->n : 1));
  double dp = (double)(pop2 - pop1) / ((double)n_seg - 1);
  int64_t slot = 0;
  int rc = 0;
  for (int i = 0; i < n_seg && rc == 0; ++i) {
    int n_particle = (int)round((double)pop1 + (double)i * dp);
    double y1 = ymin + (double)i * dy;
    double y2 = y1 + dy;
    int64_t ns = 0;
    for (int64_t k = 0; k < s->n; ++k) {
      double y = s->pos[3 * k + 1];
      if (y1 <= y && y < y2) seg[ns++] = (int32_t)k;
    }
    if (n_particle > 0 && ns == 0) rc = -3; /* the reference takes rand() % 0 */
    for (int n = 0; n < n_particle && rc == 0; ++n) {
      if (slot >= capacity) {
        rc = -4;
        break;
      }
      create_at(s, slot++, seg, ns);
    }
  }
  free(seg);
  return rc;
}

/* repopulate(y1, y2, n, list), monte_carlo.h:458-491, on slots */
static int repopulate(orc_sim* s, double y1, double y2, int64_t n_new, const int32_t* list, int64_t n_list) {
  for (int64_t e = 0; e < s->n_exc; ++e) {
    if (!s->live[e]) continue;
    double y = s->exc[e].pos[1];
    if (y >= y1 && y <= y2) {
      s->live[e] = 0;
      s->exc[e].site = -1;
    }
  }
  if (n_new > 0 && n_list == 0) return -3;
  int64_t made = 0;
  for (int64_t e = 0; e < s->n_exc && made < n_new; ++e)
    if (!s->live[e]) {
      create_at(s, e, list, n_list);
      ++made;
    }
  return made < n_new ? -4 : 0;
}

void orc_sim_use_csr(orc_sim* s, int use_csr) {
  if (use_csr && !s->rowptr) orc_sim_build_csr(s);
  s->use_csr = use_csr;
}

int orc_contacts_step(orc_sim* s, double dt, int64_t n_steps, int64_t* pop, int64_t* curr, int64_t* n_live) {
  if (s->mode != 2) return -1;
  const int n_seg = s->n_seg;
  double ymin, ymax, dy;
  contact_bounds(s, &ymin, &ymax, &dy);
  double* yif = malloc(sizeof(double) * n_seg);
  for (int i = 1; i < n_seg; ++i) yif[i - 1] = ymin + dy * (double)i; /* save_currents :595-597 */
  int rc = 0;
  for (int64_t st = 0; st < n_steps && rc == 0; ++st) {
    /* step(dt), monte_carlo.h:343-354 */
#pragma omp parallel num_threads(s->n_threads)
    {
      double* cum = NULL;
      int32_t* col = NULL;
      if (!s->use_csr) { /* the reference's neighbour search on every hop */
        cum = (double*)malloc(sizeof(double) * (s->max_list + 1));
        col = (int32_t*)malloc(sizeof(int32_t) * (s->max_list + 1));
      }
#pragma omp for schedule(dynamic, 16)
      for (int64_t e = 0; e < s->n_exc; ++e)
        if (s->live[e]) step(s, s->exc + e, dt, cum, col);
      free(cum);
      free(col);
    }
    /* save_population_profile :525-581 and save_currents :584-643 (the counts; the files hold
     * count / (area dy) and count / (interface area dt)) */
    int64_t* P = pop + st * n_seg;
    int64_t* J = curr + st * (n_seg - 1);
    for (int i = 0; i < n_seg; ++i) P[i] = 0;
    for (int i = 0; i < n_seg - 1; ++i) J[i] = 0;
    for (int64_t e = 0; e < s->n_exc; ++e) {
      if (!s->live[e]) continue;
      const orc_exc* p = s->exc + e;
      int i = (int)((p->pos[1] - ymin) / dy);
      i = i < 0 ? 0 : (i < n_seg ? i : n_seg - 1);
      P[i]++;
      for (int k = 0; k < n_seg - 1; ++k) {
        if (p->old[1] < yif[k] && p->pos[1] >= yif[k])
          J[k]++;
        else if (p->old[1] >= yif[k] && p->pos[1] < yif[k])
          J[k]--;
      }
    }
    /* repopulate_contacts, monte_carlo.h:443-455 */
    rc = repopulate(s, ymin, ymin + dy, s->c_pop[0], s->c_list[0], s->c_n[0]);
    if (rc == 0) rc = repopulate(s, ymin + (double)(n_seg - 1) * dy, ymax, s->c_pop[1], s->c_list[1], s->c_n[1]);
    int64_t live = 0;
    for (int64_t e = 0; e < s->n_exc; ++e) live += s->live[e];
    if (n_live) n_live[st] = live;
  }
  free(yif);
  return rc;
}

/* track_particle, monte_carlo.h:786-818: one exciton placed at a random contact-1 site (repopulate
 * into an empty list) and stepped until its y reaches the last slab, at most max_steps steps.
 * Track k draws from Philox stream 2^32 + k. */
int orc_contacts_track(orc_sim* s, int64_t first, int n_tracks, double dt, int64_t max_steps, double* path,
                       int64_t* len, int32_t* arrived) {
  if (s->mode != 2 || s->c_n[0] == 0) return -1;
  double ymin, ymax, dy;
  contact_bounds(s, &ymin, &ymax, &dy);
  const double y_end = ymin + (double)(s->n_seg - 1) * dy;
#pragma omp parallel for num_threads(s->n_threads) schedule(dynamic, 1)
  for (int t = 0; t < n_tracks; ++t) {
    orc_exc p;
    memset(&p, 0, sizeof p);
    orc_rng_init(&p.rng, s->c_seed, (1ull << 32) + (uint64_t)(first + t), 0);
    place(s, &p, s->c_list[0], s->c_n[0]);
    int64_t n = 0;
    double* out = path + (int64_t)t * max_steps * 3;
    while (p.pos[1] < y_end && n < max_steps) {
      step(s, &p, dt, NULL, NULL);
      for (int c = 0; c < 3; ++c) out[3 * n + c] = p.pos[c];
      ++n;
    }
    len[t] = n;
    arrived[t] = p.pos[1] < y_end ? 0 : 1;
  }
  return 0;
}

double orc_log_export(double x) { return orc_log(x); }
void orc_log_array(const double* x, double* out, int64_t n) {
  for (int64_t i = 0; i < n; ++i) out[i] = orc_log(x[i]);
}
double orc_acos_export(double x) { return orc_acos(x); }
void orc_philox_export(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) { orc_philox4x32_10(ctr, key, out); }
int orc_rand_export(uint64_t seed, uint64_t stream, uint64_t n) {
  orc_rng g;
  orc_rng_init(&g, seed, stream, n);
  return orc_rand(&g);
}
