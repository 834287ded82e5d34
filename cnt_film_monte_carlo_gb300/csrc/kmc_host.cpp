// kmc_host.cpp -- host-side reference algorithms of the C ABI (no device code).
// Compiled with -ffp-contract=off so every expression rounds as written.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/cntkmc.h"
#include "kmc_abi_guard.h"

namespace {

constexpr double kRefPi = 3.141592;  // src/helper/constants.h:10

inline double dot3(const double* a, const double* b) {
  double acc1 = 0.0, acc2 = 0.0;
  acc1 += a[0] * b[0];
  acc2 += a[1] * b[1];
  acc1 += a[2] * b[2];
  return acc1 + acc2;
}
inline double norm3(const double* a) { return std::sqrt(dot3(a, a)); }

// arma::linspace (used by monte_carlo.cpp:66-75,158-167): s + i (e - s)/(n - 1), last = e
void linspace(double start, double end, int64_t num, double* out) {
  if (num == 1) {
    out[0] = end;
    return;
  }
  if (num < 2) return;
  const double delta = (end - start) / double(num - 1);
  for (int64_t i = 0; i < num - 1; ++i) out[i] = start + double(i) * delta;
  out[num - 1] = end;
}

// A grid's point count {start, end, n}[2]: a whole number of points, 1 .. 2^31 - 1 (a NaN, a
// fraction below 1 or a huge value is refused before it is converted).
bool grid_count(double x, int64_t& n) {
  if (!(x >= 1.0 && x <= 2147483647.0)) return false;
  n = (int64_t)x;
  return true;
}

// One mesh matrix as the reference's arma::mat::load reads it: numbers separated by blanks
// (commas read as blanks), one matrix row per non-blank line, every row as long as the first.
// A token that is not a number fails the load, as it fails Armadillo's.
bool read_matrix(const std::string& path, std::vector<double>& v, int64_t& rows, int64_t& cols) {
  std::ifstream f(path);
  if (!f) return false;
  v.clear();
  rows = 0;
  cols = -1;
  std::string line;
  while (std::getline(f, line)) {
    for (auto& ch : line)
      if (ch == ',') ch = ' ';
    const char* s = line.c_str();
    int64_t c = 0;
    for (;;) {
      char* e;
      double x = std::strtod(s, &e);
      if (e == s) break;
      v.push_back(x);
      ++c;
      s = e;
    }
    while (*s == ' ' || *s == '\t' || *s == '\r' || *s == '\v' || *s == '\f') ++s;
    if (*s != '\0') return false;  // text that is not a number
    if (c == 0) continue;
    if (cols < 0) cols = c;
    if (c != cols) return false;
    ++rows;
  }
  // the stream stops at the end of the file, or on a read error (an allocation that failed inside
  // getline sets badbit rather than throwing): only the first is a matrix
  if (f.bad() || !f.eof()) return false;
  if (cols < 0) cols = 0;
  return true;
}

}  // namespace

extern "C" {

int kmc_trim_sites(int64_t n, double* pos, double* orient, int32_t* left, int32_t* right, const double lim[6],
                   int64_t* n_out) try {
  if (n < 0 || n > INT32_MAX || (n > 0 && (!pos || !orient || !left || !right)) || !lim || !n_out)
    return KMC_ERR_ARG;
  // links are followed and written below: each must be -1 or a site of the film
  for (int64_t i = 0; i < n; ++i)
    if (left[i] < -1 || left[i] >= n || right[i] < -1 || right[i] >= n) return KMC_ERR_ARG;
  // monte_carlo.h:730-750: exchange sites i and j, first pointing their tube neighbours at the new slots
  auto swap_sites = [&](int64_t i, int64_t j) {
    int32_t iL = left[i], iR = right[i], jL = left[j], jR = right[j];
    int32_t new_i = (int32_t)j, new_j = (int32_t)i;
    if (iL > -1) right[iL] = new_i;
    if (iR > -1) left[iR] = new_i;
    if (jL > -1) right[jL] = new_j;
    if (jR > -1) left[jR] = new_j;
    for (int c = 0; c < 3; ++c) {
      std::swap(pos[3 * i + c], pos[3 * j + c]);
      std::swap(orient[3 * i + c], orient[3 * j + c]);
    }
    std::swap(left[i], left[j]);
    std::swap(right[i], right[j]);
  };
  // monte_carlo.h:752-771: out-of-limit sites go to the end; their neighbours lose the link
  int64_t j = n;
  for (int64_t i = 0; i < j;) {
    const double* p = pos + 3 * i;
    if (p[0] < lim[0] || p[1] < lim[2] || p[2] < lim[4] || p[0] > lim[1] || p[1] > lim[3] || p[2] > lim[5]) {
      --j;
      swap_sites(i, j);
      if (left[j] > -1) right[left[j]] = -1;
      if (right[j] > -1) left[right[j]] = -1;
    } else {
      ++i;
    }
  }
  *n_out = j;
  return KMC_OK;
} catch (...) {
  const char* what = nullptr;
  return kmc::abi_status(&what);
}

int kmc_domain(int64_t n, const double* pos, double mn[3], double mx[3]) try {
  if (n <= 0 || !pos || !mn || !mx) return KMC_ERR_ARG;
  // find_simulation_domain, monte_carlo.h:328-340
  for (int c = 0; c < 3; ++c) mn[c] = mx[c] = pos[c];
  for (int64_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) {
      double p = pos[3 * i + c];
      mn[c] = mn[c] > p ? p : mn[c];
      mx[c] = mx[c] < p ? p : mx[c];
    }
  return KMC_OK;
} catch (...) {
  const char* what = nullptr;
  return kmc::abi_status(&what);
}

int kmc_forster2d_table(double gamma_0, const double distance[3], const double theta_deg[3], double* dist,
                        double* theta, double* rate) try {
  if (!distance || !theta_deg || !dist || !theta || !rate) return KMC_ERR_ARG;
  int64_t nd = 0, nt = 0;
  if (!grid_count(distance[2], nd) || !grid_count(theta_deg[2], nt)) return KMC_ERR_ARG;
  linspace(distance[0], distance[1], nd, dist);
  linspace(theta_deg[0], theta_deg[1], nt, theta);
  const double scale = kRefPi / 180;
  for (int64_t i = 0; i < nt; ++i) theta[i] = theta[i] * scale;
  // the Förster formula of create_forster_scatt_table (monte_carlo.cpp:174-187) at zero axis
  // shifts: gamma_0 cos^2(theta) (1 nm / d)^6
  for (int64_t i = 0; i < nd; ++i)
    for (int64_t k = 0; k < nt; ++k) {
      const double c = std::cos(theta[k]);
      rate[i * nt + k] = gamma_0 * (c * c) * std::pow(1.e-9 / dist[i], 6);
    }
  return KMC_OK;
} catch (...) {
  const char* what = nullptr;
  return kmc::abi_status(&what);
}

int kmc_species_rates(const kmc_species_model* m, int64_t n, const double* dist, const double* theta,
                      const int32_t* donor, const int32_t* acceptor, double* rate) try {
  if (!m || n < 0 || (n > 0 && (!dist || !theta || !donor || !acceptor || !rate))) return KMC_ERR_ARG;
  if (m->n_species < 1 || m->n_species > KMC_MAX_SPECIES || !m->energy || !m->diameter || !(m->diameter_ref > 0) ||
      !(m->width > 0) || !(m->kT > 0))
    return KMC_ERR_ARG;
  const double ell2 = m->near_field * m->near_field;
  for (int64_t i = 0; i < n; ++i) {
    const int32_t a = donor[i], b = acceptor[i];
    if (a < 0 || a >= m->n_species || b < 0 || b >= m->n_species) return KMC_ERR_ARG;
    // donor/acceptor factor: size of the two transition dipoles, spectral overlap of the two
    // exciton lines, and the Boltzmann factor of an uphill transfer
    const double de = m->energy[b] - m->energy[a];
    double s = (m->diameter[a] * m->diameter[b]) / (m->diameter_ref * m->diameter_ref);
    s = s * std::exp(-(de * de) / (2 * m->width * m->width));
    s = s * (de > 0 ? std::exp(-de / m->kT) : 1.0);
    // the Förster form of create_forster_scatt_table (monte_carlo.cpp:174-187) at zero axis
    // shifts, with an angle floor and a near-field length; sqrt(d^2) == d keeps the neutral
    // case equal to kmc_forster2d_table
    const double c = std::cos(theta[i]);
    const double r = std::sqrt(dist[i] * dist[i] + ell2);
    rate[i] = m->gamma_0 * s * (c * c + m->floor) * std::pow(1.e-9 / r, 6);
  }
  return KMC_OK;
} catch (...) {
  const char* what = nullptr;
  return kmc::abi_status(&what);
}

int kmc_forster_table(double gamma_0, const double theta_deg[3], const double zshift[3], const double ash1[3],
                      const double ash2[3], double* theta, double* zsh, double* a1, double* a2, double* rate) try {
  if (!theta_deg || !zshift || !ash1 || !ash2 || !theta || !zsh || !a1 || !a2 || !rate) return KMC_ERR_ARG;
  int64_t nt = 0, nz = 0, n1 = 0, n2 = 0;
  if (!grid_count(theta_deg[2], nt) || !grid_count(zshift[2], nz) || !grid_count(ash1[2], n1) ||
      !grid_count(ash2[2], n2))
    return KMC_ERR_ARG;
  linspace(zshift[0], zshift[1], nz, zsh);
  linspace(ash1[0], ash1[1], n1, a1);
  linspace(ash2[0], ash2[1], n2, a2);
  linspace(theta_deg[0], theta_deg[1], nt, theta);
  const double scale = kRefPi / 180;
  for (int64_t i = 0; i < nt; ++i) theta[i] = theta[i] * scale;
  // monte_carlo.cpp:174-195: point dipoles on two axes at angle th, separated by zsh
  for (int64_t it = 0; it < nt; ++it) {
    const double th = theta[it];
    for (int64_t iz = 0; iz < nz; ++iz)
      for (int64_t i1 = 0; i1 < n1; ++i1)
        for (int64_t i2 = 0; i2 < n2; ++i2) {
          double r1[3] = {a1[i1], 0, 0};
          double r2[3] = {a2[i2] * std::cos(th), a2[i2] * std::sin(th), zsh[iz]};
          double dR[3] = {r1[0] - r2[0], r1[1] - r2[1], r1[2] - r2[2]};
          double n_r1 = norm3(r1), n_r2 = norm3(r2), n_dR = norm3(dR);
          double d1 = n_r1 != 0 ? n_r1 : 1.0, d2 = n_r2 != 0 ? n_r2 : 1.0, dd = n_dR != 0 ? n_dR : 1.0;
          double u1[3] = {r1[0] / d1, r1[1] / d1, r1[2] / d1};
          double u2[3] = {r2[0] / d2, r2[1] / d2, r2[2] / d2};
          double ud[3] = {dR[0] / dd, dR[1] / dd, dR[2] / dd};
          double af = std::cos(th) - 3 * dot3(u1, ud) * dot3(u2, ud);
          rate[((it * nz + iz) * n1 + i1) * n2 + i2] = gamma_0 * (af * af) * std::pow(1.e-9 / n_dR, 6);
        }
  }
  return KMC_OK;
} catch (...) {
  const char* what = nullptr;
  return kmc::abi_status(&what);
}

int kmc_read_mesh(const char* dir, int64_t* n_tubes, int64_t* n_points, double* pos, double* orient, int32_t* left,
                  int32_t* right) try {
  if (!dir || !n_tubes || !n_points) return KMC_ERR_ARG;
  static const char* names[6] = {"single_cnt.pos.x.dat",    "single_cnt.pos.y.dat",    "single_cnt.pos.z.dat",
                                 "single_cnt.orient.x.dat", "single_cnt.orient.y.dat", "single_cnt.orient.z.dat"};
  std::vector<double> m[6];
  int64_t rows = -1, cols = -1;
  for (int k = 0; k < 6; ++k) {
    int64_t r = 0, c = 0;
    if (!read_matrix(std::string(dir) + "/" + names[k], m[k], r, c)) return KMC_ERR_IO;
    if (rows >= 0 && (r != rows || c != cols)) return KMC_ERR_IO;
    rows = r;
    cols = c;
  }
  if (cols > 0 && rows > INT32_MAX / cols) return KMC_ERR_IO;  // site ids are 32-bit
  *n_tubes = rows;
  *n_points = cols;
  if (!pos && !orient && !left && !right) return KMC_OK;
  if (!pos || !orient || !left || !right) return KMC_ERR_ARG;
  // monte_carlo.h:249-262; positions scaled by 1e-9 (:211,225,239)
  for (int64_t i = 0; i < rows; ++i)
    for (int64_t j = 0; j < cols; ++j) {
      int64_t s = i * cols + j;
      for (int c = 0; c < 3; ++c) {
        pos[3 * s + c] = m[c][s] * 1.e-9;
        orient[3 * s + c] = m[3 + c][s];
      }
      left[s] = j > 0 ? (int32_t)(s - 1) : -1;
      right[s] = j + 1 < cols ? (int32_t)(s + 1) : -1;
    }
  return KMC_OK;
} catch (...) {
  const char* what = nullptr;
  return kmc::abi_status(&what);
}

// Two-sided 95% quantile of Student's t with nu degrees of freedom.  nu <= 31 (every fit of up
// to 32 batches): the quantiles themselves, the doubles nearest to the root of
// I_{nu/(nu+x^2)}(nu/2, 1/2) = 0.05 computed at 40 significant digits.  Beyond: the
// Cornish-Fisher expansion about the normal quantile (Abramowitz & Stegun 26.7.5), within 1.3e-8
// relative of the quantile at nu = 32 and closer above.
static double t975(int nu) {
  static const double exact[32] = {
      0,
      12.706204736174705, 4.302652729749464, 3.1824463052837095, 2.7764451051977943,
      2.5705818356363155, 2.44691185114497, 2.3646242515927853, 2.3060041352041667,
      2.2621571627982053, 2.228138851986275, 2.2009851600916397, 2.178812829667229,
      2.1603686564627926, 2.144786687917804, 2.1314495455597755, 2.1199052992212546,
      2.109815577833317, 2.1009220402410387, 2.0930240544083096, 2.085963447265865,
      2.0796138447276804, 2.0738730679040263, 2.0686576104190486, 2.063898561628026,
      2.0595385527532977, 2.055529438642873, 2.0518305164802855, 2.048407141795245,
      2.0452296421327043, 2.042272456301238, 2.0395134463964086};
  if (nu < 1) return NAN;
  if (nu <= 31) return exact[nu];
  const double z = 1.959963984540054, v = nu;
  const double z3 = z * z * z, z5 = z3 * z * z, z7 = z5 * z * z, z9 = z7 * z * z;
  return z + (z3 + z) / (4 * v) + (5 * z5 + 16 * z3 + 3 * z) / (96 * v * v) +
         (3 * z7 + 19 * z5 + 17 * z3 - 15 * z) / (384 * v * v * v) +
         (79 * z9 + 776 * z7 + 1482 * z5 - 1920 * z3 - 945 * z) / (92160 * v * v * v * v);
}

int kmc_fit_diffusion(const double* msd, const int64_t* counts, const double* times, int64_t n_steps, int32_t batches,
                      double fit_fraction, double D[3], double ci95[3]) try {
  if (!msd || !counts || !times || !D || !ci95 || n_steps < 2 || batches < 1 || !(fit_fraction > 0) ||
      fit_fraction > 1)
    return KMC_ERR_ARG;
  int64_t s0 = n_steps - (int64_t)std::ceil(fit_fraction * (double)n_steps);
  if (s0 < 0) s0 = 0;
  if (n_steps - s0 < 2) s0 = n_steps - 2;
  const int64_t m = n_steps - s0;
  double tm = 0;
  for (int64_t s = s0; s < n_steps; ++s) tm += times[s];
  tm /= (double)m;
  double sxx = 0;
  for (int64_t s = s0; s < n_steps; ++s) sxx += (times[s] - tm) * (times[s] - tm);
  if (!(sxx > 0)) return KMC_ERR_ARG;
  for (int k = 0; k < 3; ++k) {
    std::vector<double> db;
    for (int32_t b = 0; b < batches; ++b) {
      if (counts[b] <= 0) continue;
      double ym = 0;
      for (int64_t s = s0; s < n_steps; ++s) ym += msd[(s * batches + b) * 3 + k] / (double)counts[b];
      ym /= (double)m;
      double sxy = 0;
      for (int64_t s = s0; s < n_steps; ++s)
        sxy += (times[s] - tm) * (msd[(s * batches + b) * 3 + k] / (double)counts[b] - ym);
      db.push_back(sxy / sxx / 2.0);
    }
    if (db.empty()) return KMC_ERR_ARG;
    double mean = 0;
    for (double x : db) mean += x;
    mean /= (double)db.size();
    double var = 0;
    for (double x : db) var += (x - mean) * (x - mean);
    D[k] = mean;
    ci95[k] = db.size() > 1 ? t975((int)db.size() - 1) * std::sqrt(var / (double)(db.size() - 1)) / std::sqrt((double)db.size())
                            : NAN;
  }
  return KMC_OK;
} catch (...) {
  const char* what = nullptr;
  return kmc::abi_status(&what);
}

const char* kmc_version(void) { return "cntkmc 0.3 (sm_103a)"; }

}  // extern "C"
