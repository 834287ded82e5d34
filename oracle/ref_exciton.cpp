// ref_exciton.cpp -- TEST INFRASTRUCTURE: runs the reference's own exciton physics
// (src/exciton_transfer/cnt.cpp and exciton_transfer.cpp, compiled unchanged against
// oracle/shim_et/armadillo by oracle/Makefile) and writes what it computes to a binary file
// that tests/golden/make_golden_exciton.py turns into fixtures.
//
//   ref_exciton OUT n1 m1 cells1 n2 m2 cells2 [z_shift ash1 ash2 theta]...
//
// For each tube (cnt::calculate_exciton_dispersion, cnt.cpp:1056-1080): lattice vectors,
// radius, K1/K2/dk_l, K2-extended parameters, unit-cell positions, the K2-extended bands, the
// valleys and relevant-state windows, vq, PI, eps, the three A-exciton dispersions with the
// A2-singlet wavefunctions and state indices.  For the donor/acceptor pair
// (exciton_transfer.cpp): the relevant states, the matched pairs of the first geometry with
// |Q|, J and M of each, and first_order at every geometry.  Distances in m, angles in radians.
//
// Record format: u32 name length, name, u8 kind (0 f64, 1 complex128, 2 i64), u32 ndim,
// u64 dims[ndim] (row-major, last index fastest), data.
#include <array>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <experimental/filesystem>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include <armadillo>

#include "../lib/json.hpp"
#include "exciton_transfer/constants.h"
#include "exciton_transfer/small.h"
#include "helper/prepare_directory.hpp"
#include "helper/progress.hpp"

// the driver reads the classes' internal state: every header above is already included, so
// only the reference's two class definitions see the redefinition (GCC keeps member layout in
// declaration order regardless of access, so the objects match the separately compiled code)
#define private public
#include "exciton_transfer/cnt.h"
#include "exciton_transfer/exciton_transfer.h"
#undef private

namespace {

std::ofstream out;

void rec(const std::string& name, uint8_t kind, const std::vector<uint64_t>& dims, const void* data, size_t bytes) {
  uint32_t nl = (uint32_t)name.size();
  out.write((const char*)&nl, 4);
  out.write(name.data(), nl);
  out.write((const char*)&kind, 1);
  uint32_t nd = (uint32_t)dims.size();
  out.write((const char*)&nd, 4);
  for (uint64_t d : dims) out.write((const char*)&d, 8);
  out.write((const char*)data, (std::streamsize)bytes);
}
void f64(const std::string& n, const std::vector<double>& v, std::vector<uint64_t> dims = {}) {
  if (dims.empty()) dims = {v.size()};
  rec(n, 0, dims, v.data(), v.size() * 8);
}
void c128(const std::string& n, const std::vector<std::complex<double>>& v, std::vector<uint64_t> dims) {
  rec(n, 1, dims, v.data(), v.size() * 16);
}
void i64(const std::string& n, const std::vector<int64_t>& v, std::vector<uint64_t> dims = {}) {
  if (dims.empty()) dims = {v.size()};
  rec(n, 2, dims, v.data(), v.size() * 8);
}
template <typename eT>
std::vector<double> vec_of(const arma::Mat<eT>& m) {  // row-major copy
  std::vector<double> v(m.n_elem);
  for (arma::uword r = 0; r < m.n_rows; ++r)
    for (arma::uword c = 0; c < m.n_cols; ++c) v[r * m.n_cols + c] = double(m.at(r, c));
  return v;
}
void mat(const std::string& n, const arma::mat& m) { f64(n, vec_of(m), {m.n_rows, m.n_cols}); }
void cube(const std::string& n, const arma::cube& q) {  // [r][c][s]
  std::vector<double> v(q.n_elem);
  for (arma::uword r = 0; r < q.n_rows; ++r)
    for (arma::uword c = 0; c < q.n_cols; ++c)
      for (arma::uword s = 0; s < q.n_slices; ++s) v[(r * q.n_cols + c) * q.n_slices + s] = q(r, c, s);
  f64(n, v, {q.n_rows, q.n_cols, q.n_slices});
}
void cxcube(const std::string& n, const arma::cx_cube& q) {
  std::vector<std::complex<double>> v(q.n_elem);
  for (arma::uword r = 0; r < q.n_rows; ++r)
    for (arma::uword c = 0; c < q.n_cols; ++c)
      for (arma::uword s = 0; s < q.n_slices; ++s) v[(r * q.n_cols + c) * q.n_slices + s] = q(r, c, s);
  c128(n, v, {q.n_rows, q.n_cols, q.n_slices});
}
void ucube(const std::string& n, const arma::ucube& q) {
  std::vector<int64_t> v(q.n_elem);
  for (arma::uword r = 0; r < q.n_rows; ++r)
    for (arma::uword c = 0; c < q.n_cols; ++c)
      for (arma::uword s = 0; s < q.n_slices; ++s) v[(r * q.n_cols + c) * q.n_slices + s] = (int64_t)q(r, c, s);
  i64(n, v, {q.n_rows, q.n_cols, q.n_slices});
}

void dump_tube(const std::string& p, const cnt& t) {
  i64(p + "ints", {t._n, t._m, t._number_of_cnt_unit_cells, t._Nu, t._M, t._Q, t._t1, t._t2});
  f64(p + "scalars", {t._radius, t._ch_len});
  for (auto nv : std::vector<std::pair<std::string, const arma::vec*>>{
           {"a1", &t._a1}, {"a2", &t._a2}, {"b1", &t._b1}, {"b2", &t._b2}, {"acc", &t._aCC_vec}, {"ch", &t._ch_vec},
           {"t_vec", &t._t_vec}, {"t_vec_3d", &t._t_vec_3d}, {"K1", &t._K1}, {"K2", &t._K2}, {"dk_l", &t._dk_l}})
    f64(p + nv.first, nv.second->mem);
  mat(p + "pos_a", t._pos_a);
  mat(p + "pos_b", t._pos_b);
  mat(p + "pos_u_3d", t._pos_u_3d);
  cube(p + "el_energy", t._elec_K2.energy);
  i64(p + "el_ranges", {t._elec_K2.ik_range[0], t._elec_K2.ik_range[1], t._elec_K2.mu_range[0], t._elec_K2.mu_range[1]});
  std::vector<int64_t> val;
  for (const auto& v : t._valleys_K2)
    for (const auto& a : v) val.insert(val.end(), {(int64_t)a[0], (int64_t)a[1]});
  i64(p + "valleys", val, {t._valleys_K2.size(), 2, 2});
  std::vector<int64_t> rel;
  for (const auto& v : t._relev_ik_range)
    for (const auto& a : v) rel.insert(rel.end(), {a[0], a[1]});
  i64(p + "relev", rel, {2, t._relev_ik_range[0].size(), 2});
  cxcube(p + "vq", t._vq.data);
  i64(p + "vq_ranges", {t._vq.iq_range[0], t._vq.iq_range[1], t._vq.mu_range[0], t._vq.mu_range[1]});
  mat(p + "pi", t._PI.data);
  mat(p + "eps", t._eps.data);
  for (const auto& ex : t._excitons) {
    std::string nm = ex.name == "A1 exciton" ? "A1" : ex.name == "A2 triplet exciton" ? "A2_triplet" : "A2_singlet";
    mat(p + nm, ex.energy);
    if (nm == "A2_singlet") {
      cxcube(p + "A2_singlet_psi", ex.psi);
      ucube(p + "ik_idx", ex.ik_idx);
      i64(p + "ik_cm_range", {ex.ik_cm_range[0], ex.ik_cm_range[1]});
    }
  }
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 8 || (argc - 8) % 4 != 0) {
    std::fprintf(stderr, "usage: ref_exciton OUT n1 m1 cells1 n2 m2 cells2 [z_shift ash1 ash2 theta]...\n");
    return 2;
  }
  // the classes write their data files under $HOME (exciton_transfer's constructor) and under the
  // parent directory given here; both go to a scratch directory
  const char* scratch = std::getenv("KMC_REF_SCRATCH");
  if (!scratch) {
    std::fprintf(stderr, "ref_exciton: set KMC_REF_SCRATCH to a scratch directory\n");
    return 2;
  }
  setenv("HOME", scratch, 1);
  std::streambuf* keep = std::cout.rdbuf();
  std::ofstream devnull("/dev/null");
  std::cout.rdbuf(devnull.rdbuf());  // the classes' progress output

  auto make = [&](int n, int m, int cells) {
    nlohmann::json j;
    j["chirality"] = {n, m};
    j["length"] = {cells, "cnt unit cells"};
    j["keep old results"] = false;
    return new cnt(j, std::string(scratch) + "/cnt_" + std::to_string(cells));
  };
  cnt* c1 = make(std::atoi(argv[2]), std::atoi(argv[3]), std::atoi(argv[4]));
  c1->calculate_exciton_dispersion();
  const bool same = std::atoi(argv[2]) == std::atoi(argv[5]) && std::atoi(argv[3]) == std::atoi(argv[6]) &&
                    std::atoi(argv[4]) == std::atoi(argv[7]);
  cnt* c2 = c1;
  if (!same) {
    c2 = make(std::atoi(argv[5]), std::atoi(argv[6]), std::atoi(argv[7]));
    c2->calculate_exciton_dispersion();
  }

  out.open(argv[1], std::ios::binary);
  dump_tube("d_", *c1);
  dump_tube("a_", *c2);

  exciton_transfer et(*c1, *c2);
  const double min_energy = c1->A2_singlet().energy.min();
  auto ds = et.get_relevant_states(c1->A2_singlet(), min_energy);
  auto as = et.get_relevant_states(c2->A2_singlet(), min_energy);
  for (auto sp : {std::make_pair(std::string("d_states"), &ds), std::make_pair(std::string("a_states"), &as)}) {
    std::vector<double> e;
    std::vector<int64_t> idx;
    for (const auto& s : *sp.second) {
      e.push_back(s.energy);
      idx.insert(idx.end(), {s.ik_cm, s.ik_cm_idx, s.i_principal});
    }
    f64(sp.first + "_energy", e);
    i64(sp.first + "_index", idx, {sp.second->size(), 3});
  }
  auto pairs = et.match_states(ds, as);
  std::vector<double> geo;
  for (int a = 8; a < argc; ++a) geo.push_back(std::atof(argv[a]));
  const size_t ng = geo.size() / 4;
  f64("geometries", geo, {ng, 4});
  if (ng > 0) {
    std::vector<int64_t> pidx;
    std::vector<double> absq, absm;
    std::vector<std::complex<double>> jv;
    const double zs = geo[0], th = geo[3];
    const std::array<double, 2> sh = {geo[1], geo[2]};
    for (const auto& pr : pairs) {
      std::complex<double> Q = et.calculate_Q(pr);
      std::complex<double> J = et.calculate_J(pr, sh, zs, th);
      pidx.insert(pidx.end(), {pr.i.ik_cm, pr.i.i_principal, pr.f.ik_cm, pr.f.i_principal});
      absq.push_back(std::abs(Q));
      jv.push_back(J);
      absm.push_back(std::abs(Q * J) / std::sqrt(pr.i.cnt_obj->length_in_meter() * pr.f.cnt_obj->length_in_meter()));
    }
    i64("pairs", pidx, {pairs.size(), 4});
    f64("pair_abs_q", absq);
    c128("pair_j", jv, {jv.size()});
    f64("pair_m", absm);
  }
  std::vector<double> rates;
  for (size_t g = 0; g < ng; ++g)
    rates.push_back(et.first_order(geo[4 * g], {geo[4 * g + 1], geo[4 * g + 2]}, geo[4 * g + 3], false));
  f64("first_order", rates);
  out.close();
  std::cout.rdbuf(keep);
  std::printf("ref_exciton: %zu donor states, %zu acceptor states, %zu matched pairs, %zu geometries\n", ds.size(),
              as.size(), pairs.size(), ng);
  return 0;
}
