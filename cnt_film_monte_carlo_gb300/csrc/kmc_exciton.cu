// kmc_exciton.cu -- the reference's exciton-transfer physics on the GPU: the labeller of pair
// transfer rates (the "davoody" rate table of src/monte_carlo/monte_carlo.cpp:64-153 and the
// labels of the rate surrogate).
//
// A tube (kmc_cnt_create) follows cnt::calculate_exciton_dispersion
// (src/exciton_transfer/cnt.cpp:1056-1080):
//   host:   lattice and K2-extended parameters (cnt.cpp:16-114), unit-cell positions (:120-210),
//           the two-band K2-extended bands (:302-345, closed form), valleys (:348-410) and the
//           relevant-state windows (:419-505), then the A2-singlet bookkeeping (:962-997) and
//           each state's part of the Q matrix element (exciton_transfer.cpp:276-297);
//   device: the Ohno-potential Fourier sums vq (cnt.cpp:520-631, k_vq), the static polarisation
//           PI (:634-732, k_pi), the Bethe-Salpeter kernels of every centre-of-mass momentum
//           (:783-947, k_bse_fill / k_bse_combine) and their eigen-decompositions (:949-965,
//           k_jacobi: a batched cyclic Jacobi solver for Hermitian matrices, one block per
//           matrix, the matrix in shared memory).
// A pair rate (kmc_exciton_rates) follows exciton_transfer::first_order
// (exciton_transfer.cpp:380-424): thermally relevant states and their Lorentzian matching on the
// host (:226-250, exciton_transfer.h:167-196), and the Coulomb sum J (:307-377) of every matched
// pair at every geometry on the device (k_coulomb_j): for one geometry J(p, q) = sum_i a_p(i)
// sum_j b_q(j) / |R_i - R_j| over the two tubes' graphene unit cells, with a_p, b_q the
// centre-of-mass phase factors of the donor and acceptor momenta.  It is tiled like an N-body
// kernel: each thread owns one donor cell, the acceptor cells of the geometry and their phases
// are staged through shared memory, and the per-thread sums for every acceptor momentum stay in
// registers.  KMC_PREC_FP64 computes it in FP64; KMC_PREC_MIXED uses FP32 positions, distances
// and tile sums, added into FP64 per tile (relative error ~1e-6 against FP64).  k_rates then
// forms sum_pairs w |Q J|^2 per geometry.
// Constants are evaluated as the reference evaluates them (src/exciton_transfer/constants.h,
// cnt.h:25-33), including pi = 3.141592 and the single-precision sqrt(3) of the lattice constant.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/cntkmc.h"
#include "kmc_abi_guard.h"
#include "kmc_internal.h"

using cx = std::complex<double>;

// a tube's exciton model (opaque in the C ABI)
struct kmc_cnt {
  int n = 0, m = 0, cells = 0, Nu = 0, M = 0, Q = 0, t1 = 0, t2 = 0;
  double a1[2], a2[2], b1[2], b2[2], acc[2], ch[2], t_vec[2], t3[3], K1[2], K2[2], dk_l[2];
  double radius = 0, ch_len = 0, length = 0, au = 0;
  std::vector<double> pos_a, pos_b, pos_u_3d;  // [Nu][2], [Nu][2], [Nu][3]
  int nk = 0, n_mu = 0;                        // K2-extended grid: ik in [0, nk), mu in [0, n_mu)
  std::vector<double> energy;                  // [2][nk][n_mu]
  std::vector<cx> wf;                          // [n_mu][2 atoms][2 bands][nk]
  std::vector<std::array<int, 4>> valleys;     // (ik, mu) of the two valleys of each pair
  std::vector<std::array<int, 2>> relev[2];    // relevant (ik, mu) of each valley
  int iq0 = 0, nq = 0, mq0 = 0, nmq = 0;       // vq / PI / eps ranges
  std::vector<cx> vq;                          // [nq][nmq][4]
  std::vector<double> pi, eps;                 // [nq][nmq]
  int ik_cm0 = 0, nk_cm = 0, nr = 0;           // centre-of-mass momenta, relevant states per valley
  std::vector<double> ex_energy[3];            // A1, A2 triplet, A2 singlet [nk_cm][nr]
  std::vector<cx> psi_s;                       // A2 singlet [nk_cm][2 nr][nr]
  std::vector<int> ik_idx;                     // [nk_cm][4][2 nr]
  std::vector<cx> q_part;                      // [nk_cm][nr]
};

namespace {

using kmc::ctx_device;
using kmc::ctx_set_error;
using kmc::ctx_stream;

// constants.h:10-18 and cnt.h:25-33, evaluated as the reference does
struct Consts {
  double pi = 3.141592, inv_pi = 1. / 3.141592;
  double eV = 1.6 * std::pow(10, -19.0);
  double hb = 6.5 * std::pow(10, -16.0) * (1.6 * std::pow(10, -19.0));
  double kb = 1.3865 * std::pow(10, -23.0);
  double eps0 = 8.85 * std::pow(10, -12);
  double q0 = 1.6 * std::pow(10, -19);
  double a_cc = 1.42e-10;
  double a_l = std::sqrt(float(3.0)) * 1.42e-10;
  double t0 = 2.7 * (1.6 * std::pow(10, -19.0));
  double upp = 11.3 * (1.6 * std::pow(10, -19.0));
};
const Consts& K() {
  static const Consts k;
  return k;
}

template <typename T>
struct DBuf {  // device buffer owned by one call
  T* p = nullptr;
  size_t n = 0;
  ~DBuf() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t count) {
    if (p) cudaFree(p);
    p = nullptr;
    n = count ? count : 1;
    return cudaMalloc(&p, n * sizeof(T));
  }
};

inline double dot2(const double* a, const double* b) {  // two accumulators, as the shim's dot
  double s0 = 0 + a[0] * b[0], s1 = 0 + a[1] * b[1];
  return s0 + s1;
}
inline double norm2(const double* a) { return std::sqrt(dot2(a, a)); }

void linspace(double s, double e, int64_t n, double* out) {
  if (n == 1) {
    out[0] = e;
    return;
  }
  const double d = (e - s) / double(n - 1);
  for (int64_t i = 0; i + 1 < n; ++i) out[i] = s + double(i) * d;
  out[n - 1] = e;
}

// ---------------------------------------------------------------- host steps of the tube model
bool geometry(kmc_cnt& t, std::string& err) {
  const Consts& k = K();
  const int n = t.n, m = t.m;
  const double al = k.a_l;
  // cnt.cpp:19-22 (operations in the written order)
  t.a1[0] = al * std::sqrt(3.0) / 2.0, t.a1[1] = +al / 2.0;
  t.a2[0] = al * std::sqrt(3.0) / 2.0, t.a2[1] = -al / 2.0;
  t.b1[0] = 1.0 / std::sqrt(3.0) * 2.0 * k.pi / al, t.b1[1] = +2.0 * k.pi / al;
  t.b2[0] = 1.0 / std::sqrt(3.0) * 2.0 * k.pi / al, t.b2[1] = -2.0 * k.pi / al;
  for (int d = 0; d < 2; ++d) t.acc[d] = 1.0 / 3.0 * (t.a1[d] + t.a2[d]);
  for (int d = 0; d < 2; ++d) t.ch[d] = double(n) * t.a1[d] + double(m) * t.a2[d];
  t.ch_len = norm2(t.ch);
  t.radius = t.ch_len / 2.0 / k.pi;
  const int dR = std::gcd(2 * n + m, n + 2 * m);
  t.t1 = +(2 * m + n) / dR;
  t.t2 = -(2 * n + m) / dR;
  for (int d = 0; d < 2; ++d) t.t_vec[d] = double(t.t1) * t.a1[d] + double(t.t2) * t.a2[d];
  t.Nu = int(2 * (std::pow(n, 2) + std::pow(m, 2) + n * m) / dR);
  // rotate so that the chiral vector lies along x (cnt.cpp:41-56)
  const double nc = norm2(t.ch);
  const double c = t.ch[0] / nc, s = t.ch[1] / nc;
  auto rot = [&](double* v) {
    const double x = c * v[0] + s * v[1], y = -s * v[0] + c * v[1];
    v[0] = x, v[1] = y;
  };
  for (double* v : {t.ch, t.t_vec, t.a1, t.a2, t.b1, t.b2, t.acc}) rot(v);
  t.t3[0] = 0, t.t3[1] = t.t_vec[1], t.t3[2] = 0;
  // cnt.cpp:81-87
  for (int d = 0; d < 2; ++d) {
    t.K1[d] = (-double(t.t2) * t.b1[d] + double(t.t1) * t.b2[d]) / double(t.Nu);
    t.K2[d] = (double(m) * t.b1[d] - double(n) * t.b2[d]) / double(t.Nu);
    t.dk_l[d] = t.K2[d] / double(t.cells);
  }
  // K2-extended parameters (cnt.cpp:93-112)
  const double p_min = (1. / double(t.t1) + 1. / double(n)) / (double(m) / double(n) - double(t.t2) / double(t.t1));
  const double p_max =
      (1. / double(t.t1) + double(t.Nu) / double(n)) / (double(m) / double(n) - double(t.t2) / double(t.t1));
  bool found = false;
  for (int p = (int)std::ceil(p_min); p < std::ceil(p_max); p++)
    if (((1 + t.t2 * p) % t.t1) == 0) {
      const int q = (1 + t.t2 * p) / t.t1;
      t.M = m * p - n * q;
      t.Q = std::gcd(t.Nu, t.M);
      found = true;
      break;
    }
  if (!found) {
    err = "no K2-extended representation for this chirality";
    return false;
  }
  // unit cells of one tube cell (cnt.cpp:124-165)
  t.pos_a.assign(2 * t.Nu, 0.0);
  t.pos_b.assign(2 * t.Nu, 0.0);
  int kk = 0;
  for (int i = 0; i <= t.t1 + n; i++)
    for (int j = t.t2; j <= m; j++) {
      const bool f1 = double(t.t2 * i) / (double)t.t1 <= double(j);
      const bool f2 = double(m * i) / (double)n >= double(j);
      const bool f3 = double(t.t2 * (i - n)) / double(t.t1) > double(j - m);
      const bool f4 = double(m * (i - t.t1)) / double(n) < double(j - t.t2);
      if (f1 && f2 && f3 && f4) {
        if (kk >= t.Nu) {
          err = "more unit cells than Nu";
          return false;
        }
        double* pa = &t.pos_a[2 * kk];
        double* pb = &t.pos_b[2 * kk];
        for (int d = 0; d < 2; ++d) pa[d] = double(i) * t.a1[d] + double(j) * t.a2[d];
        for (int d = 0; d < 2; ++d) pb[d] = pa[d] + t.acc[d];
        for (double* p : {pa, pb})
          for (int d = 0; d < 2; ++d) {
            if (p[d] > t.ch[d]) p[d] -= t.ch[d];
            if (p[d] < 0.0) p[d] += t.ch[d];
          }
        kk++;
      }
    }
  if (kk != t.Nu) {
    err = "unit-cell count differs from Nu";
    return false;
  }
  t.pos_u_3d.assign(3 * t.Nu, 0.0);
  for (int i = 0; i < t.Nu; ++i) {
    t.pos_u_3d[3 * i] = t.radius * std::cos(t.pos_a[2 * i] / t.radius);
    t.pos_u_3d[3 * i + 1] = t.pos_a[2 * i + 1];
    t.pos_u_3d[3 * i + 2] = t.radius * std::sin(t.pos_a[2 * i] / t.radius);
  }
  t.length = double(t.cells) * norm2(t.t_vec);                // cnt.h:306-309
  t.au = std::abs(t.a1[0] * t.a2[1] - t.a1[1] * t.a2[0]);     // cnt.h:346-349
  return true;
}

// K2-extended two-band bands (cnt.cpp:302-345, 1061-1064)
void bands(kmc_cnt& t) {
  const Consts& k = K();
  t.nk = t.Nu / t.Q * t.cells;
  t.n_mu = t.Q;
  t.energy.assign((size_t)2 * t.nk * t.n_mu, 0.0);
  t.wf.assign((size_t)t.n_mu * 4 * t.nk, cx(0));
  double d1[2], d2[2], d3[2];
  for (int d = 0; d < 2; ++d) {
    d1[d] = (t.a1[d] + t.a2[d]) / 3.;
    d2[d] = (t.a1[d] - 2. * t.a2[d]) / 3.;
    d3[d] = (t.a2[d] - 2. * t.a1[d]) / 3.;
  }
  for (int mu = 0; mu < t.n_mu; mu++)
    for (int ik = 0; ik < t.nk; ik++) {
      double kv[2];
      for (int d = 0; d < 2; ++d) kv[d] = double(mu) * t.K1[d] + double(ik) * t.dk_l[d];
      const cx fk = std::exp(cx(0, dot2(kv, d1))) + std::exp(cx(0, dot2(kv, d2))) + std::exp(cx(0, dot2(kv, d3)));
      t.energy[((size_t)1 * t.nk + ik) * t.n_mu + mu] = +k.t0 * std::abs(fk);
      t.energy[((size_t)0 * t.nk + ik) * t.n_mu + mu] = -k.t0 * std::abs(fk);
      auto w = [&](int atom, int band) -> cx& { return t.wf[(((size_t)mu * 2 + atom) * 2 + band) * t.nk + ik]; };
      w(0, 1) = +1. / std::sqrt(2.);
      w(0, 0) = +1. / std::sqrt(2.);
      w(1, 1) = -1. / std::sqrt(2.) * std::conj(fk) / std::abs(fk);
      w(1, 0) = +1. / std::sqrt(2.) * std::conj(fk) / std::abs(fk);
    }
}

double E(const kmc_cnt& t, int band, int ik, int mu) { return t.energy[((size_t)band * t.nk + ik) * t.n_mu + mu]; }

// conduction-band valleys, sorted by energy with std::sort as the reference sorts them, paired
// (cnt.cpp:348-410)
bool valleys(kmc_cnt& t, std::string& err) {
  std::vector<std::array<unsigned, 2>> idx;
  for (int ik = 0; ik < t.nk; ik++)
    for (int mu = 0; mu < t.n_mu; mu++) {
      int p1 = ik + 1, m1 = ik - 1;
      while (p1 >= t.nk) p1 -= t.nk;
      while (m1 < 0) m1 += t.nk;
      if (E(t, 1, ik, mu) < E(t, 1, m1, mu) && E(t, 1, ik, mu) < E(t, 1, p1, mu)) idx.push_back({(unsigned)ik, (unsigned)mu});
    }
  std::sort(idx.begin(), idx.end(),
            [&](const auto& s1, const auto& s2) { return E(t, 1, s1[0], s1[1]) < E(t, 1, s2[0], s2[1]); });
  for (size_t i = 0; i < idx.size() / 2; i++)
    t.valleys.push_back({(int)idx[2 * i][0], (int)idx[2 * i][1], (int)idx[2 * i + 1][0], (int)idx[2 * i + 1][1]});
  if (t.valleys.empty()) {
    err = "no conduction-band valley pair";
    return false;
  }
  return true;
}

// states within delta of each valley bottom of the first valley pair (cnt.cpp:419-505)
void relevant_window(kmc_cnt& t, double delta) {
  for (int v = 0; v < 2; ++v) {
    auto& out = t.relev[v];
    out.clear();
    const int ik_b = t.valleys[0][2 * v], mu_b = t.valleys[0][2 * v + 1];
    const double max_e = E(t, 1, ik_b, mu_b) + delta;
    out.push_back({ik_b, mu_b});
    bool in_range = true;
    int count = 0;
    while (in_range) {
      in_range = false;
      count++;
      int ik = ik_b + count;
      while (ik >= t.nk) ik -= t.nk;
      if (E(t, 1, ik, mu_b) < max_e) {
        out.push_back({ik, mu_b});
        in_range = true;
      }
      ik = ik_b - count;
      while (ik < 0) ik += t.nk;
      if (E(t, 1, ik, mu_b) < max_e) {
        out.insert(out.begin(), {ik, mu_b});
        in_range = true;
      }
    }
  }
}

// ---------------------------------------------------------------- device kernels
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }

template <int NT>
__device__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < NT / 32; ++i) s += sh[i];
  return s;  // valid in thread 0
}

// vq(q, mu, pair) = sum_R exp(i q.R) U(R) / (2 Nu n): one block per (iq, mu) (cnt.cpp:570-600)
constexpr int kVqThreads = 256;
__global__ void __launch_bounds__(kVqThreads) k_vq(const double2* __restrict__ rel, const double* __restrict__ pot,
                                                   int npos, int iq0, int mq0, int nmq, double dk0, double dk1,
                                                   double K10, double K11, double scale, double2* __restrict__ vq) {
  __shared__ double sh[kVqThreads / 32];
  const int b = blockIdx.x, iq = iq0 + b / nmq, mu = mq0 + b % nmq;
  const double q0 = double(iq) * dk0 + double(mu) * K10, q1 = double(iq) * dk1 + double(mu) * K11;
  for (int s = 0; s < 4; ++s) {
    double re = 0, im = 0;
    for (int k = threadIdx.x; k < npos; k += kVqThreads) {
      const double2 R = rel[(size_t)s * npos + k];
      const double ph = (0 + q0 * R.x) + (0 + q1 * R.y);
      double sn, cs;
      sincos(ph, &sn, &cs);
      const double u = pot[(size_t)s * npos + k];
      re += cs * u;
      im += sn * u;
    }
    const double sr = block_sum<kVqThreads>(re, sh);
    const double si = block_sum<kVqThreads>(im, sh);
    if (threadIdx.x == 0) vq[(size_t)b * 4 + s] = make_double2(sr * scale, si * scale);
  }
}

// PI(q, mu_q): one block per (iq, mu_q), threads over the band states (cnt.cpp:680-705)
constexpr int kPiThreads = 256;
__global__ void __launch_bounds__(kPiThreads) k_pi(const double* __restrict__ en, const double2* __restrict__ wf, int nk,
                                                   int n_mu, int iq0, int mq0, int nmq, int wrap, double* __restrict__ pi) {
  __shared__ double sh[kPiThreads / 32];
  const int b = blockIdx.x, iq = iq0 + b / nmq, mu_q = mq0 + b % nmq;
  auto W = [&](int mu, int atom, int band, int ik) { return wf[(((size_t)mu * 2 + atom) * 2 + band) * nk + ik]; };
  auto En = [&](int band, int ik, int mu) { return en[((size_t)band * nk + ik) * n_mu + mu]; };
  double acc = 0;
  for (int s = threadIdx.x; s < nk * n_mu; s += kPiThreads) {
    const int ik = s / n_mu, mu_k = s % n_mu;
    int mu_kq = mu_k + mu_q, ikq = ik + iq;
    while (mu_kq >= n_mu) {
      mu_kq -= n_mu;
      ikq += wrap;
    }
    while (mu_kq < 0) {
      mu_kq += n_mu;
      ikq -= wrap;
    }
    ikq %= nk;
    if (ikq < 0) ikq += nk;
    // |<v(k)|c(k+q)>|^2 and |<c(k)|v(k+q)>|^2, dot products with two accumulators
    const double2 a0 = cmul(cconj(W(mu_k, 0, 0, ik)), W(mu_kq, 0, 1, ikq));
    const double2 a1 = cmul(cconj(W(mu_k, 1, 0, ik)), W(mu_kq, 1, 1, ikq));
    const double2 c0 = cmul(cconj(W(mu_k, 0, 1, ik)), W(mu_kq, 0, 0, ikq));
    const double2 c1 = cmul(cconj(W(mu_k, 1, 1, ik)), W(mu_kq, 1, 0, ikq));
    const double x = hypot(a0.x + a1.x, a0.y + a1.y), y = hypot(c0.x + c1.x, c0.y + c1.y);
    acc += x * x / (En(1, ikq, mu_kq) - En(0, ik, mu_k)) + y * y / (En(1, ik, mu_k) - En(0, ikq, mu_kq));
  }
  const double tot = block_sum<kPiThreads>(acc, sh);
  if (threadIdx.x == 0) pi[b] = 2 * tot;
}

struct BseArgs {
  const double* en;
  const double2* wf;
  const double2* vq;
  const double* eps;
  const int2* v1;  // relevant (ik, mu) of valley 1
  const int2* v2;
  int nk, n_mu, iq0, mq0, nmq, nr, ik_cm0;
  double2* a11;  // [nk_cm][nr][nr] filled entries
  double2* a12;
  double2* ax;
};

__device__ __forceinline__ int wrapk(int ik, int nk) {
  ik %= nk;
  return ik < 0 ? ik + nk : ik;
}

// one entry of each Bethe-Salpeter kernel as calculate_A_excitons fills it (cnt.cpp:836-923):
// kernel_11 and the exchange kernel on the lower triangle, kernel_12 on (c, nr-1-vp), vp >= c
__global__ void k_bse_fill(BseArgs a) {
  const int ikc_m = blockIdx.y, ik_cm = a.ik_cm0 + ikc_m;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = a.nr;
  if (e >= n * n) return;
  const int c = e / n, col = e % n;
  auto W = [&](int mu, int atom, int band, int ik) { return a.wf[(((size_t)mu * 2 + atom) * 2 + band) * a.nk + ik]; };
  auto direct = [&](int ik_c, int mu_c, int ik_v, int mu_v, int ik_cp, int mu_cp, int ik_vp, int mu_vp) {
    const int dk = wrapk(ik_c - ik_cp, a.nk), dmu = mu_c - mu_cp;
    const size_t q = (size_t)(dk - a.iq0) * a.nmq + (dmu - a.mq0);
    double2 s = make_double2(0, 0);
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j) {
        double2 t = cmul(cmul(cmul(cconj(W(mu_c, i, 1, ik_c)), W(mu_v, j, 0, ik_v)), W(mu_cp, i, 1, ik_cp)),
                         cconj(W(mu_vp, j, 0, ik_vp)));
        t = cmul(t, a.vq[q * 4 + 2 * i + j]);
        const double ep = a.eps[q];
        s = cadd(s, make_double2(t.x / ep, t.y / ep));
      }
    return s;
  };
  auto exchange = [&](int ik_c, int mu_c, int ik_v, int mu_v, int ik_cp, int mu_cp, int ik_vp, int mu_vp) {
    const size_t q = (size_t)(ik_cm - a.iq0) * a.nmq + (0 - a.mq0);
    double2 s = make_double2(0, 0);
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j) {
        double2 t = cmul(cmul(cmul(cconj(W(mu_c, i, 1, ik_c)), W(mu_v, i, 0, ik_v)), W(mu_cp, j, 1, ik_cp)),
                         cconj(W(mu_vp, j, 0, ik_vp)));
        s = cadd(s, cmul(t, a.vq[q * 4 + 2 * i + j]));
      }
    return s;
  };
  const int ik_c = a.v1[c].x, mu_c = a.v1[c].y;
  const int ik_v = wrapk(ik_c - ik_cm, a.nk), mu_v = mu_c;
  const size_t o = ((size_t)ikc_m * n + c) * n + col;
  double2 f11 = make_double2(0, 0), fx = make_double2(0, 0), f12 = make_double2(0, 0);
  if (col <= c) {
    const int ik_cp = a.v1[col].x, mu_cp = a.v1[col].y;
    const int ik_vp = wrapk(ik_cp - ik_cm, a.nk), mu_vp = mu_cp;
    if (col == c)
      f11.x = a.en[((size_t)1 * a.nk + ik_c) * a.n_mu + mu_c] - a.en[((size_t)0 * a.nk + ik_v) * a.n_mu + mu_c];
    const double2 d = direct(ik_c, mu_c, ik_v, mu_v, ik_cp, mu_cp, ik_vp, mu_vp);
    f11 = make_double2(f11.x - d.x, f11.y - d.y);
    const double2 x = exchange(ik_c, mu_c, ik_v, mu_v, ik_cp, mu_cp, ik_vp, mu_vp);
    fx = make_double2(2 * x.x, 2 * x.y);
  }
  const int vp = n - 1 - col;
  if (vp >= c) {
    const int ik_vp = a.v2[vp].x, mu_vp = a.v2[vp].y;
    const int ik_cp = wrapk(ik_vp + ik_cm, a.nk), mu_cp = mu_vp;
    const double2 d = direct(ik_c, mu_c, ik_v, mu_v, ik_cp, mu_cp, ik_vp, mu_vp);
    f12 = make_double2(-d.x, -d.y);
  }
  a.a11[o] = f11;
  a.a12[o] = f12;
  a.ax[o] = fx;
}

// kernel += kernel^H, diagonal halved (cnt.cpp:926-935), then the three Hamiltonians:
// A1 = K11 - K12, A2 triplet = K11 + K12, A2 singlet = K11 + K12 + 2 Kx (cnt.cpp:950-962)
__global__ void k_bse_combine(const double2* a11, const double2* a12, const double2* ax, int nr, int nk_cm,
                              double2* h) {
  const int ikc_m = blockIdx.y;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nr * nr) return;
  const int r = e / nr, c = e % nr;
  const size_t base = (size_t)ikc_m * nr * nr;
  auto k = [&](const double2* A) {
    const double2 x = A[base + (size_t)r * nr + c], y = A[base + (size_t)c * nr + r];
    double2 s = make_double2(x.x + y.x, x.y - y.y);
    if (r == c) s = make_double2(s.x / 2, s.y / 2);
    return s;
  };
  const double2 k11 = k(a11), k12 = k(a12), kx = k(ax);
  const size_t sz = (size_t)nk_cm * nr * nr;
  h[base + e] = make_double2(k11.x - k12.x, k11.y - k12.y);
  h[sz + base + e] = make_double2(k11.x + k12.x, k11.y + k12.y);
  h[2 * sz + base + e] = make_double2((k11.x + k12.x) + 2 * kx.x, (k11.y + k12.y) + 2 * kx.y);
}

// Batched eigen-decomposition of Hermitian matrices by cyclic Jacobi rotations (Jacobi 1846;
// the complex rotation first removes the phase of a_pq with a diagonal unitary, then applies the
// real rotation t = sign(tau) / (|tau| + sqrt(1 + tau^2)), tau = (a_qq - a_pp) / (2 |a_pq|)).
// One block per matrix; the matrix and the eigenvectors live in shared memory; every sweep
// visits the pairs in row order, the block's threads updating the two rows and columns of each
// rotation together.  Sweeps stop when the off-diagonal mass falls below 1e-30 of the matrix's
// (at most kJacobiSweeps).  Eigenvalues ascending (stable order), vectors in the columns.
constexpr int kJacobiThreads = 128;
constexpr int kJacobiSweeps = 60;
__global__ void __launch_bounds__(kJacobiThreads) k_jacobi(const double2* __restrict__ h, int n, double* __restrict__ w,
                                                           double2* __restrict__ v, int32_t* __restrict__ sweeps_out) {
  extern __shared__ double2 smem[];
  double2* A = smem;          // [n][n] row-major
  double2* V = smem + n * n;  // [n][n]
  __shared__ double red[kJacobiThreads / 32];
  __shared__ double rot[4];   // c, s, e^{-i phi} (re, im)
  __shared__ int order[64];
  const size_t base = (size_t)blockIdx.x * n * n;
  for (int e = threadIdx.x; e < n * n; e += kJacobiThreads) {
    A[e] = h[base + e];
    V[e] = make_double2((e / n) == (e % n) ? 1.0 : 0.0, 0.0);
  }
  __syncthreads();
  double fro = 0;
  for (int e = threadIdx.x; e < n * n; e += kJacobiThreads) fro += A[e].x * A[e].x + A[e].y * A[e].y;
  fro = block_sum<kJacobiThreads>(fro, red);
  if (threadIdx.x == 0) red[0] = fro;
  __syncthreads();
  fro = red[0];
  int sweep = 0;
  for (; sweep < kJacobiSweeps; ++sweep) {
    double off = 0;
    for (int e = threadIdx.x; e < n * n; e += kJacobiThreads)
      if (e / n < e % n) off += A[e].x * A[e].x + A[e].y * A[e].y;
    off = block_sum<kJacobiThreads>(off, red);
    __syncthreads();
    if (threadIdx.x == 0) red[0] = off;
    __syncthreads();
    off = red[0];
    __syncthreads();
    if (!(off > 1e-30 * fro)) break;
    for (int p = 0; p + 1 < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double2 b = A[p * n + q];
        const double ab = hypot(b.x, b.y);
        if (ab == 0) continue;  // uniform: every thread reads the same shared value
        if (threadIdx.x == 0) {
          const double alpha = A[p * n + p].x, gamma = A[q * n + q].x;
          const double tau = (gamma - alpha) / (2 * ab);
          const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1 + tau * tau));
          const double c = 1 / sqrt(1 + t * t);
          rot[0] = c;
          rot[1] = t * c;
          rot[2] = b.x / ab;   // e^{-i phi} = conj(b) / |b|
          rot[3] = -b.y / ab;
        }
        __syncthreads();
        const double c = rot[0], s = rot[1];
        const double2 em = make_double2(rot[2], rot[3]);
        // U = [[c, s], [-s e^{-i phi}, c e^{-i phi}]] on columns p, q
        const double2 uqp = make_double2(-s * em.x, -s * em.y), uqq = make_double2(c * em.x, c * em.y);
        for (int k = threadIdx.x; k < n; k += kJacobiThreads) {  // A <- A U, V <- V U
          const double2 akp = A[k * n + p], akq = A[k * n + q];
          A[k * n + p] = cadd(make_double2(akp.x * c, akp.y * c), cmul(akq, uqp));
          A[k * n + q] = cadd(make_double2(akp.x * s, akp.y * s), cmul(akq, uqq));
          const double2 vkp = V[k * n + p], vkq = V[k * n + q];
          V[k * n + p] = cadd(make_double2(vkp.x * c, vkp.y * c), cmul(vkq, uqp));
          V[k * n + q] = cadd(make_double2(vkp.x * s, vkp.y * s), cmul(vkq, uqq));
        }
        __syncthreads();
        for (int k = threadIdx.x; k < n; k += kJacobiThreads) {  // A <- U^H A
          const double2 apk = A[p * n + k], aqk = A[q * n + k];
          A[p * n + k] = cadd(make_double2(c * apk.x, c * apk.y), cmul(cconj(uqp), aqk));
          A[q * n + k] = cadd(make_double2(s * apk.x, s * apk.y), cmul(cconj(uqq), aqk));
        }
        __syncthreads();
        if (threadIdx.x == 0) {
          A[p * n + q] = make_double2(0, 0);
          A[q * n + p] = make_double2(0, 0);
          A[p * n + p].y = 0;
          A[q * n + q].y = 0;
        }
        __syncthreads();
      }
  }
  if (threadIdx.x == 0) {  // stable ascending order of the eigenvalues
    for (int i = 0; i < n; ++i) order[i] = i;
    for (int i = 1; i < n; ++i) {
      const int o = order[i];
      int j = i - 1;
      while (j >= 0 && A[order[j] * n + order[j]].x > A[o * n + o].x) {
        order[j + 1] = order[j];
        --j;
      }
      order[j + 1] = o;
    }
    sweeps_out[blockIdx.x] = sweep;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < n; j += kJacobiThreads) w[(size_t)blockIdx.x * n + j] = A[order[j] * n + order[j]].x;
  for (int e = threadIdx.x; e < n * n; e += kJacobiThreads) {
    const int r = e / n, j = e % n;
    v[base + e] = V[r * n + order[j]];  // [row][eigenvector]
  }
}

// ---------------------------------------------------------------- Coulomb sum J on the device
struct JGeom {
  double zsh, ash1, ash2, ct, st;  // z shift, axis shifts, cos and sin of the angle
};

template <typename T>
struct Vec3;
template <>
struct Vec3<float> {
  typedef float3 type;
};
template <>
struct Vec3<double> {
  typedef double3 type;
};
template <typename T>
struct Cx;
template <>
struct Cx<float> {
  typedef float2 type;
};
template <>
struct Cx<double> {
  typedef double2 type;
};

__device__ __forceinline__ double inv_len(double r2) { return 1.0 / sqrt(r2); }

constexpr int kJThreads = 128;
constexpr int kJTile = 128;
constexpr int kJMaxQ = 16;

// part[g][tile][p][q] = sum over this block's donor cells i of a_p(i) sum_j b_q(j) / |R_i - R_j(g)|.
// Positions are the centred base positions of make_Ru_3d (exciton_transfer.cpp:310-330); the
// donor is shifted by ash1 along its axis, the acceptor by ash2 along its axis and zsh in z, then
// rotated by the angle about z.  Grid: (donor tiles, geometries).
template <typename T, int NQ>
__global__ void __launch_bounds__(kJThreads) k_coulomb_j(const double3* __restrict__ rd, int nd,
                                                         const double3* __restrict__ ra, int na,
                                                         const double2* __restrict__ ap, int np,
                                                         const double2* __restrict__ bq, int nq,
                                                         const JGeom* __restrict__ geo, double2* __restrict__ part) {
  typedef typename Vec3<T>::type V3;
  typedef typename Cx<T>::type C2;
  __shared__ V3 sr[kJTile];
  __shared__ C2 sb[kJTile * NQ];
  __shared__ double2 red[kJThreads / 32][NQ];
  const JGeom g = geo[blockIdx.y];
  const int i = blockIdx.x * kJThreads + threadIdx.x;
  const bool live = i < nd;
  T xi = 0, yi = 0, zi = 0;
  if (live) {
    const double3 r = rd[i];
    xi = (T)r.x;
    yi = (T)(r.y + g.ash1);
    zi = (T)r.z;
  }
  double2 tot[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) tot[q] = make_double2(0, 0);
  for (int j0 = 0; j0 < na; j0 += kJTile) {
    const int nt = min(kJTile, na - j0);
    __syncthreads();
    for (int j = threadIdx.x; j < nt; j += kJThreads) {
      const double3 r = ra[j0 + j];
      const double x = r.x, y = r.y + g.ash2, z = r.z + g.zsh;
      V3 v;
      v.x = (T)(x * g.ct - y * g.st);
      v.y = (T)(x * g.st + y * g.ct);
      v.z = (T)z;
      sr[j] = v;
#pragma unroll
      for (int q = 0; q < NQ; ++q) {  // momenta beyond nq are zero and add nothing
        const double2 b = q < nq ? bq[(size_t)q * na + j0 + j] : make_double2(0, 0);
        C2 c;
        c.x = (T)b.x;
        c.y = (T)b.y;
        sb[j * NQ + q] = c;
      }
    }
    __syncthreads();
    C2 acc[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc[q].x = acc[q].y = 0;
    if (live)
      for (int j = 0; j < nt; ++j) {
        const V3 r = sr[j];
        const T dx = xi - r.x, dy = yi - r.y, dz = zi - r.z;
        const T inv = inv_len(dx * dx + dy * dy + dz * dz);
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          const C2 b = sb[j * NQ + q];
          acc[q].x += b.x * inv;
          acc[q].y += b.y * inv;
        }
      }
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      tot[q].x += (double)acc[q].x;
      tot[q].y += (double)acc[q].y;
    }
  }
  // sum over the block's donor cells of a_p(i) tot_q(i), for every (p, q)
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  for (int p = 0; p < np; ++p) {
    const double2 a = live ? ap[(size_t)p * nd + i] : make_double2(0, 0);
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      double2 v = cmul(a, tot[q]);
      for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
      }
      if (l == 0) red[w][q] = v;
    }
    __syncthreads();
    if (threadIdx.x < nq) {  // this block's partial, summed over blocks in order by k_j_reduce
      double2 s = make_double2(0, 0);
      for (int k = 0; k < kJThreads / 32; ++k) s = cadd(s, red[k][threadIdx.x]);
      part[(((size_t)blockIdx.y * gridDim.x + blockIdx.x) * np + p) * nq + threadIdx.x] = s;
    }
    __syncthreads();
  }
}

// The FP32 form of k_coulomb_j for KMC_PREC_MIXED: base positions (float4) and acceptor phases
// (float2) converted once on the host, the geometry applied in FP32, products accumulated with
// fused multiply-adds and the tile sums added into a Kahan-compensated FP32 total per acceptor
// momentum, so the FP64 pipe (1/64 of the FP32 rate on this GPU) is left out of the inner loops.
template <int NQ>
__global__ void __launch_bounds__(kJThreads) k_coulomb_j32(const float4* __restrict__ rd, int nd,
                                                           const float4* __restrict__ ra, int na,
                                                           const double2* __restrict__ ap, int np,
                                                           const float2* __restrict__ bq, int nq,
                                                           const JGeom* __restrict__ geo, double2* __restrict__ part) {
  __shared__ float4 sr[kJTile];
  __shared__ float2 sb[kJTile * NQ];
  __shared__ double2 prod[kJThreads * ((NQ < 8 ? NQ : 8) + 1)];  // [donor cell][q] products of one pass (padded rows)
  __shared__ double2 runs[kJThreads];                       // [run][q] sums of NQC rows
  const JGeom g = geo[blockIdx.y];
  const float ct = (float)g.ct, st = (float)g.st, a1 = (float)g.ash1, a2 = (float)g.ash2, zs = (float)g.zsh;
  const int i = blockIdx.x * kJThreads + threadIdx.x;
  const bool live = i < nd;
  float xi = 0, yi = 0, zi = 0;
  if (live) {
    const float4 r = rd[i];
    xi = r.x;
    yi = r.y + a1;
    zi = r.z;
  }
  float hx[NQ], hy[NQ], cx_[NQ], cy_[NQ];  // Kahan sums over the tiles
#pragma unroll
  for (int q = 0; q < NQ; ++q) hx[q] = hy[q] = cx_[q] = cy_[q] = 0.f;
  for (int j0 = 0; j0 < na; j0 += kJTile) {
    const int nt = min(kJTile, na - j0);
    __syncthreads();
    for (int j = threadIdx.x; j < nt; j += kJThreads) {
      const float4 r = ra[j0 + j];
      const float y = r.y + a2;
      sr[j] = make_float4(r.x * ct - y * st, r.x * st + y * ct, r.z + zs, 0.f);
    }
    // the phases [j][q], stored by consecutive threads to consecutive words (no bank conflicts)
    for (int e = threadIdx.x; e < nt * NQ; e += kJThreads) {
      const int j = e / NQ, q = e % NQ;
      sb[e] = q < nq ? bq[(size_t)q * na + j0 + j] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float ax[NQ], ay[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) ax[q] = ay[q] = 0.f;
    if (live)
      for (int j = 0; j < nt; ++j) {
        const float4 r = sr[j];
        const float dx = xi - r.x, dy = yi - r.y, dz = zi - r.z;
        const float inv = rsqrtf(__fmaf_rn(dz, dz, __fmaf_rn(dy, dy, dx * dx)));
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          const float2 b = sb[j * NQ + q];
          ax[q] = __fmaf_rn(b.x, inv, ax[q]);
          ay[q] = __fmaf_rn(b.y, inv, ay[q]);
        }
      }
#pragma unroll
    for (int q = 0; q < NQ; ++q) {  // Kahan: sum += tile, carrying the rounding error
      float y = ax[q] - cx_[q], t = hx[q] + y;
      cx_[q] = (t - hx[q]) - y;
      hx[q] = t;
      y = ay[q] - cy_[q];
      t = hy[q] + y;
      cy_[q] = (t - hy[q]) - y;
      hy[q] = t;
    }
  }
  // The block's sum over its donor cells of a_p(i) S_q(i), in FP64: S_q(i) formed once per q;
  // per donor momentum p, the products go to shared memory and are added column by column
  // (runs of NQC rows by 128 / NQC threads, then the runs in order by NQC threads), so each
  // thread adds a few values where a warp butterfly would add five levels on every lane (the
  // FP64 pipe runs at 1/64 of the FP32 rate on this GPU).
  double2 S[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) S[q] = make_double2((double)hx[q] - (double)cx_[q], (double)hy[q] - (double)cy_[q]);
  constexpr int NQC = NQ < 8 ? NQ : 8;   // q columns per pass
  constexpr int RUN = kJThreads / NQC;   // runs per column; each run adds NQC rows
  const int qc = threadIdx.x % NQC, run = threadIdx.x / NQC;
  for (int p = 0; p < np; ++p) {
    const double2 a = live ? ap[(size_t)p * nd + i] : make_double2(0, 0);
#pragma unroll
    for (int q0 = 0; q0 < NQ; q0 += NQC) {
#pragma unroll
      for (int q = 0; q < NQC; ++q) prod[threadIdx.x * (NQC + 1) + q] = cmul(a, S[q0 + q]);
      __syncthreads();
      double2 r = prod[(run * NQC) * (NQC + 1) + qc];
#pragma unroll
      for (int k = 1; k < NQC; ++k) r = cadd(r, prod[(run * NQC + k) * (NQC + 1) + qc]);
      runs[run * NQC + qc] = r;
      __syncthreads();
      if (threadIdx.x < NQC && q0 + threadIdx.x < nq) {  // this block's partial, summed over blocks in order by k_j_reduce
        double2 t = runs[threadIdx.x];
        for (int k = 1; k < RUN; ++k) t = cadd(t, runs[k * NQC + threadIdx.x]);
        part[(((size_t)blockIdx.y * gridDim.x + blockIdx.x) * np + p) * nq + q0 + threadIdx.x] = t;
      }
      __syncthreads();
    }
  }
}

// J[g][p][q] = sum over the donor tiles of the partials, in tile order (reproducible bit for bit)
__global__ void k_j_reduce(const double2* __restrict__ part, int ntile, int npq, int64_t n, double2* __restrict__ J) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int64_t g = e / npq, pq = e % npq;
  double2 s = make_double2(0, 0);
  for (int b = 0; b < ntile; ++b) s = cadd(s, part[((size_t)g * ntile + b) * npq + pq]);
  J[e] = s;
}

// rate[g] = sum_k w_k |J[g][p_k][q_k]|^2 (first_order's sum, exciton_transfer.cpp:405-411)
__global__ void k_rates(const double2* __restrict__ J, int np, int nq, int ng, const int2* __restrict__ pq,
                        const double* __restrict__ wk, int npairs, double* __restrict__ rate) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ng) return;
  double r = 0;
  for (int k = 0; k < npairs; ++k) {
    const double2 j = J[((size_t)g * np + pq[k].x) * nq + pq[k].y];
    r += wk[k] * (j.x * j.x + j.y * j.y);
  }
  rate[g] = r;
}

#define XCK(call)                                                                                       \
  do {                                                                                                  \
    cudaError_t _e = (call);                                                                            \
    if (_e != cudaSuccess) {                                                                            \
      err = std::string(#call) + ": " + cudaGetErrorString(_e);                                         \
      return _e == cudaErrorMemoryAllocation ? KMC_ERR_NOMEM : KMC_ERR_CUDA;                             \
    }                                                                                                   \
  } while (0)

template <typename T>
cudaError_t h2d(DBuf<T>& b, const T* h, size_t n, cudaStream_t s) {
  cudaError_t e = b.alloc(n);
  if (e == cudaSuccess && n) e = cudaMemcpyAsync(b.p, h, n * sizeof(T), cudaMemcpyHostToDevice, s);
  return e;
}

// vq, PI, eps, Bethe-Salpeter kernels and their eigenpairs on the device
int screening_and_excitons(kmc_cnt& t, cudaStream_t st, std::string& err) {
  kmc::NvtxRange phase("cnt: vq");
  const Consts& k = K();
  // vq (cnt.cpp:526-600)
  int ncell = t.cells;
  if (ncell % 2 == 0) ncell++;
  const int Nu = t.Nu, npos = Nu * ncell;
  std::vector<double> pd[4];
  for (auto& v : pd) v.assign(2 * Nu, 0.0);
  for (int i = 0; i < Nu; i++) {
    for (int d = 0; d < 2; ++d) {
      pd[0][2 * i + d] = t.pos_a[2 * i + d] - t.pos_a[d];
      pd[1][2 * i + d] = t.pos_a[2 * i + d] - t.pos_b[d];
      pd[2][2 * i + d] = t.pos_b[2 * i + d] - t.pos_a[d];
      pd[3][2 * i + d] = t.pos_b[2 * i + d] - t.pos_b[d];
    }
    for (auto& v : pd)
      if (v[2 * i] > t.ch[0] / 2) v[2 * i] -= t.ch[0];
  }
  std::vector<double2> rel((size_t)4 * npos);
  std::vector<double> pot((size_t)4 * npos);
  const double coeff = std::pow(4. * k.pi * k.eps0 * k.upp / k.q0 / k.q0, 2);
  const int h = (int)std::floor(double(ncell) / 2.);
  for (int i = -h; i <= h; i++) {
    const int idx = (i + h) * Nu;
    for (int j = 0; j < Nu; j++)
      for (int s = 0; s < 4; ++s) {
        const double x = pd[s][2 * j] + (i * t.t_vec[0]), y = pd[s][2 * j + 1] + (i * t.t_vec[1]);
        rel[(size_t)s * npos + idx + j] = make_double2(x, y);
        pot[(size_t)s * npos + idx + j] = k.upp / std::sqrt(coeff * (std::pow(x, 2) + std::pow(y, 2)) + 1);
      }
  }
  t.iq0 = -(t.nk - 1);
  t.nq = 2 * t.nk - 1;
  t.mq0 = -(t.n_mu - 1);
  t.nmq = 2 * t.n_mu - 1;
  const int nb = t.nq * t.nmq;
  DBuf<double2> d_rel, d_vq, d_wf;
  DBuf<double> d_pot, d_pi, d_en, d_eps;
  XCK(h2d(d_rel, rel.data(), rel.size(), st));
  XCK(h2d(d_pot, pot.data(), pot.size(), st));
  XCK(d_vq.alloc((size_t)nb * 4));
  k_vq<<<nb, kVqThreads, 0, st>>>(d_rel.p, d_pot.p, npos, t.iq0, t.mq0, t.nmq, t.dk_l[0], t.dk_l[1], t.K1[0], t.K1[1],
                                  1.0 / double(2 * Nu * ncell), d_vq.p);
  XCK(cudaGetLastError());
  // PI (cnt.cpp:634-720)
  phase.next("cnt: polarisation");
  XCK(h2d(d_en, t.energy.data(), t.energy.size(), st));
  XCK(h2d(d_wf, reinterpret_cast<const double2*>(t.wf.data()), t.wf.size(), st));
  XCK(d_pi.alloc(nb));
  k_pi<<<nb, kPiThreads, 0, st>>>(d_en.p, d_wf.p, t.nk, t.n_mu, t.iq0, t.mq0, t.nmq, t.cells * t.M, d_pi.p);
  XCK(cudaGetLastError());
  t.vq.resize((size_t)nb * 4);
  t.pi.resize(nb);
  XCK(cudaMemcpyAsync(t.vq.data(), d_vq.p, sizeof(double2) * nb * 4, cudaMemcpyDeviceToHost, st));
  XCK(cudaMemcpyAsync(t.pi.data(), d_pi.p, sizeof(double) * nb, cudaMemcpyDeviceToHost, st));
  XCK(cudaStreamSynchronize(st));
  // eps = 1 + Re(mean over the four sublattice pairs of vq) PI (cnt.cpp:735-757)
  t.eps.resize(nb);
  for (int b = 0; b < nb; ++b) {
    cx mv = cx(0);
    for (int s = 0; s < 4; ++s) mv += t.vq[(size_t)b * 4 + s];
    t.eps[b] = std::real(mv / 4.0) * t.pi[b] + 1.;
  }
  XCK(h2d(d_eps, t.eps.data(), t.eps.size(), st));
  // Bethe-Salpeter kernels (cnt.cpp:818-947)
  phase.next("cnt: Bethe-Salpeter kernels and eigen-solve");
  const int nr = (int)t.relev[0].size();
  if ((int)t.relev[1].size() != nr) {
    err = "valleys with different numbers of relevant states";
    return KMC_ERR_ARG;
  }
  if (nr > KMC_CNT_MAX_RELEVANT) {
    err = "more relevant states per valley than KMC_CNT_MAX_RELEVANT";
    return KMC_ERR_ARG;
  }
  t.nr = nr;
  t.ik_cm0 = -nr;
  t.nk_cm = 2 * nr;
  std::vector<int2> v1(nr), v2(nr);
  for (int i = 0; i < nr; ++i) {
    v1[i] = make_int2(t.relev[0][i][0], t.relev[0][i][1]);
    v2[i] = make_int2(t.relev[1][i][0], t.relev[1][i][1]);
  }
  DBuf<int2> d_v1, d_v2;
  DBuf<double2> d_a11, d_a12, d_ax, d_h, d_vec;
  DBuf<double> d_w;
  DBuf<int32_t> d_sw;
  const size_t msz = (size_t)t.nk_cm * nr * nr;
  XCK(h2d(d_v1, v1.data(), v1.size(), st));
  XCK(h2d(d_v2, v2.data(), v2.size(), st));
  XCK(d_a11.alloc(msz));
  XCK(d_a12.alloc(msz));
  XCK(d_ax.alloc(msz));
  XCK(d_h.alloc(3 * msz));
  XCK(d_vec.alloc(3 * msz));
  XCK(d_w.alloc((size_t)3 * t.nk_cm * nr));
  XCK(d_sw.alloc((size_t)3 * t.nk_cm));
  BseArgs ba{d_en.p, d_wf.p, d_vq.p, d_eps.p, d_v1.p, d_v2.p, t.nk, t.n_mu, t.iq0, t.mq0, t.nmq, nr, t.ik_cm0,
             d_a11.p, d_a12.p, d_ax.p};
  const dim3 gb((unsigned)((nr * nr + 127) / 128), (unsigned)t.nk_cm);
  k_bse_fill<<<gb, 128, 0, st>>>(ba);
  k_bse_combine<<<gb, 128, 0, st>>>(d_a11.p, d_a12.p, d_ax.p, nr, t.nk_cm, d_h.p);
  XCK(cudaGetLastError());
  const size_t smem = 2 * (size_t)nr * nr * sizeof(double2);
  XCK(cudaFuncSetAttribute(k_jacobi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_jacobi<<<3 * t.nk_cm, kJacobiThreads, smem, st>>>(d_h.p, nr, d_w.p, d_vec.p, d_sw.p);
  XCK(cudaGetLastError());
  std::vector<double> wv((size_t)3 * t.nk_cm * nr);
  std::vector<cx> vec(3 * msz);
  std::vector<int32_t> sw(3 * t.nk_cm);
  XCK(cudaMemcpyAsync(wv.data(), d_w.p, sizeof(double) * wv.size(), cudaMemcpyDeviceToHost, st));
  XCK(cudaMemcpyAsync(vec.data(), d_vec.p, sizeof(double2) * vec.size(), cudaMemcpyDeviceToHost, st));
  XCK(cudaMemcpyAsync(sw.data(), d_sw.p, sizeof(int32_t) * sw.size(), cudaMemcpyDeviceToHost, st));
  XCK(cudaStreamSynchronize(st));
  for (int32_t s : sw)
    if (s >= kJacobiSweeps) {
      err = "Jacobi eigen-decomposition did not converge";
      return KMC_ERR_CUDA;
    }
  for (int a = 0; a < 3; ++a)
    t.ex_energy[a].assign(wv.begin() + (size_t)a * t.nk_cm * nr, wv.begin() + (size_t)(a + 1) * t.nk_cm * nr);
  // A2 singlet states over both valleys (cnt.cpp:962-965) and their state indices (:969-997)
  const int nkc = 2 * nr;
  t.psi_s.assign((size_t)t.nk_cm * nkc * nr, cx(0));
  t.ik_idx.assign((size_t)t.nk_cm * 4 * nkc, 0);
  for (int m = 0; m < t.nk_cm; ++m) {
    const int ik_cm = t.ik_cm0 + m;
    for (int r = 0; r < nr; ++r)
      for (int j = 0; j < nr; ++j) {
        const cx pv = vec[2 * msz + ((size_t)m * nr + r) * nr + j];
        t.psi_s[((size_t)m * nkc + r) * nr + j] = (+1 / std::sqrt(2.)) * pv;
        t.psi_s[((size_t)m * nkc + nr + r) * nr + j] = (+1 / std::sqrt(2.)) * pv;
      }
    auto put = [&](int row, int ik_c, int mu_c, int ik_v, int mu_v) {
      t.ik_idx[((size_t)m * 4 + 0) * nkc + row] = ik_c;
      t.ik_idx[((size_t)m * 4 + 1) * nkc + row] = mu_c;
      t.ik_idx[((size_t)m * 4 + 2) * nkc + row] = ik_v;
      t.ik_idx[((size_t)m * 4 + 3) * nkc + row] = mu_v;
    };
    for (int c = 0; c < nr; ++c) {
      const int ik_c = t.relev[0][c][0], mu_c = t.relev[0][c][1];
      int ik_v = ik_c - ik_cm;
      while (ik_v >= t.nk) ik_v -= t.nk;
      while (ik_v < 0) ik_v += t.nk;
      put(c, ik_c, mu_c, ik_v, mu_c);
    }
    for (int v = 0; v < nr; ++v) {
      const int ik_v = t.relev[1][v][0], mu_v = t.relev[1][v][1];
      int ik_c = ik_v + ik_cm;
      while (ik_c >= t.nk) ik_c -= t.nk;
      while (ik_c < 0) ik_c += t.nk;
      put(nkc - 1 - v, ik_c, mu_v, ik_v, mu_v);
    }
  }
  // each A2-singlet state's part of the Q matrix element (exciton_transfer.cpp:276-297)
  t.q_part.assign((size_t)t.nk_cm * nr, cx(0));
  auto W = [&](int mu, int atom, int band, int ik) { return t.wf[(((size_t)mu * 2 + atom) * 2 + band) * t.nk + ik]; };
  for (int m = 0; m < t.nk_cm; ++m) {
    const int ik_cm = t.ik_cm0 + m;
    double kv[2] = {ik_cm * t.dk_l[0], ik_cm * t.dk_l[1]};
    const double dA[2] = {0, 0};
    const cx e0 = std::exp(cx(0., +1.) * dot2(kv, dA)), e1 = std::exp(cx(0., +1.) * dot2(kv, t.acc));
    for (int i_n = 0; i_n < nr; ++i_n) {
      cx qp = 0;
      for (int r = 0; r < nkc; ++r) {
        const int* ix = &t.ik_idx[(size_t)m * 4 * nkc];
        const int ikc = ix[0 * nkc + r], muc = ix[1 * nkc + r], ikv = ix[2 * nkc + r], muv = ix[3 * nkc + r];
        const cx acc = (cx(0) + W(muc, 0, 1, ikc) * std::conj(W(muv, 0, 0, ikv)) * e0) +
                       W(muc, 1, 1, ikc) * std::conj(W(muv, 1, 0, ikv)) * e1;
        qp += t.psi_s[((size_t)m * nkc + r) * nr + i_n] * acc;
      }
      t.q_part[(size_t)m * nr + i_n] = qp;
    }
  }
  return KMC_OK;
}

// thermally relevant A2-singlet states (exciton_transfer.cpp:226-250): (energy, ik_cm, idx, n)
struct ExState {
  double energy;
  int ik_cm, ik_cm_idx, i_n;
};
std::vector<ExState> relevant_states(const kmc_cnt& t, double min_energy, double temperature) {
  const Consts& k = K();
  const double thr = min_energy + std::abs(std::log(1.e-3) * k.kb * temperature);
  std::vector<ExState> out;
  const auto& e = t.ex_energy[2];
  for (int i_n = 0; i_n < t.nr; i_n++)
    for (int m = 0; m < t.nk_cm; m++)
      if (e[(size_t)m * t.nr + i_n] <= thr) out.push_back({e[(size_t)m * t.nr + i_n], t.ik_cm0 + m, m, i_n});
  std::sort(out.begin(), out.end(), [](const ExState& a, const ExState& b) { return a.energy < b.energy; });
  return out;
}

// The matched pairs' weights and the distinct donor / acceptor momenta of a pair of tubes:
// w = (2 pi / hbar) exp(-E_i / kT) / Z |Q|^2 / (L_i L_f) L(E_i - E_f) (exciton_transfer.cpp:380-411)
struct RatePlan {
  std::vector<int> kd, ka;          // distinct ik_cm of donor, acceptor states
  std::vector<int2> pq;             // per matched pair: index into kd, ka
  std::vector<double> w;
};
RatePlan plan_rates(const kmc_cnt& d, const kmc_cnt& a, double temperature, double broadening) {
  const Consts& k = K();
  double min_e = d.ex_energy[2][0];
  for (double x : d.ex_energy[2]) min_e = x < min_e ? x : min_e;
  const auto ds = relevant_states(d, min_e, temperature), as = relevant_states(a, min_e, temperature);
  double Z = 0;
  for (const auto& s : ds) Z += std::exp(-s.energy / (k.kb * temperature));
  auto lor = [&](double e) { return k.inv_pi * broadening / (e * e + broadening * broadening); };
  const double coeff = (std::pow(k.q0, 2) * d.au * a.au) /
                       (16 * std::pow(k.pi, 3) * k.eps0 * d.radius * a.radius * std::sqrt(d.length * a.length));
  RatePlan p;
  auto slot = [](std::vector<int>& v, int x) {
    auto it = std::find(v.begin(), v.end(), x);
    if (it != v.end()) return (int)(it - v.begin());
    v.push_back(x);
    return (int)v.size() - 1;
  };
  for (const auto& s : ds)
    for (const auto& f : as) {
      const double de = s.energy - f.energy;
      if (!(lor(de) > 1.e-2 * lor(0))) continue;
      const cx Q = cx(coeff) * std::conj(d.q_part[(size_t)s.ik_cm_idx * d.nr + s.i_n]) *
                   a.q_part[(size_t)f.ik_cm_idx * a.nr + f.i_n];
      const double q2 = std::norm(Q) / (d.length * a.length);
      p.pq.push_back(make_int2(slot(p.kd, s.ik_cm), slot(p.ka, f.ik_cm)));
      p.w.push_back((2 * k.pi / k.hb) * (std::exp(-s.energy / (k.kb * temperature)) / Z) * q2 * lor(de));
    }
  return p;
}

// centred base positions of make_Ru_3d and the phase factors of make_Ru_2d
// (exciton_transfer.cpp:310-366) for the momenta ks (sign -1: donor, +1: acceptor)
void tube_cells(const kmc_cnt& t, const std::vector<int>& ks, double sign, std::vector<double3>& r,
                std::vector<double2>& ph) {
  const int Nu = t.Nu, n = Nu * t.cells;
  r.resize(n);
  std::vector<double> r2(2 * (size_t)n);
  for (int i = 0; i < t.cells; i++)
    for (int j = 0; j < Nu; j++) {
      const int a = i * Nu + j;
      r[a] = make_double3(t.pos_u_3d[3 * j] + i * t.t3[0], t.pos_u_3d[3 * j + 1] + i * t.t3[1],
                          t.pos_u_3d[3 * j + 2] + i * t.t3[2]);
      r2[2 * a] = t.pos_a[2 * j] + i * t.t_vec[0];
      r2[2 * a + 1] = t.pos_a[2 * j + 1] + i * t.t_vec[1];
    }
  double ymax = r[0].y, ymin = r[0].y;
  for (const auto& v : r) ymax = v.y > ymax ? v.y : ymax, ymin = v.y < ymin ? v.y : ymin;
  for (auto& v : r) v.y -= ((ymax + ymin) / 2.);
  ph.resize(ks.size() * (size_t)n);
  for (size_t p = 0; p < ks.size(); ++p) {
    const double kv[2] = {ks[p] * t.dk_l[0], ks[p] * t.dk_l[1]};
    for (int a = 0; a < n; ++a) {
      const cx e = std::exp(cx(0, sign) * dot2(kv, &r2[2 * (size_t)a]));
      ph[p * n + a] = make_double2(e.real(), e.imag());
    }
  }
}

// the instantiation for nq acceptor momenta (rounded up to 2, 4, 8 or 16; the padding is zero)
template <typename T>
void launch_nq(int nq, dim3 grid, cudaStream_t st, const double3* rd, int nd, const double3* ra, int na,
               const double2* ap, int np, const double2* bq, const JGeom* geo, double2* part) {
  if (nq <= 2)
    k_coulomb_j<T, 2><<<grid, kJThreads, 0, st>>>(rd, nd, ra, na, ap, np, bq, nq, geo, part);
  else if (nq <= 4)
    k_coulomb_j<T, 4><<<grid, kJThreads, 0, st>>>(rd, nd, ra, na, ap, np, bq, nq, geo, part);
  else if (nq <= 8)
    k_coulomb_j<T, 8><<<grid, kJThreads, 0, st>>>(rd, nd, ra, na, ap, np, bq, nq, geo, part);
  else
    k_coulomb_j<T, 16><<<grid, kJThreads, 0, st>>>(rd, nd, ra, na, ap, np, bq, nq, geo, part);
}
void launch_coulomb_j32(int nq, dim3 grid, cudaStream_t st, const float4* rd, int nd, const float4* ra, int na,
                        const double2* ap, int np, const float2* bq, const JGeom* geo, double2* part) {
  if (nq <= 2)
    k_coulomb_j32<2><<<grid, kJThreads, 0, st>>>(rd, nd, ra, na, ap, np, bq, nq, geo, part);
  else if (nq <= 4)
    k_coulomb_j32<4><<<grid, kJThreads, 0, st>>>(rd, nd, ra, na, ap, np, bq, nq, geo, part);
  else if (nq <= 8)
    k_coulomb_j32<8><<<grid, kJThreads, 0, st>>>(rd, nd, ra, na, ap, np, bq, nq, geo, part);
  else
    k_coulomb_j32<16><<<grid, kJThreads, 0, st>>>(rd, nd, ra, na, ap, np, bq, nq, geo, part);
}

// J[g][p][q] for the geometries geo[g] = (z_shift, ash1, ash2, theta)
int coulomb_j(const kmc_cnt& d, const kmc_cnt& a, const std::vector<int>& kd, const std::vector<int>& ka,
              const double* geo, int64_t ng, int32_t precision, cudaStream_t st, std::vector<double2>& J,
              DBuf<double2>* keep_on_device, std::string& err) {
  std::vector<double3> rd, ra;
  std::vector<double2> pd, pa;
  tube_cells(d, kd, -1.0, rd, pd);
  tube_cells(a, ka, +1.0, ra, pa);
  const int np = (int)kd.size(), nq_all = (int)ka.size();
  DBuf<double3> d_rd, d_ra;
  DBuf<double2> d_pd, d_pa, d_J;
  DBuf<JGeom> d_g;
  XCK(h2d(d_rd, rd.data(), rd.size(), st));
  XCK(h2d(d_ra, ra.data(), ra.size(), st));
  XCK(h2d(d_pd, pd.data(), pd.size(), st));
  // the FP32 form's inputs, converted once
  DBuf<float4> d_rd32, d_ra32;
  DBuf<float2> d_pa32;
  std::vector<float2> pa32;
  if (precision != KMC_PREC_FP64) {
    std::vector<float4> r32(rd.size());
    for (size_t k = 0; k < rd.size(); ++k) r32[k] = make_float4((float)rd[k].x, (float)rd[k].y, (float)rd[k].z, 0.f);
    XCK(h2d(d_rd32, r32.data(), r32.size(), st));
    r32.resize(ra.size());
    for (size_t k = 0; k < ra.size(); ++k) r32[k] = make_float4((float)ra[k].x, (float)ra[k].y, (float)ra[k].z, 0.f);
    XCK(h2d(d_ra32, r32.data(), r32.size(), st));
    XCK(cudaStreamSynchronize(st));  // r32 is reused below only after its copies are done
    pa32.resize(pa.size());
    for (size_t k = 0; k < pa.size(); ++k) pa32[k] = make_float2((float)pa[k].x, (float)pa[k].y);
  }
  std::vector<JGeom> g(ng);
  for (int64_t i = 0; i < ng; ++i)
    g[i] = JGeom{geo[4 * i], geo[4 * i + 1], geo[4 * i + 2], std::cos(geo[4 * i + 3]), std::sin(geo[4 * i + 3])};
  XCK(h2d(d_g, g.data(), g.size(), st));
  DBuf<double2>& out = keep_on_device ? *keep_on_device : d_J;
  XCK(out.alloc((size_t)ng * np * nq_all));
  XCK(cudaMemsetAsync(out.p, 0, sizeof(double2) * ng * np * nq_all, st));
  // acceptor momenta in chunks of kJMaxQ; each chunk writes its own columns
  std::vector<double2> Jc;
  for (int q0 = 0; q0 < nq_all; q0 += kJMaxQ) {
    const int nq = std::min(kJMaxQ, nq_all - q0);
    if (precision == KMC_PREC_FP64)
      XCK(h2d(d_pa, pa.data() + (size_t)q0 * ra.size(), (size_t)nq * ra.size(), st));
    else
      XCK(h2d(d_pa32, pa32.data() + (size_t)q0 * ra.size(), (size_t)nq * ra.size(), st));
    DBuf<double2> d_Jc, d_part;
    const int ntile = (int)((rd.size() + kJThreads - 1) / kJThreads);
    XCK(d_Jc.alloc((size_t)ng * np * nq));
    XCK(d_part.alloc((size_t)ng * ntile * np * nq));
    for (int64_t g0 = 0; g0 < ng; g0 += 65535) {
      const int gn = (int)std::min<int64_t>(65535, ng - g0);
      const dim3 grid((unsigned)ntile, (unsigned)gn);
      double2* pp = d_part.p + (size_t)g0 * ntile * np * nq;
      if (precision == KMC_PREC_FP64)
        launch_nq<double>(nq, grid, st, d_rd.p, (int)rd.size(), d_ra.p, (int)ra.size(), d_pd.p, np, d_pa.p,
                          d_g.p + g0, pp);
      else
        launch_coulomb_j32(nq, grid, st, d_rd32.p, (int)rd.size(), d_ra32.p, (int)ra.size(), d_pd.p, np, d_pa32.p,
                           d_g.p + g0, pp);
      XCK(cudaGetLastError());
    }
    const int64_t nj = (int64_t)ng * np * nq;
    k_j_reduce<<<(unsigned)((nj + 255) / 256), 256, 0, st>>>(d_part.p, ntile, np * nq, nj, d_Jc.p);
    XCK(cudaGetLastError());
    // scatter the chunk's columns into [g][p][q] (a strided device copy)
    XCK(cudaMemcpy2DAsync(out.p + q0, sizeof(double2) * nq_all, d_Jc.p, sizeof(double2) * nq, sizeof(double2) * nq,
                          (size_t)ng * np, cudaMemcpyDeviceToDevice, st));
    XCK(cudaStreamSynchronize(st));
  }
  if (!keep_on_device) {
    J.resize((size_t)ng * np * nq_all);
    XCK(cudaMemcpyAsync(J.data(), out.p, sizeof(double2) * J.size(), cudaMemcpyDeviceToHost, st));
    XCK(cudaStreamSynchronize(st));
  }
  return KMC_OK;
}

int rates(const kmc_cnt& d, const kmc_cnt& a, const kmc_transfer_cfg& cfg, int64_t ng, const double* geo,
          double* out, cudaStream_t st, std::string& err) {
  const RatePlan p = plan_rates(d, a, cfg.temperature, cfg.broadening);
  if (p.pq.empty()) {
    for (int64_t g = 0; g < ng; ++g) out[g] = 0;
    return KMC_OK;
  }
  const int64_t chunk = 1 << 15;  // partials: chunk x donor tiles x pairs of momenta x 16 B
  for (int64_t g0 = 0; g0 < ng; g0 += chunk) {
    const int64_t gn = std::min(chunk, ng - g0);
    DBuf<double2> d_J;
    std::vector<double2> unused;
    int rc = coulomb_j(d, a, p.kd, p.ka, geo + 4 * g0, gn, cfg.precision, st, unused, &d_J, err);
    if (rc) return rc;
    DBuf<int2> d_pq;
    DBuf<double> d_w, d_r;
    XCK(h2d(d_pq, p.pq.data(), p.pq.size(), st));
    XCK(h2d(d_w, p.w.data(), p.w.size(), st));
    XCK(d_r.alloc(gn));
    k_rates<<<(unsigned)((gn + 255) / 256), 256, 0, st>>>(d_J.p, (int)p.kd.size(), (int)p.ka.size(), (int)gn,
                                                          d_pq.p, d_w.p, (int)p.pq.size(), d_r.p);
    XCK(cudaGetLastError());
    XCK(cudaMemcpyAsync(out + g0, d_r.p, sizeof(double) * gn, cudaMemcpyDeviceToHost, st));
    XCK(cudaStreamSynchronize(st));
  }
  return KMC_OK;
}

int fail(kmc_ctx* c, int code, const std::string& msg) {
  if (c) ctx_set_error(c, msg.c_str());
  return code;
}

bool cfg_ok(const kmc_transfer_cfg* cfg) {
  return cfg && cfg->temperature > 0 && cfg->broadening > 0 &&
         (cfg->precision == KMC_PREC_FP64 || cfg->precision == KMC_PREC_MIXED);
}

}  // namespace

extern "C" {

int kmc_cnt_create(kmc_ctx* ctx, int32_t n, int32_t m, int32_t length_cells, kmc_cnt** out) try {
  if (!ctx || !out) return KMC_ERR_ARG;
  *out = nullptr;
  if (n < 1 || m < 1 || m > n || length_cells < 1 || length_cells > 4096)
    return fail(ctx, KMC_ERR_ARG, "kmc_cnt_create: need chirality n >= m >= 1 and 1..4096 unit cells");
  if (cudaSetDevice(ctx_device(ctx)) != cudaSuccess) return fail(ctx, KMC_ERR_CUDA, "kmc_cnt_create: cudaSetDevice");
  kmc::NvtxRange nv("kmc_cnt_create");
  kmc_cnt* t = new kmc_cnt();
  t->n = n;
  t->m = m;
  t->cells = length_cells;
  std::string err;
  int rc = KMC_OK;
  if (!geometry(*t, err)) {
    rc = KMC_ERR_ARG;
  } else {
    bands(*t);
    if (!valleys(*t, err)) {
      rc = KMC_ERR_ARG;
    } else {
      relevant_window(*t, 1. * K().eV);  // calculate_exciton_dispersion: 1 eV window (cnt.cpp:1068)
      rc = screening_and_excitons(*t, ctx_stream(ctx), err);
    }
  }
  if (rc != KMC_OK) {
    delete t;
    return fail(ctx, rc, "kmc_cnt_create: " + err);
  }
  *out = t;
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(ctx, "kmc_cnt_create");
}

void kmc_cnt_destroy(kmc_cnt* t) { delete t; }

int kmc_cnt_get_info(const kmc_cnt* t, kmc_cnt_info* info) try {
  if (!t || !info) return KMC_ERR_ARG;
  kmc_cnt_info& o = *info;
  o.n = t->n, o.m = t->m, o.cells = t->cells, o.Nu = t->Nu, o.M = t->M, o.Q = t->Q, o.t1 = t->t1, o.t2 = t->t2;
  o.nk = t->nk, o.n_mu = t->n_mu, o.n_valley_pairs = (int32_t)t->valleys.size(), o.n_relevant = t->nr;
  o.iq0 = t->iq0, o.nq = t->nq, o.mq0 = t->mq0, o.nmq = t->nmq, o.ik_cm0 = t->ik_cm0, o.nk_cm = t->nk_cm;
  o.radius = t->radius, o.length = t->length, o.area_u = t->au;
  return KMC_OK;
} catch (...) {
  const char* what = nullptr;
  return kmc::abi_status(&what);
}

int kmc_cnt_get_array(const kmc_cnt* t, int32_t which, void* out, int64_t count) try {
  if (!t || !out || count < 0) return KMC_ERR_ARG;
  std::vector<double> dv;
  std::vector<int32_t> iv;
  auto cxs = [&](const std::vector<cx>& v) {
    for (const cx& z : v) dv.push_back(z.real()), dv.push_back(z.imag());
  };
  switch (which) {
    case KMC_CNT_GEOMETRY:
      for (const double* v : {t->a1, t->a2, t->b1, t->b2, t->acc, t->ch, t->t_vec, t->K1, t->K2, t->dk_l})
        dv.insert(dv.end(), v, v + 2);
      dv.insert(dv.end(), t->t3, t->t3 + 3);
      dv.insert(dv.end(), {t->radius, t->ch_len, t->length});
      break;
    case KMC_CNT_POS_U_3D: dv = t->pos_u_3d; break;
    case KMC_CNT_BANDS: dv = t->energy; break;
    case KMC_CNT_VALLEYS:
      for (const auto& v : t->valleys) iv.insert(iv.end(), v.begin(), v.end());
      break;
    case KMC_CNT_RELEVANT:
      for (int v = 0; v < 2; ++v)
        for (const auto& s : t->relev[v]) iv.insert(iv.end(), s.begin(), s.end());
      break;
    case KMC_CNT_VQ: cxs(t->vq); break;
    case KMC_CNT_PI: dv = t->pi; break;
    case KMC_CNT_EPS: dv = t->eps; break;
    case KMC_CNT_A1: dv = t->ex_energy[0]; break;
    case KMC_CNT_A2_TRIPLET: dv = t->ex_energy[1]; break;
    case KMC_CNT_A2_SINGLET: dv = t->ex_energy[2]; break;
    case KMC_CNT_IK_IDX: iv.assign(t->ik_idx.begin(), t->ik_idx.end()); break;
    case KMC_CNT_Q_PARTIAL: cxs(t->q_part); break;
    default: return KMC_ERR_ARG;
  }
  const int64_t have = dv.empty() ? (int64_t)iv.size() : (int64_t)dv.size();
  if (count != have) return KMC_ERR_ARG;
  if (!dv.empty()) std::memcpy(out, dv.data(), dv.size() * sizeof(double));
  else if (!iv.empty()) std::memcpy(out, iv.data(), iv.size() * sizeof(int32_t));
  return KMC_OK;
} catch (...) {
  const char* what = nullptr;
  return kmc::abi_status(&what);
}

int kmc_exciton_j(kmc_ctx* ctx, const kmc_cnt* donor, const kmc_cnt* acceptor, int64_t n_pairs,
                  const int32_t* ik_cm_pairs, const double geometry[4], int32_t precision, double* j_out) try {
  if (!ctx || !donor || !acceptor || n_pairs < 0 || (n_pairs > 0 && (!ik_cm_pairs || !geometry || !j_out)) ||
      (precision != KMC_PREC_FP64 && precision != KMC_PREC_MIXED))
    return fail(ctx, KMC_ERR_ARG, "kmc_exciton_j: bad arguments");
  if (n_pairs == 0) return KMC_OK;
  if (cudaSetDevice(ctx_device(ctx)) != cudaSuccess) return fail(ctx, KMC_ERR_CUDA, "kmc_exciton_j: cudaSetDevice");
  kmc::NvtxRange nv("kmc_exciton_j");
  std::vector<int> kd, ka;
  std::vector<int2> pq(n_pairs);
  auto slot = [](std::vector<int>& v, int x) {
    auto it = std::find(v.begin(), v.end(), x);
    if (it != v.end()) return (int)(it - v.begin());
    v.push_back(x);
    return (int)v.size() - 1;
  };
  for (int64_t i = 0; i < n_pairs; ++i) pq[i] = make_int2(slot(kd, ik_cm_pairs[2 * i]), slot(ka, ik_cm_pairs[2 * i + 1]));
  std::vector<double2> J;
  std::string err;
  int rc = coulomb_j(*donor, *acceptor, kd, ka, geometry, 1, precision, ctx_stream(ctx), J, nullptr, err);
  if (rc) return fail(ctx, rc, "kmc_exciton_j: " + err);
  for (int64_t i = 0; i < n_pairs; ++i) {
    const double2 v = J[(size_t)pq[i].x * ka.size() + pq[i].y];
    j_out[2 * i] = v.x;
    j_out[2 * i + 1] = v.y;
  }
  return KMC_OK;
} catch (...) {
  return kmc::abi_fail(ctx, "kmc_exciton_j");
}

int kmc_exciton_rates(kmc_ctx* ctx, const kmc_cnt* donor, const kmc_cnt* acceptor, const kmc_transfer_cfg* cfg,
                      int64_t n_geometries, const double* geometries, double* rate) try {
  if (!ctx || !donor || !acceptor || !cfg_ok(cfg) || n_geometries < 0 || (n_geometries > 0 && (!geometries || !rate)))
    return fail(ctx, KMC_ERR_ARG, "kmc_exciton_rates: bad arguments");
  if (cudaSetDevice(ctx_device(ctx)) != cudaSuccess) return fail(ctx, KMC_ERR_CUDA, "kmc_exciton_rates: cudaSetDevice");
  kmc::NvtxRange nv("kmc_exciton_rates");
  std::string err;
  int rc = rates(*donor, *acceptor, *cfg, n_geometries, geometries, rate, ctx_stream(ctx), err);
  return rc ? fail(ctx, rc, "kmc_exciton_rates: " + err) : KMC_OK;
} catch (...) {
  return kmc::abi_fail(ctx, "kmc_exciton_rates");
}

int kmc_davoody_table(kmc_ctx* ctx, const kmc_cnt* donor, const kmc_cnt* acceptor, const kmc_transfer_cfg* cfg,
                      const double theta_deg[3], const double zshift[3], const double ash1[3], const double ash2[3],
                      double* theta, double* zsh, double* a1, double* a2, double* rate) try {
  if (!ctx || !donor || !acceptor || !cfg_ok(cfg) || !theta_deg || !zshift || !ash1 || !ash2 || !theta || !zsh ||
      !a1 || !a2 || !rate)
    return fail(ctx, KMC_ERR_ARG, "kmc_davoody_table: bad arguments");
  // point counts: numbers in [1, 2^31 - 1], checked before they are converted; the table at most
  // 2^34 entries (its geometries are a host array of four doubles each)
  auto count = [](double x, int64_t& n) {
    if (!(x >= 1.0 && x <= 2147483647.0)) return false;
    n = (int64_t)x;
    return true;
  };
  int64_t nt = 0, nz = 0, n1 = 0, n2 = 0;
  if (!count(theta_deg[2], nt) || !count(zshift[2], nz) || !count(ash1[2], n1) || !count(ash2[2], n2))
    return fail(ctx, KMC_ERR_ARG, "kmc_davoody_table: a grid's point count is not in [1, 2^31 - 1]");
  const double entries = (double)nt * (double)nz * (double)n1 * (double)n2;
  if (entries > 17179869184.0) return fail(ctx, KMC_ERR_ARG, "kmc_davoody_table: table too large");
  // monte_carlo.cpp:65-75: linspace grids, theta scaled by the reference's pi / 180
  linspace(zshift[0], zshift[1], nz, zsh);
  linspace(ash1[0], ash1[1], n1, a1);
  linspace(ash2[0], ash2[1], n2, a2);
  linspace(theta_deg[0], theta_deg[1], nt, theta);
  const double scale = K().pi / 180;
  for (int64_t i = 0; i < nt; ++i) theta[i] = theta[i] * scale;
  std::vector<double> geo((size_t)4 * nt * nz * n1 * n2);
  size_t g = 0;
  for (int64_t it = 0; it < nt; ++it)
    for (int64_t iz = 0; iz < nz; ++iz)
      for (int64_t i1 = 0; i1 < n1; ++i1)
        for (int64_t i2 = 0; i2 < n2; ++i2, ++g) {
          geo[4 * g] = zsh[iz];
          geo[4 * g + 1] = a1[i1];
          geo[4 * g + 2] = a2[i2];
          geo[4 * g + 3] = theta[it];
        }
  return kmc_exciton_rates(ctx, donor, acceptor, cfg, (int64_t)g, geo.data(), rate);
} catch (...) {
  return kmc::abi_fail(ctx, "kmc_davoody_table");
}

}  // extern "C"
