// ref_driver.cpp -- TEST INFRASTRUCTURE: drives the reference's own Green-Kubo engine
// (mc::monte_carlo of src/monte_carlo/, compiled unchanged against oracle/shim) the way
// src/main.cpp:62-76 does, and dumps everything the oracle is checked against.
//
// Parity build (default):
//   * rand() is defined here and serves per-exciton Philox-4x32-10 streams (oracle/kmc_math.h):
//     during kubo_create_particles the draws of exciton i are, in order, the injection dice
//     (monte_carlo.cpp:311), the dwell-time draws (scatterer.h:76, repeated while 0) and the
//     heading (particle.h:51); during kubo_step, particle::step is wrapped (ld --wrap) so the
//     exciton being stepped owns the stream, which also serves its reinjection dice
//     (monte_carlo.cpp:331).  The run must be single threaded (OMP_NUM_THREADS=1).
//   * log() and acos() are defined here as the oracle's orc_log / orc_acos.
// Timing build (-DKMC_REF_TIMING): glibc rand/log/acos and OpenMP as shipped; only the hop
// counter wrapper around scatterer::update_state is added.
//
// usage: ref_kubo input.json out.bin n_steps seed n_trace trace_cap dump_csr
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <string>
#include <vector>
#include <list>
#include <sstream>
#include <thread>
#include <algorithm>
#include <cassert>
#include <cmath>
#include <iomanip>
#include <omp.h>
#include <experimental/filesystem>
#include <regex>
#include <tuple>
#include <exception>
#include <stdexcept>
#include <memory>
#include <array>
#include <limits>
#include <ctime>

#include <armadillo>
#include "json.hpp"

#include "kmc_math.h"

#define private public
#include "monte_carlo/monte_carlo.h"
#undef private

#define STEP_SYM _ZN2mc8particle4stepEdRKSt6vectorINS_9scattererESaIS2_EERKd
#define UPD_SYM _ZNK2mc9scatterer12update_stateERKd
#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)

namespace {
std::atomic<long long> g_hops{0};
#ifndef KMC_REF_TIMING
int g_mode = 0;  // 1: creating excitons, 2: stepping
std::vector<orc_rng> g_streams;
long long g_cur = 0;
int g_cstate = 0;
const mc::particle* g_pbase = nullptr;
const mc::scatterer* g_sbase = nullptr;
std::vector<std::vector<int32_t>> g_trace;
long long g_trace_cap = 0;
#endif
}  // namespace

extern "C" {
const mc::scatterer* CAT(__real_, UPD_SYM)(const mc::scatterer* self, const double& r);
const mc::scatterer* CAT(__wrap_, UPD_SYM)(const mc::scatterer* self, const double& r) {
  const mc::scatterer* out = CAT(__real_, UPD_SYM)(self, r);
  g_hops.fetch_add(1, std::memory_order_relaxed);
#ifndef KMC_REF_TIMING
  if (g_cur < (long long)g_trace.size()) {
    auto& t = g_trace[g_cur];
    t.push_back((int32_t)(out - g_sbase));
    if ((long long)t.size() > g_trace_cap) t.pop_back();
  }
#endif
  return out;
}

#ifndef KMC_REF_TIMING
void CAT(__real_, STEP_SYM)(mc::particle* self, double dt, const std::vector<mc::scatterer>& l, const double& r);
void CAT(__wrap_, STEP_SYM)(mc::particle* self, double dt, const std::vector<mc::scatterer>& l, const double& r) {
  g_cur = self - g_pbase;
  CAT(__real_, STEP_SYM)(self, dt, l, r);
}

int rand(void) __THROW {
  if (g_mode == 1) {
    int v = orc_rand(&g_streams[g_cur]);
    if (g_cstate == 0) {
      g_cstate = 1;  // injection dice taken; next: dwell time
    } else if (g_cstate == 1) {
      if (v != 0) g_cstate = 2;  // dwell time accepted; next: heading
    } else {
      g_cstate = 0;  // heading taken; the next draw belongs to the next exciton
      ++g_cur;
    }
    return v;
  }
  if (g_mode == 2) return orc_rand(&g_streams[g_cur]);
  std::fprintf(stderr, "ref_driver: rand() outside exciton creation/stepping\n");
  std::abort();
}
double log(double x) __THROW { return orc_log(x); }
double acos(double x) __THROW { return orc_acos(x); }
#endif
}

namespace {
struct Dump {
  std::ofstream f;
  explicit Dump(const char* path) : f(path, std::ios::binary) { f.write("KMCREF1\n", 8); }
  template <typename T>
  void put(const char* name, const char* dt, const T* p, long long n) {
    char nm[32] = {0};
    std::strncpy(nm, name, 31);
    char d[8] = {0};
    std::strncpy(d, dt, 7);
    f.write(nm, 32);
    f.write(d, 8);
    f.write(reinterpret_cast<const char*>(&n), 8);
    f.write(reinterpret_cast<const char*>(p), sizeof(T) * n);
  }
};
}  // namespace

int main(int argc, char** argv) {
  if (argc < 8) {
    std::fprintf(stderr, "usage: %s input.json out.bin n_steps seed n_trace trace_cap dump_csr\n", argv[0]);
    return 2;
  }
  std::ifstream in(argv[1]);
  nlohmann::json j;
  in >> j;
  nlohmann::json json_mc = j["exciton monte carlo"];
  long long n_steps = std::atoll(argv[3]);
  unsigned long long seed = std::strtoull(argv[4], nullptr, 10);
  long long n_trace = std::atoll(argv[5]);
  long long trace_cap = std::atoll(argv[6]);
  int dump_csr = std::atoi(argv[7]);
  double time_step = json_mc["monte carlo time step"];

  std::streambuf* cout_buf = std::cout.rdbuf();
  std::ostringstream sink;
  std::cout.rdbuf(sink.rdbuf());  // the reference prints progress; keep stdout for results

  mc::monte_carlo sim(json_mc);
  sim._time = 0;  // monte_carlo.h:45 leaves it uninitialised
  sim.kubo_init();
  const long long n = (long long)sim._all_scat_list.size();
  Dump d(argv[2]);
  {
    std::vector<double> pos(3 * n), ori(3 * n), tot(n), inv(n);
    std::vector<int32_t> L(n), R(n);
    for (long long i = 0; i < n; ++i) {
      const auto& s = sim._all_scat_list[i];
      for (int c = 0; c < 3; ++c) {
        pos[3 * i + c] = s.pos(c);
        ori[3 * i + c] = s.orientation(c);
      }
      L[i] = s.left;
      R[i] = s.right;
      tot[i] = s._max_rate;
      inv[i] = s._inverse_max_rate;
    }
    d.put("pos", "f8", pos.data(), 3 * n);
    d.put("orient", "f8", ori.data(), 3 * n);
    d.put("left", "i4", L.data(), n);
    d.put("right", "i4", R.data(), n);
    d.put("total", "f8", tot.data(), n);
    d.put("inv_total", "f8", inv.data(), n);
    double dom[6] = {sim._domain.first(0), sim._domain.first(1), sim._domain.first(2),
                     sim._domain.second(0), sim._domain.second(1), sim._domain.second(2)};
    d.put("domain", "f8", dom, 6);
    const auto& t = sim._scat_table;
    d.put("table_theta", "f8", t.theta.memptr(), (long long)t.theta.n_elem);
    d.put("table_zsh", "f8", t.z_shift.memptr(), (long long)t.z_shift.n_elem);
    d.put("table_ash1", "f8", t.axis_shift_1.memptr(), (long long)t.axis_shift_1.n_elem);
    d.put("table_ash2", "f8", t.axis_shift_2.memptr(), (long long)t.axis_shift_2.n_elem);
    std::vector<double> rate;
    for (arma::uword a = 0; a < t.theta.n_elem; ++a)
      for (arma::uword b = 0; b < t.z_shift.n_elem; ++b)
        for (arma::uword c = 0; c < t.axis_shift_1.n_elem; ++c)
          for (arma::uword e = 0; e < t.axis_shift_2.n_elem; ++e) rate.push_back(t.rate(a)(b, c, e));
    d.put("table_rate", "f8", rate.data(), (long long)rate.size());
    std::vector<int32_t> inj;
    for (auto* s : sim._inject_scats) inj.push_back((int32_t)(s - sim._all_scat_list.data()));
    d.put("inject", "i4", inj.data(), (long long)inj.size());
    double rem[6] = {sim._removal_domain.first(0), sim._removal_domain.first(1), sim._removal_domain.first(2),
                     sim._removal_domain.second(0), sim._removal_domain.second(1), sim._removal_domain.second(2)};
    d.put("removal", "f8", rem, 6);
    if (dump_csr) {
      std::vector<long long> rp(1, 0);
      std::vector<int32_t> col;
      std::vector<double> cum;
      for (long long i = 0; i < n; ++i) {
        auto nl = sim._all_scat_list[i].find_neighbors(sim._max_hopping_radius);
        for (auto& p : nl) {
          cum.push_back(p.first);
          col.push_back((int32_t)(p.second - sim._all_scat_list.data()));
        }
        rp.push_back((long long)col.size());
      }
      d.put("csr_rowptr", "i8", rp.data(), (long long)rp.size());
      d.put("csr_col", "i4", col.data(), (long long)col.size());
      d.put("csr_cum", "f8", cum.data(), (long long)cum.size());
    }
  }

  const long long n_exc = json_mc["number of particles for kubo simulation"];
#ifndef KMC_REF_TIMING
  g_streams.resize(n_exc);
  for (long long e = 0; e < n_exc; ++e) orc_rng_init(&g_streams[e], seed, (uint64_t)e, 0);
  g_sbase = sim._all_scat_list.data();
  g_trace.assign(std::min(n_trace, n_exc), {});
  g_trace_cap = trace_cap;
  g_mode = 1;
  g_cur = 0;
  g_cstate = 0;
#else
  (void)seed;
  (void)n_trace;
  (void)trace_cap;
#endif
  sim.kubo_create_particles();
#ifndef KMC_REF_TIMING
  g_pbase = sim._particle_list.data();
  g_mode = 2;
  g_cur = 1LL << 62;
#endif
  auto dump_state = [&](const char* suffix) {
    std::vector<int32_t> site(n_exc), head(n_exc);
    std::vector<double> pos(3 * n_exc), old(3 * n_exc), del(3 * n_exc), ff(n_exc);
    std::vector<unsigned long long> draws(n_exc, 0);
    for (long long e = 0; e < n_exc; ++e) {
      const auto& p = sim._particle_list[e];
      site[e] = (int32_t)(p._scat_ptr - sim._all_scat_list.data());
      head[e] = p._heading_right ? 1 : 0;
      ff[e] = p._ff_time;
      for (int c = 0; c < 3; ++c) {
        pos[3 * e + c] = p._pos(c);
        old[3 * e + c] = p._old_pos(c);
        del[3 * e + c] = p._delta_pos(c);
      }
#ifndef KMC_REF_TIMING
      draws[e] = g_streams[e].n;
#endif
    }
    std::string s(suffix);
    d.put(("site" + s).c_str(), "i4", site.data(), n_exc);
    d.put(("heading" + s).c_str(), "i4", head.data(), n_exc);
    d.put(("ff" + s).c_str(), "f8", ff.data(), n_exc);
    d.put(("xpos" + s).c_str(), "f8", pos.data(), 3 * n_exc);
    d.put(("xold" + s).c_str(), "f8", old.data(), 3 * n_exc);
    d.put(("delta" + s).c_str(), "f8", del.data(), 3 * n_exc);
    d.put(("draws" + s).c_str(), "u8", draws.data(), n_exc);
  };
  dump_state("_init");

  std::vector<double> msd, times;
  auto t0 = std::chrono::steady_clock::now();
  long long steps_done = 0;
  // main.cpp:70-76 runs until sim.time() reaches kubo_max_time(); n_steps < 0 keeps that rule
  while (n_steps < 0 ? sim.time() < sim.kubo_max_time() : steps_done < n_steps) {
    sim.kubo_step(time_step);
    double sx = 0, sy = 0, sz = 0;  // the sums of kubo_save_avg_dispalcement_squared, monte_carlo.cpp:398-402
    for (const auto& p : sim._particle_list) {
      sx += std::pow(p.delta_pos(0), 2);
      sy += std::pow(p.delta_pos(1), 2);
      sz += std::pow(p.delta_pos(2), 2);
    }
    msd.push_back(sx);
    msd.push_back(sy);
    msd.push_back(sz);
    times.push_back(sim.time());
    ++steps_done;
  }
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  d.put("msd", "f8", msd.data(), (long long)msd.size());
  d.put("time", "f8", times.data(), (long long)times.size());
  dump_state("");
#ifndef KMC_REF_TIMING
  std::vector<long long> tl;
  std::vector<int32_t> tr;
  for (auto& t : g_trace) {
    tl.push_back((long long)t.size());
    tr.insert(tr.end(), t.begin(), t.end());
  }
  d.put("trace_len", "i8", tl.data(), (long long)tl.size());
  d.put("trace", "i4", tr.data(), (long long)tr.size());
#endif
  long long hops = g_hops.load();
  d.put("hops", "i8", &hops, 1);
  d.put("seconds", "f8", &secs, 1);
  d.f.close();
  std::cout.rdbuf(cout_buf);
  std::printf("{\"hops\": %lld, \"seconds\": %.6f, \"threads\": %d, \"steps\": %lld, \"sites\": %lld}\n", hops, secs,
              omp_get_max_threads(), steps_done, n);
  return 0;
}
