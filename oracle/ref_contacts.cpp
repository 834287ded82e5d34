// ref_contacts.cpp -- TEST INFRASTRUCTURE: drives the reference's contacts (steady-state flux)
// mode -- mc::monte_carlo::init, step, save_metrics and repopulate (src/monte_carlo/monte_carlo.h,
// compiled unchanged against oracle/shim) -- the way src/main.cpp:85-106 does, and dumps what the
// oracle's contacts mode is checked against.
//
// Exciton slots (the engine's layout) are mapped onto the reference's particle vector:
//   * rand() is defined here.  While excitons are created (create_particles inside init,
//     monte_carlo.h:274-316, and repopulate :458-491) every creation takes a slot -- the lowest
//     slot emptied so far, else the next never-used one -- and its three kinds of draw (site dice,
//     dwell time repeated while 0 (scatterer.h:76), heading (particle.h:51)) come from that slot's
//     Philox stream, which keeps its counter across the slot's excitons.
//   * the slot of each particle is stamped into its _delta_pos(0) (as slot + 1): contacts mode
//     never reads or updates _delta_pos (update_delta_pos is only called by kubo_step), and the
//     stamp travels with the particle through repopulate's swaps.  particle::step is wrapped
//     (ld --wrap) so that the particle being stepped draws from its slot's stream.
//   * log() and acos() are the oracle's orc_log / orc_acos.
// repopulate_contacts (monte_carlo.h:443-455) is called here as its two repopulate calls, so
// that the new particles of contact 1 are stamped before contact 2 moves them; the slab bounds
// are computed with the same expressions.  Run single threaded (OMP_NUM_THREADS=1).
//
// track_particle (monte_carlo.h:786-818), called n_tracks times before the loop as main.cpp:90-92
// does, draws from stream 2^32 + k for track k; its positions are taken from the wrapped
// particle::step.
//
// usage: ref_contacts input.json out.bin n_steps seed [n_tracks]
#include <algorithm>
#include <array>
#include <cassert>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <exception>
#include <experimental/filesystem>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <list>
#include <map>
#include <memory>
#include <omp.h>
#include <regex>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

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
unsigned long long g_seed = 0;
int g_mode = 0;  // 1: creating particles, 2: stepping, 3: track_particle
orc_rng g_track;                  // stream of the current track_particle call
std::vector<double> g_track_path; // its positions after every step
const long long kTrackStepCap = 5000000;
std::vector<orc_rng> g_streams;  // one per slot
std::vector<long long> g_hops;   // per slot
std::set<long long> g_free;      // emptied slots below the high-water mark
long long g_hwm = 0;
std::vector<long long> g_created;  // slots of the particles created by the current call, in order
long long g_cur = -1;
int g_cstate = 0;

[[noreturn]] void die(const char* m) {
  std::fprintf(stderr, "ref_contacts: %s\n", m);
  std::abort();
}

orc_rng& stream_of(long long slot) {
  while ((long long)g_streams.size() <= slot) {
    g_streams.emplace_back();
    orc_rng_init(&g_streams.back(), g_seed, (uint64_t)(g_streams.size() - 1), 0);
    g_hops.push_back(0);
  }
  return g_streams[slot];
}

long long slot_of(const mc::particle& p) {
  double v = p._delta_pos(0);
  if (!(v >= 1.0) || v != std::floor(v)) die("particle without a slot stamp");
  return (long long)v - 1;
}
}  // namespace

extern "C" {
const mc::scatterer* CAT(__real_, UPD_SYM)(const mc::scatterer* self, const double& r);
const mc::scatterer* CAT(__wrap_, UPD_SYM)(const mc::scatterer* self, const double& r) {
  if (g_mode == 2 && g_cur >= 0) g_hops[g_cur]++;  // hops of the slots' excitons (not of tracks)
  return CAT(__real_, UPD_SYM)(self, r);
}

void CAT(__real_, STEP_SYM)(mc::particle* self, double dt, const std::vector<mc::scatterer>& l, const double& r);
void CAT(__wrap_, STEP_SYM)(mc::particle* self, double dt, const std::vector<mc::scatterer>& l, const double& r) {
  if (g_mode == 3) {  // the particle of track_particle (not in the list, no slot)
    CAT(__real_, STEP_SYM)(self, dt, l, r);
    for (int c = 0; c < 3; ++c) g_track_path.push_back(self->_pos(c));
    if ((long long)g_track_path.size() > 3 * kTrackStepCap) die("a tracked particle did not reach the last slab");
    return;
  }
  g_cur = slot_of(*self);
  CAT(__real_, STEP_SYM)(self, dt, l, r);
  g_cur = -1;
}

int rand(void) __THROW {
  if (g_mode == 1) {
    if (g_cstate == 0) {  // a new particle: take its slot
      if (!g_free.empty()) {
        g_cur = *g_free.begin();
        g_free.erase(g_free.begin());
      } else {
        g_cur = g_hwm++;
      }
      g_created.push_back(g_cur);
    }
    int v = orc_rand(&stream_of(g_cur));
    if (g_cstate == 0) {
      g_cstate = 1;  // site dice taken; next: dwell time
    } else if (g_cstate == 1) {
      if (v != 0) g_cstate = 2;  // dwell time accepted; next: heading
    } else {
      g_cstate = 0;  // heading taken
    }
    return v;
  }
  if (g_mode == 3) return orc_rand(&g_track);
  if (g_mode == 2) {
    if (g_cur < 0) die("rand() outside a particle step");
    return orc_rand(&stream_of(g_cur));
  }
  die("rand() outside particle creation/stepping");
}
double log(double x) __THROW { return orc_log(x); }
double acos(double x) __THROW { return orc_acos(x); }
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

// stamp the particles created since the last call: they sit at the end of the list in creation
// order (repopulate :476-490 overwrites from the kept count on, then appends)
void stamp_new(std::vector<mc::particle>& list) {
  const size_t n = g_created.size();
  if (n > list.size()) die("more creations than particles");
  for (size_t t = 0; t < n; ++t) {
    auto& p = list[list.size() - n + t];
    if (p._delta_pos(0) != 0.0) die("a created particle already carries a stamp");
    p._delta_pos(0) = (double)(g_created[t] + 1);
  }
  g_created.clear();
  if (g_cstate != 0) die("creation draws out of step");
}
}  // namespace

int main(int argc, char** argv) {
  if (argc < 5) {
    std::fprintf(stderr, "usage: %s input.json out.bin n_steps seed [n_tracks]\n", argv[0]);
    return 2;
  }
  std::ifstream in(argv[1]);
  nlohmann::json j;
  in >> j;
  nlohmann::json json_mc = j["exciton monte carlo"];
  const long long n_steps = std::atoll(argv[3]);
  g_seed = std::strtoull(argv[4], nullptr, 10);
  const double time_step = json_mc["monte carlo time step"];

  std::streambuf* cout_buf = std::cout.rdbuf();
  std::ostringstream sink;
  std::cout.rdbuf(sink.rdbuf());

  mc::monte_carlo sim(json_mc);
  sim._time = 0;  // monte_carlo.h:45 leaves it uninitialised
  g_mode = 1;
  sim.init();  // builds the film, writes scatterer_statistics.dat, creates the particles
  stamp_new(sim._particle_list);
  g_mode = 0;

  const long long n = (long long)sim._all_scat_list.size();
  const unsigned n_seg = sim._n_seg;
  const double ymin = sim._domain.first(1), ymax = sim._domain.second(1);
  const double dy = (ymax - ymin) / double(n_seg);
  Dump d(argv[2]);
  {
    std::vector<double> pos(3 * n);
    for (long long i = 0; i < n; ++i)
      for (int c = 0; c < 3; ++c) pos[3 * i + c] = sim._all_scat_list[i].pos(c);
    d.put("pos", "f8", pos.data(), 3 * n);
    d.put("area", "f8", sim._area.data(), (long long)sim._area.size());
    std::vector<int32_t> c1, c2;
    for (auto* s : sim._c1_scat) c1.push_back((int32_t)(s - sim._all_scat_list.data()));
    for (auto* s : sim._c2_scat) c2.push_back((int32_t)(s - sim._all_scat_list.data()));
    d.put("contact1", "i4", c1.data(), (long long)c1.size());
    d.put("contact2", "i4", c2.data(), (long long)c2.size());
    long long pops[2] = {(long long)sim._c1_pop, (long long)sim._c2_pop};
    d.put("contact_pop", "i8", pops, 2);
    long long n0 = (long long)sim._particle_list.size();
    d.put("n_initial", "i8", &n0, 1);
  }

  // main.cpp:90-92: track_particle(time_step, n) before the loop
  const long long n_tracks = argc > 5 ? std::atoll(argv[5]) : 0;
  {
    std::vector<long long> tlen;
    std::vector<double> tpath;
    for (long long k = 0; k < n_tracks; ++k) {
      orc_rng_init(&g_track, g_seed, (1ull << 32) + (uint64_t)k, 0);
      g_track_path.clear();
      g_mode = 3;
      sim.track_particle(time_step, (int)k);
      g_mode = 0;
      tlen.push_back((long long)g_track_path.size() / 3);
      tpath.insert(tpath.end(), g_track_path.begin(), g_track_path.end());
    }
    d.put("track_len", "i8", tlen.data(), (long long)tlen.size());
    d.put("track_path", "f8", tpath.data(), (long long)tpath.size());
  }

  std::vector<long long> pop_all, curr_all, live_all;
  std::vector<double> times;
  for (long long st = 0; st < n_steps; ++st) {
    g_mode = 2;
    sim.step(time_step);
    g_mode = 0;
    sim.save_metrics(time_step);  // the reference's own files
    // the integer counts behind those files (save_population_profile :568-573, save_currents :628-636)
    std::vector<long long> pop(n_seg, 0), curr(n_seg - 1, 0);
    for (const auto& p : sim._particle_list) {
      int i = (p.pos(1) - ymin) / dy;
      i = i < 0 ? 0 : (i < int(n_seg) ? i : int(n_seg) - 1);
      pop[i]++;
    }
    for (unsigned i = 1; i < n_seg; ++i) {
      double y = ymin + dy * double(i);
      for (const auto& p : sim._particle_list) {
        if (p.old_pos(1) < y && p.pos(1) >= y)
          curr[i - 1]++;
        else if (p.old_pos(1) >= y && p.pos(1) < y)
          curr[i - 1]--;
      }
    }
    pop_all.insert(pop_all.end(), pop.begin(), pop.end());
    curr_all.insert(curr_all.end(), curr.begin(), curr.end());
    times.push_back(sim.time());
    // repopulate_contacts (monte_carlo.h:443-455) as its two repopulate calls
    const double y1[2] = {ymin, ymin + double(n_seg - 1) * dy};
    const double y2[2] = {ymin + dy, ymax};
    const unsigned cpop[2] = {sim._c1_pop, sim._c2_pop};
    const std::vector<const mc::scatterer*>* cl[2] = {&sim._c1_scat, &sim._c2_scat};
    for (int c = 0; c < 2; ++c) {
      std::set<long long> kept;
      for (const auto& p : sim._particle_list) {
        long long s = slot_of(p);
        if (p.pos(1) >= y1[c] && p.pos(1) <= y2[c])
          g_free.insert(s);
        else
          kept.insert(s);
      }
      g_mode = 1;
      sim.repopulate(y1[c], y2[c], cpop[c], *cl[c], sim._particle_list);
      g_mode = 0;
      if (sim._particle_list.size() != kept.size() + cpop[c]) die("unexpected list size after repopulate");
      for (size_t k = 0; k + cpop[c] < sim._particle_list.size(); ++k)
        if (!kept.count(slot_of(sim._particle_list[k]))) die("a kept particle lost its place");
      stamp_new(sim._particle_list);
    }
    live_all.push_back((long long)sim._particle_list.size());
  }

  // final state per slot (site -1: empty)
  const long long ns = g_hwm;
  std::vector<int32_t> site(ns, -1), head(ns, 0);
  std::vector<double> pos(3 * ns, 0.0), old(3 * ns, 0.0), ff(ns, 0.0);
  std::vector<unsigned long long> draws(ns, 0);
  std::vector<long long> hops(ns, 0);
  for (const auto& p : sim._particle_list) {
    long long s = slot_of(p);
    if (s >= ns || site[s] != -1) die("slot out of range or taken twice");
    site[s] = (int32_t)(p._scat_ptr - sim._all_scat_list.data());
    head[s] = p._heading_right ? 1 : 0;
    ff[s] = p._ff_time;
    for (int c = 0; c < 3; ++c) {
      pos[3 * s + c] = p._pos(c);
      old[3 * s + c] = p._old_pos(c);
    }
  }
  for (long long s = 0; s < ns; ++s) {
    draws[s] = stream_of(s).n;
    hops[s] = g_hops[s];
  }
  d.put("pop", "i8", pop_all.data(), (long long)pop_all.size());
  d.put("curr", "i8", curr_all.data(), (long long)curr_all.size());
  d.put("n_live", "i8", live_all.data(), (long long)live_all.size());
  d.put("time", "f8", times.data(), (long long)times.size());
  d.put("site", "i4", site.data(), ns);
  d.put("heading", "i4", head.data(), ns);
  d.put("ff", "f8", ff.data(), ns);
  d.put("xpos", "f8", pos.data(), 3 * ns);
  d.put("xold", "f8", old.data(), 3 * ns);
  d.put("draws", "u8", draws.data(), ns);
  d.put("hops", "i8", hops.data(), ns);
  d.f.close();
  sim._pop_file.close();
  sim._curr_file.close();
  std::cout.rdbuf(cout_buf);
  std::printf("{\"slots\": %lld, \"live\": %lld, \"steps\": %lld, \"sites\": %lld}\n", ns,
              (long long)sim._particle_list.size(), n_steps, n);
  return 0;
}
