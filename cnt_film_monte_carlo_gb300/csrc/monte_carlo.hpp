// monte_carlo.hpp -- C++ mirror of the reference's mc::monte_carlo interface
// (src/monte_carlo/monte_carlo.h:35-844, monte_carlo.cpp:254-409) on top of the C ABI: the
// Green-Kubo driver (kubo_*) and the contacts / steady-state flux driver (init, step,
// save_metrics, repopulate_contacts).
//
// Same method names, JSON keys ("exciton monte carlo" section of input.json) and output files
// (particle_dispalcement.avg.squared.dat; scatterer_statistics.dat, population_profile.dat,
// region_current.dat).  Every step runs on the GPU engine.  Errors are
// thrown as std::runtime_error / std::invalid_argument, as the reference throws.
// Extensions: "philox seed" (default 100), "injection": "region" | "uniform",
// "precision": "mixed" | "fp64", "rate type": "forster2d" with "distance [m]" and
// "theta 2d [degrees]" grids, "rate table directory" for a table saved by the reference.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <initializer_list>
#include <stdexcept>
#include <string>
#include <vector>

#include "cntkmc.h"
#include "json_lite.hpp"

namespace cntkmc {

namespace fs = std::filesystem;

inline std::string expand_home(std::string p) {
  if (!p.empty() && p[0] == '~') {
    const char* h = std::getenv("HOME");
    p = std::string(h ? h : "") + p.substr(1);
  }
  return p;
}

// prepare_directory (src/helper/prepare_directory.hpp:8-65)
inline std::string prepare_directory(std::string path, bool keep_old_files = true) {
  path = expand_home(path);
  if (!fs::exists(path)) {
    fs::create_directories(path);
    return path;
  }
  if (!fs::is_directory(path)) throw std::invalid_argument("The input value for output directory is not acceptable.");
  if (!fs::is_empty(path)) {
    if (keep_old_files) {
      int n = 1;
      while (fs::exists(path + "." + std::to_string(n))) ++n;
      fs::rename(path, path + "." + std::to_string(n));
    } else {
      fs::remove_all(path);
    }
    fs::create_directories(path);
  }
  return path;
}

// check_directory (prepare_directory.hpp:68-105)
inline std::string check_directory(std::string path, bool should_be_empty = false) {
  path = expand_home(path);
  if (!fs::exists(path)) throw std::invalid_argument("directory does NOT exists!!!");
  if (!fs::is_directory(path)) throw std::invalid_argument("input path is NOT a directory!!!");
  if (fs::is_empty(path) && !should_be_empty) throw std::invalid_argument("directory is empty!!!");
  return path;
}

class monte_carlo {
 public:
  explicit monte_carlo(const jl::Value& j, int device = 0) : j_(j) {
    bool keep = j.has("keep old results") ? j["keep old results"].as_bool() : true;
    out_dir_ = prepare_directory(j["output directory"].as_string(), keep);
    in_dir_ = check_directory(j["mesh input directory"].as_string(), false);
    int st = 0;
    ctx_ = kmc_create(device, &st);
    if (!ctx_) throw std::runtime_error("cntkmc: no usable CUDA device (status " + std::to_string(st) + ")");
  }
  ~monte_carlo() {
    if (msd_) std::fclose(msd_);
    if (pop_f_) std::fclose(pop_f_);
    if (cur_f_) std::fclose(cur_f_);
    kmc_destroy(ctx_);
  }
  monte_carlo(const monte_carlo&) = delete;
  monte_carlo& operator=(const monte_carlo&) = delete;

  const double& time() const { return time_; }
  const double& kubo_max_time() const { return max_time_; }
  const std::string& output_path() const { return out_dir_; }
  unsigned number_of_particles() const { return (unsigned)n_particles_; }

  // monte_carlo.cpp:254-305
  void kubo_init() {
    setup_film();
    n_sections_ = j_["number of sections for injection region"].as_int32();
    max_time_ = j_["maximum time for kubo simulation [seconds]"].as_double();
  }

  // Contacts (steady-state flux) mode, monte_carlo.h:157-195: the film as kubo_init builds it, the
  // y slabs ("number of segments"), scatterer_statistics.dat, the contact sites and the initial
  // linear profile of excitons.  Extensions: "contact populations" (default [1100, 0], the
  // reference's hard-coded _c1_pop/_c2_pop), "contacts capacity" (exciton slots),
  // "maximum time for contacts simulation [seconds]" (the reference's loop never ends).
  void init() {
    setup_film();
    n_seg_ = j_["number of segments"].as_int32();
    int64_t pops[2] = {1100, 0};
    if (j_.has("contact populations"))
      for (int k = 0; k < 2; ++k) pops[k] = j_["contact populations"][k].as_int();
    kmc_contacts cfg{};
    cfg.n_segments = n_seg_;
    cfg.contact_pop[0] = pops[0];
    cfg.contact_pop[1] = pops[1];
    cfg.seed = seed();
    cfg.capacity = j_.has("contacts capacity") ? j_["contacts capacity"].as_int() : 0;
    area_.assign((size_t)std::max(n_seg_, 0), 0.0);
    std::vector<int64_t> stat(area_.size(), 0);
    check(kmc_contacts_init(ctx_, &cfg, &cinfo_, area_.data(), stat.data()), "kmc_contacts_init");
    pop_.assign((size_t)n_seg_, 0);
    cur_.assign((size_t)n_seg_ - 1, 0);
    n_particles_ = cinfo_.n_initial;
    max_time_ = j_.has("maximum time for contacts simulation [seconds]")
                    ? j_["maximum time for contacts simulation [seconds]"].as_double()
                    : 0.0;
    // get_scatterer_statistics, monte_carlo.h:691-719
    std::FILE* f = std::fopen((fs::path(out_dir_) / "scatterer_statistics.dat").c_str(), "w");
    if (!f) throw std::runtime_error("cannot open scatterer_statistics.dat");
    std::fprintf(f, "position,distribution,population,density\n");
    const double n_sites = double(nbr_.n_sites);
    for (int32_t i = 0; i < n_seg_; ++i)
      std::fprintf(f, "%e,%e,%lld,%e\n", cinfo_.ymin + (double(i) + 0.5) * cinfo_.dy, double(stat[i]) / n_sites,
                   (long long)stat[i], double(stat[i]) / (area_[i] * cinfo_.dy));
    std::fclose(f);
  }

  // step (monte_carlo.h:343-354).  The engine runs the step, the counts behind save_metrics and
  // repopulate_contacts as one unit, in the order of src/main.cpp:99-102.
  void step(double dt) {
    if (!cinfo_.capacity) throw std::logic_error("step: call init() first");
    int64_t live = 0;
    check(kmc_contacts_run(ctx_, 1, dt, velocity_, precision(), pop_.data(), cur_.data(), &live), "kmc_contacts_run");
    device_ms_ += run_stats().last_run_ms;
    dt_ = dt;
    live_ = live;
    time_ += dt;
    ++steps_;
  }

  // save_metrics (monte_carlo.h:519-643): population_profile.dat and region_current.dat rows of
  // the last step
  void save_metrics(double dt) {
    const double dy = cinfo_.dy, ymin = cinfo_.ymin;
    const int32_t n = n_seg_;
    if (!pop_f_) {
      pop_f_ = std::fopen((fs::path(out_dir_) / "population_profile.dat").c_str(), "w");
      cur_f_ = std::fopen((fs::path(out_dir_) / "region_current.dat").c_str(), "w");
      if (!pop_f_ || !cur_f_) throw std::runtime_error("cannot open the contacts output files");
      std::fprintf(pop_f_, "area");
      for (int32_t i = 0; i < n; ++i) std::fprintf(pop_f_, ",%+e", area_[i]);
      std::fprintf(pop_f_, "\n\ndy");
      for (int32_t i = 0; i < n; ++i) std::fprintf(pop_f_, ",%+e", dy);
      std::fprintf(pop_f_, "\n\nsection pos");
      for (int32_t i = 0; i < n; ++i) std::fprintf(pop_f_, ",%+e", ymin + (double(i) + 0.5) * dy);
      std::fprintf(pop_f_, "\n\ntime");
      for (int32_t i = 0; i < n; ++i) std::fprintf(pop_f_, ",section%d", i);
      std::fprintf(pop_f_, "\n");
      // showpos prints the sign of the (signed) interface numbers too
      std::fprintf(cur_f_, "interface area");
      for (int32_t i = 1; i < n; ++i) std::fprintf(cur_f_, ",%+e", (area_[i - 1] + area_[i]) / 2);
      std::fprintf(cur_f_, "\n\ninterface pos");
      for (int32_t i = 1; i < n; ++i) std::fprintf(cur_f_, ",%+e", ymin + dy * double(i));
      std::fprintf(cur_f_, "\n\ntime");
      for (int32_t i = 1; i < n; ++i) std::fprintf(cur_f_, ",interface%+d", i - 1);
      std::fprintf(cur_f_, "\n");
    }
    if (pop_sum_.size() != (size_t)n) {
      pop_sum_.assign((size_t)n, 0);
      cur_sum_.assign((size_t)n - 1, 0);
    }
    for (int32_t i = 0; i < n; ++i) pop_sum_[i] += pop_[i];
    for (int32_t i = 0; i + 1 < n; ++i) cur_sum_[i] += cur_[i];
    ++metric_rows_;
    std::fprintf(pop_f_, "%+e", time_);
    for (int32_t i = 0; i < n; ++i) std::fprintf(pop_f_, ",%+e", double(pop_[i]) / (area_[i] * dy));
    std::fprintf(pop_f_, "\n");
    std::fprintf(cur_f_, "%+e", time_);
    for (int32_t i = 1; i < n; ++i)
      std::fprintf(cur_f_, ",%+e", double(cur_[i - 1]) / (((area_[i - 1] + area_[i]) / 2) * dt));
    std::fprintf(cur_f_, "\n");
    std::fflush(pop_f_);
    std::fflush(cur_f_);
  }

  // repopulate_contacts (monte_carlo.h:443-455): done by the engine at the end of step(); the
  // particle count is updated here, where the reference's list changes size
  void repopulate_contacts() { n_particles_ = live_; }

  // track_particle (monte_carlo.h:786-818): particle_path.<fileNo>.dat.  Track fileNo draws from
  // its own stream, so track_particles(dt, n) (all n in one launch) writes the same files as n
  // calls.  The reference loops until the exciton reaches the last slab; here at most
  // "maximum steps per tracked particle" (default 2^18) steps, with a warning when it has not.
  void track_particle(double dt, int fileNo) { tracks(dt, fileNo, 1); }
  void track_particles(double dt, int count) { tracks(dt, 0, count); }

  double contacts_max_time() const { return max_time_; }
  const kmc_contacts_info& contacts_info() const { return cinfo_; }

  // monte_carlo.h:319-324
  void save_json_properties() const {
    std::ofstream f(fs::path(out_dir_) / "input.json");
    jl::write(f, j_);
    f << "\n";
  }

  // monte_carlo.cpp:308-316.  The MSD sums are also kept per exciton batch (exciton i in batch
  // (i / 32) mod B, B = min(32, n / 32)), for the diffusion coefficient's interval in the run
  // report; the file's rows are the batch sums added in batch order.
  void kubo_create_particles() {
    n_particles_ = j_["number of particles for kubo simulation"].as_int();
    uint64_t seed = this->seed();
    bool uniform = j_.has("injection") && j_["injection"].as_string() == "uniform";
    int64_t ne = n_particles_;
    batches_ = (int32_t)std::max<int64_t>(1, std::min<int64_t>(32, ne / 32));
    batch_counts_.assign((size_t)batches_, 0);
    for (int64_t w = 0; w * 32 < ne; ++w) batch_counts_[(size_t)(w % batches_)] += std::min<int64_t>(32, ne - w * 32);
    check(kmc_set_msd_batches(ctx_, batches_), "kmc_set_msd_batches");
    kmc_inject inj{uniform ? KMC_INJECT_UNIFORM : KMC_INJECT_REGION, n_sections_, &ne, &seed};
    check(kmc_init_excitons(ctx_, &inj), "kmc_init_excitons");
    steps_ = 0;
    times_.clear();
  }

  // monte_carlo.cpp:319-342
  void kubo_step(double dt) {
    run(1, dt);
    ++steps_;
    time_ += dt;
    times_.push_back(time_);
  }

  // monte_carlo.cpp:382-409
  void kubo_save_avg_dispalcement_squared() {
    open_msd_file();
    double s[3];
    check(kmc_get_msd(ctx_, steps_ - 1, 1, s), "kmc_get_msd");
    double n = double(n_particles_);
    std::fprintf(msd_, "%+e,%+e,%+e,%+e\n", time_, s[0] / n, s[1] / n, s[2] / n);
    std::fflush(msd_);
  }

  // n calls of kubo_step(dt), each followed by kubo_save_avg_dispalcement_squared, run as one
  // engine call (the rows and times are those of the n separate calls)
  void kubo_steps_and_save(int64_t n, double dt) {
    if (n <= 0) return;
    run(n, dt);
    std::vector<double> s((size_t)(3 * n));
    check(kmc_get_msd(ctx_, steps_, n, s.data()), "kmc_get_msd");
    open_msd_file();
    const double np = double(n_particles_);
    for (int64_t k = 0; k < n; ++k) {
      time_ += dt;
      ++steps_;
      times_.push_back(time_);
      std::fprintf(msd_, "%+e,%+e,%+e,%+e\n", time_, s[3 * k] / np, s[3 * k + 1] / np, s[3 * k + 2] / np);
    }
    std::fflush(msd_);
  }

  // n rounds of step(dt), save_metrics(dt), repopulate_contacts() as one engine call
  void contacts_steps_and_save(int64_t n, double dt) {
    if (n <= 0) return;
    if (!cinfo_.capacity) throw std::logic_error("contacts_steps_and_save: call init() first");
    std::vector<int64_t> pop((size_t)(n * n_seg_)), cur((size_t)(n * (n_seg_ - 1))), live((size_t)n);
    check(kmc_contacts_run(ctx_, n, dt, velocity_, precision(), pop.data(), cur.data(), live.data()),
          "kmc_contacts_run");
    device_ms_ += run_stats().last_run_ms;
    dt_ = dt;
    for (int64_t k = 0; k < n; ++k) {
      std::copy(pop.begin() + k * n_seg_, pop.begin() + (k + 1) * n_seg_, pop_.begin());
      std::copy(cur.begin() + k * (n_seg_ - 1), cur.begin() + (k + 1) * (n_seg_ - 1), cur_.begin());
      live_ = live[(size_t)k];
      time_ += dt;
      ++steps_;
      save_metrics(dt);
      repopulate_contacts();
    }
  }

  // the number of steps of main.cpp's `while (time < max time) step(dt)` from the current time,
  // with the same floating-point accumulation of the time
  // The number of steps of main.cpp's `while (time < max time)` loop from the current time, with
  // the loop's own accumulation of the time.  A time step that cannot advance the clock (not
  // positive, or too small to change it) would make that loop run forever, and one that needs
  // more than 1e10 steps practically so: both are refused.
  int64_t steps_until(double t_max, double dt) const {
    if (time_ < t_max && (t_max - time_) / dt > 1e10)
      throw std::invalid_argument("monte carlo time step: more than 1e10 steps to the maximum time");
    int64_t n = 0;
    for (double t = time_; t < t_max; t += dt) {
      if (!(dt > 0) || !std::isfinite(dt) || t + dt == t)
        throw std::invalid_argument("monte carlo time step does not advance the time");
      ++n;
    }
    return n;
  }

  const kmc_nbr_stats& neighbor_stats() const { return nbr_; }
  double device_seconds() const { return device_ms_ / 1e3; }

  // run_report.json in the output directory (no counterpart in the reference, which prints only
  // wall-clock start and end, main.cpp:26-27,109-111): what ran (mode, precision, seed,
  // injection, particles, steps, time step), the film's neighbour lists, the hop counters, device
  // and wall seconds with hops/s, and in Green-Kubo mode the diffusion coefficient per axis with
  // its 95 % interval from the exciton batches (kmc_fit_diffusion over the last 80 % of the steps).
  void write_run_report(double wall_seconds) const {
    const kmc_run_stats rs = run_stats();
    const bool kubo = !cinfo_.capacity;
    std::FILE* f = std::fopen((fs::path(out_dir_) / "run_report.json").c_str(), "w");
    if (!f) throw std::runtime_error("cannot open run_report.json");
    auto num = [&](double v) {
      if (std::isfinite(v))
        std::fprintf(f, "%.17g", v);
      else
        std::fprintf(f, "null");
    };
    std::fprintf(f, "{\n  \"engine\": \"%s\",\n  \"mode\": \"%s\",\n", kmc_version(), kubo ? "kubo" : "contacts");
    std::fprintf(f, "  \"precision\": \"%s\",\n  \"philox seed\": %llu,\n", precision() == KMC_PREC_FP64 ? "fp64" : "mixed",
                 (unsigned long long)seed());
    if (kubo)
      std::fprintf(f, "  \"injection\": \"%s\",\n",
                   j_.has("injection") && j_["injection"].as_string() == "uniform" ? "uniform" : "region");
    std::fprintf(f, "  \"particles\": %lld,\n  \"steps\": %lld,\n  \"time step [s]\": ", (long long)n_particles_,
                 (long long)steps_);
    num(dt_);
    std::fprintf(f, ",\n  \"simulated time [s]\": ");
    num(time_);
    std::fprintf(f, ",\n  \"sites\": %lld,\n  \"neighbour entries\": %lld,\n  \"mean neighbours per site\": ",
                 (long long)nbr_.n_sites, (long long)nbr_.nnz);
    num(nbr_.k_mean);
    std::fprintf(f, ",\n  \"max neighbours per site\": %d,\n  \"neighbour build [s]\": ", nbr_.k_max);
    num(nbr_.build_ms / 1e3);
    std::fprintf(f, ",\n  \"hops\": %lld,\n  \"crossings\": %lld,\n  \"exact re-resolves\": %lld,\n", (long long)rs.hops,
                 (long long)rs.crossings, (long long)rs.exact_resolves);
    const double dev_s = device_ms_ / 1e3;
    std::fprintf(f, "  \"device seconds\": ");
    num(dev_s);
    std::fprintf(f, ",\n  \"hops per second (device)\": ");
    num(dev_s > 0 ? (double)rs.hops / dev_s : NAN);
    std::fprintf(f, ",\n  \"wall seconds\": ");
    num(wall_seconds);
    std::fprintf(f, ",\n  \"hops per second (wall)\": ");
    num(wall_seconds > 0 ? (double)rs.hops / wall_seconds : NAN);
    if (kubo) {
      double D[3] = {NAN, NAN, NAN}, ci[3] = {NAN, NAN, NAN};
      if (steps_ >= 2 && (int64_t)times_.size() == steps_) {
        std::vector<double> m((size_t)steps_ * (size_t)batches_ * 3);
        check(kmc_get_msd_batches(ctx_, 0, steps_, m.data()), "kmc_get_msd_batches");
        check(kmc_fit_diffusion(m.data(), batch_counts_.data(), times_.data(), steps_, batches_, 0.8, D, ci),
              "kmc_fit_diffusion");
      }
      std::fprintf(f, ",\n  \"msd batches\": %d,\n  \"fit fraction\": 0.8,\n  \"diffusion coefficient [m^2/s]\": [",
                   batches_);
      for (int k = 0; k < 3; ++k) {
        if (k) std::fprintf(f, ", ");
        num(D[k]);
      }
      std::fprintf(f, "],\n  \"diffusion 95%% interval [m^2/s]\": [");
      for (int k = 0; k < 3; ++k) {
        if (k) std::fprintf(f, ", ");
        num(ci[k]);
      }
      std::fprintf(f, "]");
    } else {
      // the flux-gradient D of every slab interface (visualization/monte_carlo_results.py:428-442):
      // steady current over the gradient of the average density, both averaged over the rows of
      // the output files, here from their exact counts
      std::fprintf(f, ",\n  \"live excitons\": %lld,\n  \"flux-gradient D [m^2/s]\": [", (long long)live_);
      const double dy = cinfo_.dy;
      for (int32_t k = 0; k + 1 < n_seg_ && metric_rows_ > 0; ++k) {
        const double rows = double(metric_rows_);
        const double p0 = double(pop_sum_[k]) / rows / (area_[k] * dy), p1 = double(pop_sum_[k + 1]) / rows / (area_[k + 1] * dy);
        const double steady = double(cur_sum_[k]) / rows / (((area_[k] + area_[k + 1]) / 2) * dt_);
        if (k) std::fprintf(f, ", ");
        num(steady / ((p1 - p0) / dy));
      }
      std::fprintf(f, "]");
    }
    std::fprintf(f, "\n}\n");
    std::fclose(f);
  }
  kmc_run_stats run_stats() const {
    kmc_run_stats s{};
    kmc_get_run_stats(ctx_, &s);
    return s;
  }

 private:
  void open_msd_file() {
    if (msd_) return;
    msd_ = std::fopen((fs::path(out_dir_) / "particle_dispalcement.avg.squared.dat").c_str(), "w");
    if (!msd_) throw std::runtime_error("cannot open the MSD file");
    std::fprintf(msd_, "# this file contains the average of dx^2, dy^2, and dz^2 of the particle ensemble over time\n");
    std::fprintf(msd_, "# number of particles: %lld\n\ntime,x,y,z\n", (long long)n_particles_);
  }
  void tracks(double dt, int first, int count) {
    if (count <= 0) return;
    const int64_t cap = j_.has("maximum steps per tracked particle") ? j_["maximum steps per tracked particle"].as_int()
                                                                      : (int64_t)1 << 18;
    std::vector<double> path((size_t)count * (size_t)cap * 3);
    std::vector<int64_t> len((size_t)count);
    std::vector<int32_t> arrived((size_t)count);
    check(kmc_contacts_track(ctx_, first, count, dt, velocity_, cap, path.data(), len.data(), arrived.data()),
          "kmc_contacts_track");
    for (int t = 0; t < count; ++t) {
      const std::string name = "particle_path." + std::to_string(first + t) + ".dat";
      std::FILE* f = std::fopen((fs::path(out_dir_) / name).c_str(), "w");
      if (!f) throw std::runtime_error("cannot open " + name);
      const double* p = &path[(size_t)t * (size_t)cap * 3];
      for (int64_t k = 0; k < len[t]; ++k) std::fprintf(f, "   %+e %+e %+e\n", p[3 * k], p[3 * k + 1], p[3 * k + 2]);
      std::fprintf(f, "\n");
      std::fclose(f);
      if (!arrived[t])
        std::fprintf(stderr, "track_particle %d: not at the last slab after %lld steps\n", first + t, (long long)cap);
    }
  }
  uint64_t seed() const { return j_.has("philox seed") ? (uint64_t)j_["philox seed"].as_int() : 100u; }
  void run(int64_t n, double dt) {
    check(kmc_run(ctx_, n, dt, velocity_, precision()), "kmc_run");
    device_ms_ += run_stats().last_run_ms;
    dt_ = dt;
  }
  int precision() const {
    return (j_.has("precision") && j_["precision"].as_string() == "fp64") ? KMC_PREC_FP64 : KMC_PREC_MIXED;
  }
  // the film part of kubo_init / init: table, mesh, trim_scats, buckets and neighbour lists
  void setup_film() {
    r_max_ = j_["max hopping radius [m]"].as_double();
    velocity_ = j_["exciton velocity [m/s]"].as_double();
    create_scattering_table();
    int64_t nt = 0, np = 0;
    check(kmc_read_mesh(in_dir_.c_str(), &nt, &np, nullptr, nullptr, nullptr, nullptr), "kmc_read_mesh");
    int64_t n = nt * np;
    pos_.resize(3 * n);
    orient_.resize(3 * n);
    left_.resize(n);
    right_.resize(n);
    check(kmc_read_mesh(in_dir_.c_str(), &nt, &np, pos_.data(), orient_.data(), left_.data(), right_.data()),
          "kmc_read_mesh");
    const jl::Value& tl = j_["trim limits"];
    double lim[6] = {tl["xlim"][0].as_double(), tl["xlim"][1].as_double(), tl["ylim"][0].as_double(),
                     tl["ylim"][1].as_double(), tl["zlim"][0].as_double(), tl["zlim"][1].as_double()};
    int64_t kept = 0;
    check(kmc_trim_sites(n, pos_.data(), orient_.data(), left_.data(), right_.data(), lim, &kept), "kmc_trim_sites");
    if (kept == 0) throw std::invalid_argument("no site left inside the trim limits");
    int64_t off[2] = {0, kept};
    kmc_film f{1, off, pos_.data(), orient_.data(), left_.data(), right_.data()};
    check(kmc_load_film(ctx_, &f), "kmc_load_film");
    kmc_table t{};
    t.kind = table_kind_;
    for (size_t d = 0; d < grids_.size(); ++d) {
      t.n[d] = (int32_t)grids_[d].size();
      t.grid[d] = grids_[d].data();
    }
    t.rate = rates_.data();
    check(kmc_set_rate_table(ctx_, &t), "kmc_set_rate_table");
    check(kmc_build_neighbors(ctx_, r_max_, &nbr_), "kmc_build_neighbors");
  }
  void check(int rc, const char* what) const {
    if (rc != KMC_OK) throw std::runtime_error(std::string(what) + ": " + kmc_last_error(ctx_));
  }
  // A table grid's point count {start, end, n}[2]: a number in [1, 2^31 - 1], as the library
  // checks it, taken before any array is sized from it.
  static size_t grid_n(double x) {
    if (!(x >= 1.0 && x <= 2147483647.0)) throw std::invalid_argument("bad rate-table grids");
    return (size_t)x;
  }
  // entries of a table with these grid sizes, refused past 2^34 (128 GiB of rates) so that the
  // product cannot wrap and leave the library a buffer smaller than the table it writes
  static size_t table_size(std::initializer_list<size_t> n) {
    const size_t cap = size_t(1) << 34;
    size_t p = 1;
    for (size_t k : n) {
      if (k > cap / p) throw std::invalid_argument("rate table too large");
      p *= k;
    }
    return p;
  }
  // monte_carlo.cpp:24-61
  void create_scattering_table() {
    std::string rt = j_["rate type"].as_string();
    if (rt == "forster" || rt == "wong") {
      double g0 = rt == "forster" ? 1.e15 : 1.e13;
      const jl::Value *th = &j_["theta [degrees]"], *z = &j_["zshift [m]"], *a1 = &j_["axis shift 1 [m]"],
                      *a2 = &j_["axis shift 2 [m]"];
      double gt[3] = {(*th)[0].as_double(), (*th)[1].as_double(), (*th)[2].as_double()};
      double gz[3] = {(*z)[0].as_double(), (*z)[1].as_double(), (*z)[2].as_double()};
      double g1[3] = {(*a1)[0].as_double(), (*a1)[1].as_double(), (*a1)[2].as_double()};
      double g2[3] = {(*a2)[0].as_double(), (*a2)[1].as_double(), (*a2)[2].as_double()};
      const size_t nt = grid_n(gt[2]), nz = grid_n(gz[2]), n1 = grid_n(g1[2]), n2 = grid_n(g2[2]);
      const size_t n_rates = table_size({nt, nz, n1, n2});
      grids_.assign(4, {});
      grids_[0].resize(nt);
      grids_[1].resize(nz);
      grids_[2].resize(n1);
      grids_[3].resize(n2);
      rates_.resize(n_rates);
      if (kmc_forster_table(g0, gt, gz, g1, g2, grids_[0].data(), grids_[1].data(), grids_[2].data(), grids_[3].data(),
                            rates_.data()) != KMC_OK)
        throw std::invalid_argument("bad rate-table grids");
      table_kind_ = KMC_TABLE_4D;
      return;
    }
    if (rt == "forster2d") {
      auto g3 = [&](const char* key, double a, double b, double n, double* out) {
        if (j_.has(key)) {
          const jl::Value& g = j_[key];
          a = g[0].as_double();
          b = g[1].as_double();
          n = g[2].as_double();
        }
        out[0] = a;
        out[1] = b;
        out[2] = n;
      };
      double gd[3], gt[3];
      g3("distance [m]", 0.5e-9, 10e-9, 96, gd);
      g3("theta 2d [degrees]", 0, 90, 91, gt);
      const size_t nd = grid_n(gd[2]), nt = grid_n(gt[2]);
      const size_t n_rates = table_size({nd, nt});
      grids_.assign(2, {});
      grids_[0].resize(nd);
      grids_[1].resize(nt);
      rates_.resize(n_rates);
      if (kmc_forster2d_table(1.e15, gd, gt, grids_[0].data(), grids_[1].data(), rates_.data()) != KMC_OK)
        throw std::invalid_argument("bad rate-table grids");
      table_kind_ = KMC_TABLE_2D;
      return;
    }
    if (rt == "davoody") {
      if (!j_.has("rate table directory"))
        throw std::invalid_argument("rate type davoody needs \"rate table directory\" (a table saved by the reference)");
      read_reference_table(expand_home(j_["rate table directory"].as_string()));
      return;
    }
    throw std::invalid_argument("rate type must be one of the following: \"davoody\", \"forster\", \"wong\", \"forster2d\"");
  }
  // scat_table.*.dat written by scattering_struct::save (scattering_struct.h:56-94)
  void read_reference_table(const std::string& dir) {
    auto col = [&](const char* name) {
      std::ifstream f(fs::path(dir) / (std::string("scat_table.") + name + ".dat"));
      if (!f) throw std::runtime_error(std::string("missing scat_table.") + name + ".dat");
      std::vector<double> v;
      double x;
      while (f >> x) v.push_back(x);
      if (!f.eof()) throw std::runtime_error(std::string("scat_table.") + name + ".dat: a token that is not a number");
      return v;
    };
    grids_ = {col("theta"), col("z_shift"), col("axis_shift_1"), col("axis_shift_2")};
    std::ifstream f(fs::path(dir) / "scat_table.rates.dat");
    std::string line;
    for (int i = 0; i < 4 && std::getline(f, line); ++i) {
    }
    rates_.clear();
    double x;
    while (f >> x) rates_.push_back(x);
    if (!f.eof()) throw std::runtime_error("scat_table.rates.dat: missing, or a token that is not a number");
    for (const auto& g : grids_)
      if (g.empty()) throw std::runtime_error("scat_table: an empty grid file");
    if (rates_.size() != table_size({grids_[0].size(), grids_[1].size(), grids_[2].size(), grids_[3].size()}))
      throw std::runtime_error("scat_table.rates.dat does not match its grids");
    table_kind_ = KMC_TABLE_4D;
  }

  jl::Value j_;
  std::string out_dir_, in_dir_;
  kmc_ctx* ctx_ = nullptr;
  double time_ = 0, max_time_ = 0, r_max_ = 0, velocity_ = 0;
  int n_sections_ = 5;
  int64_t n_particles_ = 0, steps_ = 0;
  double dt_ = 0, device_ms_ = 0;
  int32_t batches_ = 1;
  std::vector<int64_t> batch_counts_;
  std::vector<double> times_;  // end time of every Green-Kubo step, accumulated as time_
  int table_kind_ = KMC_TABLE_4D;
  std::vector<std::vector<double>> grids_;
  std::vector<double> rates_, pos_, orient_;
  std::vector<int32_t> left_, right_;
  kmc_nbr_stats nbr_{};
  std::FILE* msd_ = nullptr;
  // contacts mode
  int32_t n_seg_ = 0;
  kmc_contacts_info cinfo_{};
  std::vector<double> area_;
  std::vector<int64_t> pop_, cur_;
  std::vector<long long> pop_sum_, cur_sum_;  // the counts summed over the metric rows written
  int64_t metric_rows_ = 0;
  int64_t live_ = 0;
  std::FILE *pop_f_ = nullptr, *cur_f_ = nullptr;
};

}  // namespace cntkmc
