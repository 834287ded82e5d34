// driver.cpp -- cntkmc_run: drop-in replacement for the reference's src/main.cpp.
//
//   cntkmc_run [input.json]
//
// Reads the "exciton monte carlo" section of input.json (default file name as main.cpp:34-38),
// then runs the same loop as main.cpp:64-76: kubo_init, save_json_properties,
// kubo_create_particles, and while time < max time: kubo_step(dt), kubo_save_avg_dispalcement_squared.
// With "mode": "contacts" it runs the reference's contacts loop instead (main.cpp:85-106).
// Either way it ends by writing run_report.json (what ran, hop counters, hops/s, and in
// Green-Kubo mode D with its 95 % interval) beside the reference's output files.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>

#include "monte_carlo.hpp"

static const int64_t kChunk = 256;  // time steps per engine call

int main(int argc, char** argv) {
  try {
    std::string filename = argc <= 1 ? "input.json" : argv[1];
    std::ifstream in(filename);
    if (!in) throw std::invalid_argument("cannot open " + filename);
    std::stringstream ss;
    ss << in.rdbuf();
    jl::Value j = jl::parse(ss.str());
    if (!j.has("exciton monte carlo"))
      throw std::invalid_argument("json input file does not contain \"exciton monte carlo\"");
    const jl::Value& jm = j["exciton monte carlo"];
    double time_step = jm["monte carlo time step"].as_double();
    auto t0 = std::chrono::steady_clock::now();
    if (jm.has("mode") && jm["mode"].as_string() == "contacts") {
      // main.cpp:85-106: init, save_json_properties, the tracked particles, then step /
      // save_metrics / repopulate_contacts -- until "maximum time for contacts simulation [seconds]" (the
      // reference's loop has no end)
      if (!jm.has("maximum time for contacts simulation [seconds]"))
        throw std::invalid_argument("contacts mode needs \"maximum time for contacts simulation [seconds]\"");
      cntkmc::monte_carlo sim(jm);
      sim.init();
      sim.save_json_properties();
      // main.cpp:90-92: 100 tracked particles ("number of tracked particles"), in one launch
      sim.track_particles(time_step, jm.has("number of tracked particles") ? jm["number of tracked particles"].as_int32()
                                                                           : 100);
      // the loop's steps in chunks of one engine call each (same rows as one call per step)
      for (int64_t left = sim.steps_until(sim.contacts_max_time(), time_step); left > 0; left -= kChunk)
        sim.contacts_steps_and_save(std::min<int64_t>(kChunk, left), time_step);
      kmc_run_stats rs = sim.run_stats();
      double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      sim.write_run_report(wall);
      std::printf("contacts simulation finished: %lld steps, %lld hops, %u particles, device %.3f s, wall %.3f s\n",
                  (long long)rs.steps_done, (long long)rs.hops, sim.number_of_particles(), sim.device_seconds(), wall);
      std::printf("output: %s\n", sim.output_path().c_str());
      return 0;
    }
    cntkmc::monte_carlo sim(jm);
    sim.kubo_init();
    sim.save_json_properties();
    sim.kubo_create_particles();
    const kmc_nbr_stats& nb = sim.neighbor_stats();
    std::printf("sites: %lld  neighbour entries: %lld (mean %.2f, max %d)  build: %.3f ms\n", (long long)nb.n_sites,
                (long long)nb.nnz, nb.k_mean, nb.k_max, nb.build_ms);
    // main.cpp:70-76's loop, its steps in chunks of one engine call each (same rows)
    for (int64_t left = sim.steps_until(sim.kubo_max_time(), time_step); left > 0; left -= kChunk)
      sim.kubo_steps_and_save(std::min<int64_t>(kChunk, left), time_step);
    kmc_run_stats rs = sim.run_stats();
    double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    sim.write_run_report(wall);
    std::printf("Green-Kubo simulation finished: %lld steps, %lld hops, %lld crossings, device %.3f s, wall %.3f s\n",
                (long long)rs.steps_done, (long long)rs.hops, (long long)rs.crossings, sim.device_seconds(), wall);
    std::printf("output: %s\n", sim.output_path().c_str());
    return 0;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "cntkmc_run: %s\n", e.what());
    return 1;
  }
}
