// ref_stubs.h -- TEST INFRASTRUCTURE: pre-included (g++ -include) when oracle/Makefile
// compiles the reference's Monte Carlo sources into oracle/_ref.
//
// The reference's monte_carlo.{h,cpp} include the exciton_transfer physics
// (src/exciton_transfer/cnt.h, exciton_transfer.h) for the "davoody" rate table only.
// Those files need Armadillo's LAPACK-backed solvers, which are absent, so their include
// guards are defined here and two link stubs take their place.  The Green-Kubo path runs
// with the "forster"/"wong" tables (monte_carlo.cpp:51-57), which need neither class; a call
// into a stub throws.
#ifndef KMC_REF_STUBS_H
#define KMC_REF_STUBS_H

#define _cnt_h_
#define _exciton_transfer_h_

#include <array>
#include <experimental/filesystem>
#include <stdexcept>
#include <string>

#include <armadillo>
#include "json.hpp"

class cnt {
 public:
  cnt(const nlohmann::json, const std::string) { throw std::logic_error("cnt: exciton_transfer physics is not built in the oracle"); }
  void calculate_exciton_dispersion() {}
};

class exciton_transfer {
 public:
  exciton_transfer(const cnt&, const cnt&) { throw std::logic_error("exciton_transfer is not built in the oracle"); }
  template <typename P>
  void save_atom_locations(P, const std::array<double, 2>&, const double&, const double&, std::string = "") {}
  double first_order(const double&, const std::array<double, 2>, const double&, const bool& = false) { return 0; }
};

#endif
