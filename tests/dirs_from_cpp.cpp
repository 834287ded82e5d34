// dirs_from_cpp.cpp -- test helper for the drop-in driver's directory helpers (monte_carlo.hpp:
// expand_home, prepare_directory, check_directory, after src/helper/prepare_directory.hpp):
//   dirs_from_cpp prepare <path> <keep_old_files 0|1>
//   dirs_from_cpp check <path> <should_be_empty 0|1>
// prints the returned path and exits 0, or prints "error: <message>" and exits 1.
#include <iostream>
#include <stdexcept>
#include <string>

#include "monte_carlo.hpp"

int main(int argc, char** argv) {
  if (argc != 4) {
    std::cerr << "usage: dirs_from_cpp prepare|check <path> 0|1\n";
    return 2;
  }
  const std::string op = argv[1], path = argv[2];
  const bool flag = std::string(argv[3]) == "1";
  try {
    if (op == "prepare")
      std::cout << cntkmc::prepare_directory(path, flag) << "\n";
    else if (op == "check")
      std::cout << cntkmc::check_directory(path, flag) << "\n";
    else
      return 2;
  } catch (const std::exception& e) {
    std::cout << "error: " << e.what() << "\n";
    return 1;
  }
  return 0;
}
