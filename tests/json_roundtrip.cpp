// json_roundtrip.cpp -- test helper for the drop-in driver's JSON reader/writer (json_lite.hpp):
// reads a JSON file, parses it and writes it back to stdout.  Exit status 2 and the parser's
// message on stderr when the file is not valid JSON.
#include <fstream>
#include <iostream>
#include <sstream>

#include "json_lite.hpp"

int main(int argc, char** argv) {
  if (argc != 2) {
    std::cerr << "usage: json_roundtrip FILE\n";
    return 1;
  }
  std::ifstream f(argv[1], std::ios::binary);
  std::stringstream ss;
  ss << f.rdbuf();
  try {
    const jl::Value v = jl::parse(ss.str());
    jl::write(std::cout, v);
    std::cout << "\n";
  } catch (const std::exception& e) {
    std::cerr << e.what() << "\n";
    return 2;
  }
  return 0;
}
