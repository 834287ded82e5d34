// json_roundtrip.cpp -- test helper for the drop-in driver's JSON reader/writer (json_lite.hpp):
// reads a JSON file, parses it and writes it back to stdout.  Exit status 2 and the parser's
// message on stderr when the file is not valid JSON.  With a second argument "int" or "int32"
// it prints the document's number through Value::as_int / as_int32 instead.
#include <fstream>
#include <iostream>
#include <sstream>

#include "json_lite.hpp"

int main(int argc, char** argv) {
  if (argc != 2 && argc != 3) {
    std::cerr << "usage: json_roundtrip FILE [int|int32]\n";
    return 1;
  }
  const std::string mode = argc == 3 ? argv[2] : "";
  std::ifstream f(argv[1], std::ios::binary);
  std::stringstream ss;
  ss << f.rdbuf();
  try {
    const jl::Value v = jl::parse(ss.str());
    if (mode == "int")
      std::cout << v.as_int() << "\n";
    else if (mode == "int32")
      std::cout << v.as_int32() << "\n";
    else {
      jl::write(std::cout, v);
      std::cout << "\n";
    }
  } catch (const std::exception& e) {
    std::cerr << e.what() << "\n";
    return 2;
  }
  return 0;
}
