// Derived from GAL-DAWN (lxrzlyr/GAL-DAWN), Copyright (c) 2024 lxrzlyr,
// Apache License 2.0 (see NOTICE): interface kept for drop-in use.
// Command-line options, API of include/dawn/parameters.hxx in the reference
// project (getopt flags -i -o -l -p -w -s -h).
#pragma once
#include <dawn/include.hxx>
#include <getopt.h>

namespace DAWN {
namespace IO {
struct parameters_t {
  std::string input_path;
  std::string output_path;
  std::string sourceList_path;
  bool print = false;
  bool weighted = false;
  int source = -1;
};
parameters_t parameters(int argc, char* argv[]);
void printHelp();
}  // namespace IO
}  // namespace DAWN
