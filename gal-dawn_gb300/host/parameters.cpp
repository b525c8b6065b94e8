// Derived from GAL-DAWN (lxrzlyr/GAL-DAWN), Copyright (c) 2024 lxrzlyr,
// Apache License 2.0 (see NOTICE): interface kept for drop-in use.
// Command-line parsing (flags, messages and exit codes of
// src/parameters.cpp:3-98 in the reference project).
#include <dawn/parameters.hxx>

namespace DAWN {
namespace IO {

void printHelp() {
  const int w = 30;
  std::cout << "Usage: program [options]\n"
            << "Options:\n"
            << std::left << "  " << std::setw(w) << "-h, --help"
            << "Show this help message and exit\n"
            << "  " << std::setw(w) << "-i, --input PATH"
            << "Input file path\n"
            << "  " << std::setw(w) << "-o, --output PATH"
            << "Output file path\n"
            << "  " << std::setw(w) << "-l, --sourceList PATH"
            << "List of Source nodes file path\n"
            << "  " << std::setw(w) << "-p, --print [true|false]"
            << "Print source information\n"
            << "  " << std::setw(w) << "-w, --weighted [true|false]"
            << "Set graph as weighted\n"
            << "  " << std::setw(w) << "-s, --source NUM"
            << "Source node (optional, defaults to a random value)\n";
}

static bool parse_bool(const char* arg, const char* what) {
  if (std::string(arg) == "true") return true;
  if (std::string(arg) == "false") return false;
  std::cerr << "Invalid value for " << what << " option. Use 'true' or 'false'.\n";
  exit(EXIT_FAILURE);
}

parameters_t parameters(int argc, char* argv[]) {
  parameters_t params;
  int opt;
  int option_index = 0;
  static struct option long_options[] = {{"help", no_argument, nullptr, 'h'},
                                         {"input", required_argument, nullptr, 'i'},
                                         {"output", required_argument, nullptr, 'o'},
                                         {"sourceList", required_argument, nullptr, 'l'},
                                         {"print", required_argument, nullptr, 'p'},
                                         {"weighted", required_argument, nullptr, 'w'},
                                         {"source", required_argument, nullptr, 's'},
                                         {nullptr, 0, nullptr, 0}};
  while ((opt = getopt_long(argc, argv, "hi:o:l:p:w:s:", long_options, &option_index)) != -1) {
    switch (opt) {
      case 'h':
        printHelp();
        exit(EXIT_SUCCESS);
      case 'i':
        params.input_path = optarg;
        break;
      case 'o':
        params.output_path = optarg;
        break;
      case 'l':
        params.sourceList_path = optarg;
        break;
      case 'p':
        params.print = parse_bool(optarg, "print");
        break;
      case 'w':
        params.weighted = parse_bool(optarg, "weighted");
        break;
      case 's':
        params.source = std::atoi(optarg);
        break;
      default:
        printHelp();
        exit(EXIT_FAILURE);
    }
  }
  if (params.input_path.empty()) {
    std::cerr << "Error: Missing the input file path.\n";
    printHelp();
    exit(EXIT_FAILURE);
  }
  if (params.source == -1) params.source = std::rand();
  return params;
}

}  // namespace IO
}  // namespace DAWN
