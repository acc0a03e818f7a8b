// `procell`: the command-line drop-in for the reference binary.
//
// Flags, messages and exit codes follow io::CmdArgs (src/io/cmdargs.cpp:11-375) and main
// (src/main.cu:18-34): every message goes to stdout, a bad or repeated flag exits 1, the
// histogram goes to -o or to stdout. Differences, all additive:
//   * -p/--phi-min is optional; without it the smallest value with a nonzero frequency
//     is used, the rule README.md documents and parser.cu:80-96 implements;
//   * --output and --phi are accepted as the README spells them;
//   * -s/--seed N fixes the random stream (default: time(NULL), as the reference seeds);
//   * --stats prints one JSON line of run statistics to stderr;
//   * -d/--tree-depth is range-checked as before but has no effect: it only bounded the
//     reference's per-launch recursion depth, never the result.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <iostream>
#include <string>

#include "../../include/procell.h"

namespace {

const unsigned kMaxTreeDepth = 23;

struct Args {
  bool h0_given = false, types_given = false, output_given = false, t_given = false, phi_given = false,
       depth_given = false, track_ratio = false, seed_given = false, stats = false;
  std::string h0, types, output;
  double t_max = 0.0, phi = 0.0;
  unsigned tree_depth = kMaxTreeDepth;
  uint64_t seed = 0;
};

[[noreturn]] void die(const std::string& msg) {
  std::cout << msg << std::endl;
  std::exit(EXIT_FAILURE);
}

bool take_file(int argc, char** argv, int& i, bool& given, std::string& dst, const char* longf,
               const char* shortf, const char* longname) {
  const std::string s(argv[i]);
  if (s != longf && s != shortf && !(longname && s == longname)) return false;
  if (given) die(std::string("Option ") + longf + " (" + shortf + ") already given");
  if (i < argc - 1) {
    ++i;
    given = true;
    dst = argv[i];
  } else {
    die(std::string("Option ") + longf + " (" + shortf + ") requires a filename");
  }
  return true;
}

bool take_t_max(int argc, char** argv, int& i, Args& a) {
  const std::string s(argv[i]);
  if (s != "--time-max" && s != "-t") return false;
  if (a.t_given) die("Option --time-max (-t) already given");
  if (i >= argc - 1) die("Option --time-max (-t) requires an integer value >= 0");
  ++i;
  const double v = std::atof(argv[i]);
  if (!(v >= 0)) die("Option --time-max (-t) requires an integer value >= 0");
  a.t_given = true;
  a.t_max = v;
  return true;
}

bool take_phi(int argc, char** argv, int& i, Args& a) {
  const std::string s(argv[i]);
  if (s != "--phi-min" && s != "-p" && s != "--phi") return false;
  if (a.phi_given) die("Option --phi-min (-p) already given");
  if (i >= argc - 1) die("Option --phi-min (-p) requires a double value > 0");
  ++i;
  const double v = std::atof(argv[i]);
  if (!(v > 0)) die("Option --phi-min (-p) requires a double value > 0");
  a.phi_given = true;
  a.phi = v;
  return true;
}

bool take_depth(int argc, char** argv, int& i, Args& a) {
  const std::string s(argv[i]);
  if (s != "--tree-depth" && s != "-d") return false;
  if (a.depth_given) die("Option --tree-depth (-d) already given");
  if (i >= argc - 1) die("Option --tree-depth (-d) requires an integer value >= 1");
  ++i;
  int v = 0;
  if (std::sscanf(argv[i], "%d", &v) != 1) v = 0;
  if (!(v >= 1 && (unsigned)v <= kMaxTreeDepth))
    die("Option --tree-depth (-d) requires an integer value >= 1 && <= " + std::to_string(kMaxTreeDepth));
  a.depth_given = true;
  a.tree_depth = (unsigned)v;
  return true;
}

bool take_flag(char** argv, int i, bool& flag, const char* longf, const char* shortf) {
  const std::string s(argv[i]);
  if (s != longf && !(shortf && s == shortf)) return false;
  if (flag) die(std::string("Option ") + longf + (shortf ? std::string(" (") + shortf + ")" : std::string()) + " already given");
  flag = true;
  return true;
}

bool take_seed(int argc, char** argv, int& i, Args& a) {
  const std::string s(argv[i]);
  if (s != "--seed" && s != "-s") return false;
  if (a.seed_given) die("Option --seed (-s) already given");
  if (i >= argc - 1) die("Option --seed (-s) requires an unsigned integer value");
  ++i;
  char* end = nullptr;
  const unsigned long long v = std::strtoull(argv[i], &end, 10);
  if (end == argv[i] || *end != '\0' || argv[i][0] == '-') die("Option --seed (-s) requires an unsigned integer value");
  a.seed_given = true;
  a.seed = v;
  return true;
}

void usage() {
  std::cout << "usage: procell -h HISTOGRAM -c CELL_TYPES -t TIME_MAX [-p PHI] [-o OUTPUT] [-r]\n"
               "               [-s SEED] [-d DEPTH] [--stats]\n"
               "  -h, --histogram FILE         initial fluorescence histogram: <value> <frequency> rows\n"
               "  -c, --cell-types FILE        cell types: <ratio> <mean> <stddev> rows (-1 -1: quiescent)\n"
               "  -t, --time-max T             simulated time limit (>= 0)\n"
               "  -p, --phi-min PHI            fluorescence threshold (> 0; default: smallest value\n"
               "                               with a nonzero frequency)\n"
               "  -o, --output-histogram FILE  output file (default: stdout)\n"
               "  -r, --track-ratio            add one count column per cell type (file order)\n"
               "  -s, --seed N                 random stream seed (default: time)\n"
               "  -d, --tree-depth N           accepted for compatibility (1..23); no effect\n"
               "      --stats                  print run statistics as JSON on stderr"
            << std::endl;
}

}  // namespace

int main(int argc, char** argv) {
  Args a;
  for (int i = 1; i < argc; ++i) {
    const std::string s(argv[i]);
    bool legal = take_file(argc, argv, i, a.h0_given, a.h0, "--histogram", "-h", nullptr);
    legal = legal || take_file(argc, argv, i, a.types_given, a.types, "--cell-types", "-c", nullptr);
    legal = legal || take_file(argc, argv, i, a.output_given, a.output, "--output-histogram", "-o", "--output");
    legal = legal || take_t_max(argc, argv, i, a);
    legal = legal || take_phi(argc, argv, i, a);
    legal = legal || take_depth(argc, argv, i, a);
    legal = legal || take_flag(argv, i, a.track_ratio, "--track-ratio", "-r");
    legal = legal || take_seed(argc, argv, i, a);
    legal = legal || take_flag(argv, i, a.stats, "--stats", nullptr);
    if (s == "--help") {
      usage();
      return EXIT_SUCCESS;
    }
    if (!legal) die("Invalid option " + s);
  }
  if (!a.h0_given || !a.types_given || !a.t_given) {
    std::cout << "The following missing arguments are required:" << std::endl;
    if (!a.h0_given) std::cout << "--histogram (-h)" << std::endl;
    if (!a.types_given) std::cout << "--cell-types (-c)" << std::endl;
    if (!a.t_given) std::cout << "--t-max (-t)" << std::endl;
    return EXIT_FAILURE;
  }
  if (!a.seed_given) a.seed = (uint64_t)std::time(nullptr);

  pc_bin* bins = nullptr;
  uint64_t nbins = 0;
  int rc = pc_load_histogram(a.h0.c_str(), &bins, &nbins);
  if (rc == PC_ERR_IO) die("ERROR: cannot open histogram file " + a.h0);
  if (rc != PC_OK) die("ERROR: cannot read histogram file " + a.h0);
  pc_cell_type* types = nullptr;
  uint32_t ntypes = 0;
  rc = pc_load_cell_types(a.types.c_str(), &types, &ntypes);
  if (rc == PC_ERR_IO) die("ERROR: cannot open cell types file " + a.types);
  if (rc != PC_OK) die("ERROR: proportion distribution of cell types does not sum to 1, aborting.");

  pc_context* ctx = nullptr;
  rc = pc_create(&ctx, 0);
  if (rc != PC_OK) die(std::string("ERROR: ") + pc_last_error(nullptr));
  pc_histogram h;
  std::memset(&h, 0, sizeof(h));
  rc = pc_simulate(ctx, bins, nbins, types, ntypes, a.t_max, a.phi_given ? a.phi : 0.0, a.seed, &h);
  if (rc != PC_OK) die(std::string("ERROR: ") + pc_last_error(ctx));
  rc = pc_write_histogram(a.output_given ? a.output.c_str() : nullptr, &h, a.track_ratio ? 1 : 0);
  if (rc != PC_OK) die("ERROR: cannot write " + (a.output_given ? a.output : std::string("stdout")));
  if (a.stats) {
    const pc_stats& s = h.stats;
    std::fprintf(stderr,
                 "{\"seed\": %llu, \"roots\": %llu, \"divisions\": %llu, \"leaves\": %llu, "
                 "\"uncounted\": %llu, \"vanished\": %llu, \"max_generation\": %u, \"sweeps\": %u, "
                 "\"device_ms\": %.3f}\n",
                 (unsigned long long)a.seed, (unsigned long long)s.roots, (unsigned long long)s.divisions,
                 (unsigned long long)s.leaves, (unsigned long long)s.uncounted,
                 (unsigned long long)s.vanished, s.max_generation, s.sweeps, s.device_ms);
  }
  pc_histogram_free(&h);
  pc_destroy(ctx);
  pc_free(bins);
  pc_free(types);
  return EXIT_SUCCESS;
}
