// ammsb_main.cpp -- command-line driver of the GB300 sampler.
//
// The sequential branch of the reference's apps/main/main.cc:7-99 over the C
// ABI of include/ammsb_gpu.h: echo "Command line: ...", --help prints the
// options with their defaults, the options are the reference's
// (options.h:142-203: same long and short names, parse_size_t integers of
// options.cc:5-67, a `--config` file of `name = value` lines with [section]
// prefixes, unrecognised arguments left over as in allow_unregistered), the
// graph comes from a relativity/SNAP text file (-f, -c relativity), the
// held-out and test sets are drawn (held-out ratio 0 means 0.1, as
// learner.cc:87-92) -- or a network saved before is read back with
// -c preprocessed -f DIR (network.cc:49-65) --, then init() and run() print
// the reference's perplexity lines and its PrintStats tables.  IO and
// option errors exit with status 33 (main.cc:79-86).
//
// GB300 additions: -c synthetic takes -f as comma-separated generator
// parameters (n=5000,k_true=50,size_min=10,size_max=500,intra_degree=4,
// seed=0, ...); --gb300.pi-dtype f32|bf16, --gb300.chain, --gb300.device,
// --gb300.graph 0|1, --gb300.pipeline 0|1, --gb300.verbose; --gb300.save PATH writes a checkpoint
// of the final chain and --gb300.resume PATH continues a saved one;
// --gb300.save-network DIR saves the loaded network as the reference's
// preprocessing tool does (test/preprocess/main.cc, --save).
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/ammsb_gpu.h"

namespace {

struct OptionError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct IOError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// options.cc:5-67: decimal, 0x hex, leading-0 octal, k/m/g suffixes
uint64_t parse_size_t(const std::string& arg) {
  std::string s = arg;
  int base = 10;
  if (s.size() >= 2 && s[0] == '0' && (s[1] == 'x' || s[1] == 'X')) {
    base = 16;
    s = s.substr(2);
  } else if (!s.empty() && s[0] == '0') {
    base = 8;
    s = s.substr(1);
  }
  unsigned __int128 n = 0;
  for (size_t i = 0; i < s.size(); ++i) {
    const char ch = s[i];
    std::string rest = s.substr(i);
    for (auto& c : rest) c = (char)std::tolower((unsigned char)c);
    int d = -1;
    if (ch >= '0' && ch <= '9') d = ch - '0';
    else if (base == 16 && std::isxdigit((unsigned char)ch)) d = std::tolower(ch) - 'a' + 10;
    if (d >= 0 && d < base) {
      n = n * (unsigned)base + (unsigned)d;
    } else if (rest == "g" || rest == "gb") {
      n <<= 30;
      break;
    } else if (rest == "m" || rest == "mb") {
      n <<= 20;
      break;
    } else if (rest == "k" || rest == "kb") {
      n <<= 10;
      break;
    } else {
      throw OptionError(std::string("Unknown characters in number: '") + ch + "'");
    }
    if (n >> 64) throw OptionError("Overflow in parse_size_t");
  }
  if (n >> 64) throw OptionError("Overflow in parse_size_t");
  return (uint64_t)n;
}

int64_t parse_int(const std::string& arg, int bits, bool is_signed) {
  const bool neg = !arg.empty() && arg[0] == '-';
  const uint64_t mag = parse_size_t(neg ? arg.substr(1) : arg);
  const unsigned __int128 lim = is_signed ? ((unsigned __int128)1 << (bits - 1))
                                          : ((unsigned __int128)1 << bits);
  if (neg && (!is_signed || mag > (uint64_t)lim)) throw OptionError("number out of range");
  if (!neg && mag >= lim) throw OptionError("number out of range");
  return neg ? -(int64_t)mag : (int64_t)mag;
}

double parse_double(const std::string& arg) {
  char* end = nullptr;
  errno = 0;
  const double v = std::strtod(arg.c_str(), &end);
  if (end == arg.c_str() || *end != '\0' || errno == ERANGE)
    throw OptionError("invalid number '" + arg + "'");
  return v;
}

enum Kind { kDouble, kSize, kInt, kStrategy, kStr, kSwitch, kDtype };

struct Spec {
  const char* long_name;
  char short_name;
  Kind kind;
  const char* help;
};

const Spec kSpecs[] = {
    {"mcmc.alpha", 0, kDouble, "alpha"},
    {"mcmc.eta0", 0, kDouble, "eta0"},
    {"mcmc.eta1", 0, kDouble, "eta1"},
    {"mcmc.epsilon", 0, kDouble, "epsilon"},
    {"mcmc.a", 0, kDouble, "a"},
    {"mcmc.b", 0, kDouble, "b"},
    {"mcmc.c", 0, kDouble, "c"},
    {"mcmc.K", 'K', kSize, "K"},
    {"mcmc.mini-batch-size", 'm', kSize, "mini_batch_size"},
    {"mcmc.num-node-sample", 'n', kSize, "neighbor sample size"},
    {"mcmc.strategy", 0, kStrategy, "sampling strategy"},
    {"mcmc.sampler.max-source", 0, kSize, "minibatch sampler max source nodes"},
    {"mcmc.max-iteration", 'x', kSize, "max_iteration"},
    {"mcmc.interval", 'i', kSize, "perplexity interval"},
    {"mcmc.stats", 'I', kSize, "stats interval"},
    {"mcmc.num-updates", 0, kSize, "num_updates"},
    {"mcmc.held-out-ratio", 'h', kDouble, "held_out_ratio"},
    {"mcmc.seed", 0, kInt, "random seed"},
    {"mcmc.convergence", 0, kDouble, "convergence threshold"},
    {"mcmc.input.file", 'f', kStr, "input file"},
    {"mcmc.input.class", 'c', kStr, "input class"},
    {"mcmc.input.contiguous", 0, kSwitch, "contiguous input data"},
    {"mcmc.input.compressed", 0, kSwitch, "compressed input data"},
    {"config", 0, kStr, "config file"},
    {"gb300.pi-dtype", 0, kDtype, "pi storage type: f32 or bf16"},
    {"gb300.chain", 0, kInt, "chain index (Philox key word)"},
    {"gb300.device", 0, kInt, "CUDA device"},
    {"gb300.graph", 0, kInt, "launch iterations as CUDA graphs (0/1)"},
    {"gb300.pipeline", 0, kInt,
     "draw the next iterations on a second stream during the update (1) or in loop order (0)"},
    {"gb300.verbose", 0, kInt, "verbosity"},
    {"gb300.save", 0, kStr, "write a checkpoint of the final state to this file"},
    {"gb300.resume", 0, kStr, "continue the chain saved in this checkpoint"},
    {"gb300.save-network", 0, kStr,
     "save the network (graph, held-out and test sets) into this directory; "
     "read it back with -c preprocessed -f DIR"},
};

const Spec* find_long(const std::string& name) {
  for (const auto& s : kSpecs)
    if (name == s.long_name) return &s;
  return nullptr;
}
const Spec* find_short(char c) {
  for (const auto& s : kSpecs)
    if (s.short_name && s.short_name == c) return &s;
  return nullptr;
}

struct Cli {
  ammsb_options o;
  std::string input_file, input_class = "relativity", config_file, save_path, resume_path;
  std::string save_network;
  bool contiguous = false, compressed = false;
  std::vector<std::string> remains;
  std::map<std::string, bool> seen;

  Cli() { ammsb_options_default(&o); }

  void set(const Spec& s, const std::string& v) {
    const std::string n = s.long_name;
    if (n == "mcmc.alpha") o.alpha = parse_double(v);
    else if (n == "mcmc.eta0") o.eta0 = parse_double(v);
    else if (n == "mcmc.eta1") o.eta1 = parse_double(v);
    else if (n == "mcmc.epsilon") o.epsilon = parse_double(v);
    else if (n == "mcmc.a") o.a = parse_double(v);
    else if (n == "mcmc.b") o.b = parse_double(v);
    else if (n == "mcmc.c") o.c = parse_double(v);
    else if (n == "mcmc.K") o.K = (int64_t)parse_size_t(v);
    else if (n == "mcmc.mini-batch-size") o.mini_batch_size = (int64_t)parse_size_t(v);
    else if (n == "mcmc.num-node-sample") o.num_node_sample = (int64_t)parse_size_t(v);
    else if (n == "mcmc.strategy") {
      // types.h:11-40
      if (v == "stratified-random-node") o.strategy = AMMSB_STRATIFIED_RANDOM_NODE;
      else if (v == "stratified-random-node-links") o.strategy = AMMSB_STRATIFIED_RANDOM_NODE_LINKS;
      else if (v == "stratified-random-node-nonlinks")
        o.strategy = AMMSB_STRATIFIED_RANDOM_NODE_NONLINKS;
      else if (v == "random-edge") o.strategy = AMMSB_RANDOM_EDGE;
      else throw OptionError("Unknown strategy");
    } else if (n == "mcmc.sampler.max-source") o.sampler_max_source = (int64_t)parse_size_t(v);
    else if (n == "mcmc.max-iteration") o.max_iteration = (int64_t)parse_size_t(v);
    else if (n == "mcmc.interval") o.interval = (int64_t)parse_size_t(v);
    else if (n == "mcmc.stats") o.stats_print_interval = (int64_t)parse_size_t(v);
    else if (n == "mcmc.num-updates") o.num_updates = (int64_t)parse_size_t(v);
    else if (n == "mcmc.held-out-ratio") o.held_out_ratio = parse_double(v);
    else if (n == "mcmc.seed") o.random_seed = (int32_t)parse_int(v, 32, true);
    else if (n == "mcmc.convergence") o.convergence_threshold = parse_double(v);
    else if (n == "mcmc.input.file") input_file = v;
    else if (n == "mcmc.input.class") input_class = v;
    else if (n == "config") config_file = v;
    else if (n == "gb300.pi-dtype") {
      if (v == "f32" || v == "fp32" || v == "float32") o.pi_dtype = AMMSB_PI_F32;
      else if (v == "bf16" || v == "bfloat16") o.pi_dtype = AMMSB_PI_BF16;
      else throw OptionError("pi dtype must be f32 or bf16");
    } else if (n == "gb300.chain") o.chain = (int32_t)parse_int(v, 32, true);
    else if (n == "gb300.device") o.device = (int32_t)parse_int(v, 32, true);
    else if (n == "gb300.graph") o.use_graph = (int32_t)parse_int(v, 32, true);
    else if (n == "gb300.pipeline") o.pipeline = (int32_t)parse_int(v, 32, true);
    else if (n == "gb300.verbose") o.verbose = (int32_t)parse_int(v, 32, true);
    else if (n == "gb300.save") save_path = v;
    else if (n == "gb300.resume") resume_path = v;
    else if (n == "gb300.save-network") save_network = v;
  }

  void take(const Spec& s, const std::string& v, bool from_config) {
    if (seen.count(s.long_name)) {
      if (from_config) return;  // the command line wins
      throw OptionError(std::string("option '--") + s.long_name +
                        "' cannot be specified more than once");
    }
    seen[s.long_name] = true;
    set(s, v);
  }

  void parse(const std::vector<std::string>& argv) {
    for (size_t i = 0; i < argv.size(); ++i) {
      const std::string& tok = argv[i];
      const Spec* s = nullptr;
      std::string value;
      bool has_value = false;
      if (tok.rfind("--", 0) == 0) {
        std::string name = tok.substr(2);
        const size_t eq = name.find('=');
        if (eq != std::string::npos) {
          value = name.substr(eq + 1);
          name = name.substr(0, eq);
          has_value = true;
        }
        s = find_long(name);
      } else if (tok.size() >= 2 && tok[0] == '-' && !std::isdigit((unsigned char)tok[1]) &&
                 tok[1] != '.') {
        s = find_short(tok[1]);
        if (s && tok.size() > 2) {
          value = tok.substr(2);
          has_value = true;
        }
      }
      if (!s) {
        remains.push_back(tok);
        continue;
      }
      if (s->kind == kSwitch) {
        if (std::string(s->long_name) == "mcmc.input.contiguous") contiguous = true;
        else compressed = true;
        continue;
      }
      if (!has_value) {
        if (i + 1 >= argv.size())
          throw OptionError(std::string("the required argument for option '--") + s->long_name +
                            "' is missing");
        value = argv[++i];
      }
      take(*s, value, false);
    }
    if (!config_file.empty()) parse_config(config_file);
    // options.h:257-262
    if (o.a == 0.0) o.a = std::pow(o.b, -o.c);
    if (o.alpha == 0.0) o.alpha = 1.0 / (double)o.K;
  }

  void parse_config(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw IOError("cannot open config file " + path);
    std::string line, section;
    while (std::getline(f, line)) {
      const size_t hash = line.find('#');
      if (hash != std::string::npos) line = line.substr(0, hash);
      const size_t b = line.find_first_not_of(" \t\r");
      if (b == std::string::npos) continue;
      line = line.substr(b, line.find_last_not_of(" \t\r") - b + 1);
      if (line.front() == '[' && line.back() == ']') {
        section = line.substr(1, line.size() - 2) + ".";
        continue;
      }
      const size_t eq = line.find('=');
      if (eq == std::string::npos) throw OptionError("invalid config line: " + line);
      auto trim = [](std::string x) {
        const size_t p = x.find_first_not_of(" \t");
        if (p == std::string::npos) return std::string();
        return x.substr(p, x.find_last_not_of(" \t") - p + 1);
      };
      const std::string key = section + trim(line.substr(0, eq));
      const std::string val = trim(line.substr(eq + 1));
      const Spec* s = find_long(key);
      if (!s) throw OptionError("unrecognised option '" + key + "' in config");
      if (s->kind == kSwitch) {
        if (val == "1" || val == "true" || val == "yes" || val == "on") {
          if (key == "mcmc.input.contiguous") contiguous = true;
          else compressed = true;
        }
        continue;
      }
      take(*s, val, true);
    }
  }
};

void print_help(std::ostream& os) {
  ammsb_options d;
  ammsb_options_default(&d);
  os << "Options:\n";
  for (const auto& s : kSpecs) {
    os << "  --" << s.long_name;
    if (s.short_name) os << " [-" << s.short_name << "]";
    os << "\t" << s.help << "\n";
  }
  os << "defaults: alpha " << d.alpha << " (0: 1/K) eta (" << d.eta0 << "," << d.eta1
     << ") epsilon " << d.epsilon << " a " << d.a << " (0: b^-c) b " << d.b << " c " << d.c
     << " K " << d.K << " mini-batch-size " << d.mini_batch_size << " (0: N/10)"
     << " num-node-sample " << d.num_node_sample << " (0: N/50) max-iteration "
     << d.max_iteration << " interval " << d.interval << " held-out-ratio " << d.held_out_ratio
     << " (0: 0.1) seed " << d.random_seed << " convergence " << d.convergence_threshold
     << "\n";
}

ammsb_graph_buf* load_graph(const Cli& c) {
  ammsb_graph_buf* g = nullptr;
  if (c.input_class == "relativity") {
    if (c.input_file.empty()) throw IOError("no input file (-f)");
    if (c.compressed) throw IOError("compressed input is not supported");
    if (ammsb_read_relativity(c.input_file.c_str(), c.contiguous ? 1 : 0, &g) != AMMSB_OK)
      throw IOError("cannot read " + c.input_file);
    return g;
  }
  if (c.input_class == "synthetic") {
    ammsb_gen_params p{};
    p.n = 5000; p.k_true = 50; p.zipf_s = 1.5; p.size_min = 10; p.size_max = 500;
    p.p1 = 0.7; p.p2 = 0.25; p.intra_degree = 4.0; p.background_frac = 0.1; p.seed = 0;
    std::stringstream ss(c.input_file);
    std::string kv;
    while (std::getline(ss, kv, ',')) {
      if (kv.empty()) continue;
      const size_t eq = kv.find('=');
      if (eq == std::string::npos) throw OptionError("synthetic parameter without '=': " + kv);
      const std::string k = kv.substr(0, eq), v = kv.substr(eq + 1);
      if (k == "n") p.n = (int64_t)parse_size_t(v);
      else if (k == "k_true") p.k_true = (int64_t)parse_size_t(v);
      else if (k == "zipf_s") p.zipf_s = parse_double(v);
      else if (k == "size_min") p.size_min = (int64_t)parse_size_t(v);
      else if (k == "size_max") p.size_max = (int64_t)parse_size_t(v);
      else if (k == "p1") p.p1 = parse_double(v);
      else if (k == "p2") p.p2 = parse_double(v);
      else if (k == "intra_degree") p.intra_degree = parse_double(v);
      else if (k == "background_frac") p.background_frac = parse_double(v);
      else if (k == "seed") p.seed = (uint32_t)parse_size_t(v);
      else throw OptionError("unknown synthetic parameter " + k);
    }
    if (ammsb_generate_graph(&p, &g) != AMMSB_OK) throw IOError("graph generation failed");
    return g;
  }
  throw IOError("unsupported input class '" + c.input_class +
                "' (relativity, synthetic or preprocessed)");
}

}  // namespace

int main(int argc, char* argv[]) {
  std::cout << "Command line: ";
  for (int i = 0; i < argc; ++i) std::cout << argv[i] << " ";
  std::cout << std::endl;
  std::vector<std::string> args(argv + 1, argv + argc);
  for (const auto& a : args)
    if (a == "--help") {
      print_help(std::cout);
      return 0;
    }
  Cli cli;
  ammsb_graph_buf* g = nullptr;
  ammsb_split_buf* split = nullptr;
  ammsb_handle* h = nullptr;
  int status = 0;
  try {
    cli.parse(args);
    for (const auto& r : cli.remains) std::cerr << "ignored argument: " << r << std::endl;
    double ratio = cli.o.held_out_ratio;
    if (ratio == 0.0) {
      ratio = 0.1;
      std::cerr << "Set held_out_ratio to default " << ratio << std::endl;
    }
    if (cli.input_class == "preprocessed") {  // network.cc:49-65
      if (cli.input_file.empty()) throw IOError("no input directory (-f)");
      double saved_ratio = 0.0;
      if (ammsb_load_preprocessed(cli.input_file.c_str(), &g, &split, &saved_ratio) != AMMSB_OK)
        throw IOError("cannot read the preprocessed network in " + cli.input_file);
      ammsb_graph gv;
      ammsb_edge_set hv, tv;
      ammsb_graph_view(g, &gv);
      ammsb_split_view(split, &hv, &tv);
      const int64_t want = (int64_t)(ratio * (double)(gv.row_ptr[gv.n] / 2));
      if (hv.count != 2 * (want / 2))
        std::cerr << "WARNING: Expect held-out size " << want << ", get " << hv.count << std::endl;
    } else {
      g = load_graph(cli);
      if (ammsb_make_held_out(g, ratio, (uint32_t)cli.o.random_seed, &split) != AMMSB_OK)
        throw IOError("held-out construction failed");
    }
    cli.o.held_out_ratio = ratio;
    ammsb_graph graph;
    ammsb_edge_set held, test;
    ammsb_graph_view(g, &graph);
    ammsb_split_view(split, &held, &test);
    if (!cli.save_network.empty() &&  // the reference's preprocessing tool, --save
        ammsb_save_preprocessed(&graph, &held, &test, ratio, cli.save_network.c_str()) != AMMSB_OK)
      throw IOError("cannot save the network into " + cli.save_network);
    std::cout << "start MCMC stochastical" << std::endl;
    if (ammsb_create(&cli.o, &graph, &held, &test, &h) != AMMSB_OK) {
      std::cerr << "MCMC error: " << ammsb_create_error() << std::endl;
      status = 1;
    } else {
      ammsb_options r;
      ammsb_get_options(h, &r);
      const double E = (double)graph.row_ptr[graph.n] / 2.0;
      const double N = (double)graph.n;
      // Learner::info (learner.cc:103-118), sampler_stochastic_info (cc:81-88)
      std::cerr << "N " << graph.n << " E " << (int64_t)E << " link ratio "
                << E / (N * (N - 1) / 2.0) << " K " << r.K << std::endl;
      std::cerr << "minibatch size " << r.mini_batch_size << " epsilon " << r.epsilon
                << " alpha " << r.alpha << " iterations " << r.max_iteration << " convergence "
                << r.convergence_threshold << std::endl;
      std::cerr << "num_node_sample " << r.num_node_sample << std::endl;
      std::cerr << "a " << r.a << " b " << r.b << " c " << r.c << " eta (" << r.eta0 << ","
                << r.eta1 << ")" << std::endl;
      double ppx = 0.0;
      const int rc0 = cli.resume_path.empty()
                          ? ammsb_init_state(h)
                          : ammsb_load_checkpoint(h, cli.resume_path.c_str());
      if (rc0 != AMMSB_OK || ammsb_run(h, &ppx) != AMMSB_OK) {
        std::cerr << "MCMC error: " << ammsb_last_error(h) << std::endl;
        status = 1;
      } else if (!cli.save_path.empty() &&
                 ammsb_save_checkpoint(h, cli.save_path.c_str()) != AMMSB_OK) {
        std::cerr << "IO error: " << ammsb_last_error(h) << std::endl;
        status = 33;
      }
    }
  } catch (const IOError& e) {
    std::cerr << "IO error: " << e.what() << std::endl;
    status = 33;
  } catch (const OptionError& e) {
    std::cerr << "Option error: " << e.what() << std::endl;
    status = 33;
  }
  if (h) ammsb_destroy(h);
  if (split) ammsb_split_free(split);
  if (g) ammsb_graph_free(g);
  return status;
}
