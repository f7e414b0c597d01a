// ref_harness.cc -- C entry points over the reference's own sequential
// sampler, compiled from the reference sources (c++/src/mcmc/...) by
// oracle/ref/build_ref.py into oracle/_ref/libammsb_ref.so.
//
// TEST INFRASTRUCTURE ONLY: used to pin the CPU oracle (and through it the
// CUDA path) to the reference's arithmetic, and by bench.py's reference arm
// to time the reference's run() loop.  Nothing here is part of the product.
//
// A subclass of mcmc::learning::MCMCSamplerStochastic exposes its protected
// steps: update_phi (mcmc_sampler_stochastic.cc:269-313), update_beta
// (cc:200-267), cal_perplexity_held_out (learner.cc:128, 138-183), the
// minibatch and neighbour samplers, and the state vectors.  Noise draws are
// reproduced by copying the sampler's Random object before the call: the
// copy yields exactly the normals the call will consume.
#include <cstring>
#include <string>
#include <vector>

#include "mcmc/learning/mcmc_sampler_stochastic.h"
#include "mcmc/preprocess/netscience.h"

namespace mcmc {
namespace preprocess {
// The XML reader is not built (no tinyxml2); the oracle only feeds text.
NetScience::NetScience(const std::string& filename) : DataSet(filename) {}
NetScience::~NetScience() {}
const mcmc::Data* NetScience::process() {
  throw MCMCException("netscience input is not part of the oracle build");
}
}  // namespace preprocess
}  // namespace mcmc

namespace {

using mcmc::Edge;
using mcmc::Float;
using mcmc::Vertex;

class RefSampler : public mcmc::learning::MCMCSamplerStochastic {
 public:
  explicit RefSampler(const mcmc::Options& o) : MCMCSamplerStochastic(o) {}

  int64_t num_nodes() const { return N; }
  int64_t num_k() const { return K; }
  int64_t num_edges() const { return network.get_num_linked_edges(); }
  int64_t nns() const { return num_node_sample; }
  int64_t mbs() const { return mini_batch_size; }
  const mcmc::EdgeMap& held_out() const { return network.get_held_out_set(); }
  const mcmc::EdgeMap& test_set() const { return network.get_test_set(); }
  const mcmc::NetworkGraph& graph() const { return network.get_linked_edges(); }

  void get_state(float* phi_out, float* pi_out, float* theta_out, float* beta_out) const {
    for (int64_t i = 0; i < N; ++i)
      for (int64_t k = 0; k < (int64_t)K; ++k) {
        if (phi_out) phi_out[i * K + k] = phi[i][k];
        if (pi_out) pi_out[i * K + k] = pi[i][k];
      }
    for (int64_t k = 0; k < (int64_t)K; ++k) {
      if (theta_out) {
        theta_out[2 * k] = theta[k][0];
        theta_out[2 * k + 1] = theta[k][1];
      }
      if (beta_out) beta_out[k] = beta[k];
    }
  }

  // phi as given, pi = normalize(phi) (cc:162-166), beta from theta (cc:262-266)
  void set_state(const float* phi_in, const float* theta_in) {
    for (int64_t i = 0; i < N; ++i) {
      for (int64_t k = 0; k < (int64_t)K; ++k) phi[i][k] = phi_in[i * K + k];
      mcmc::np::normalize(&pi[i], phi[i]);
    }
    for (int64_t k = 0; k < (int64_t)K; ++k) {
      theta[k][0] = theta_in[2 * k];
      theta[k][1] = theta_in[2 * k + 1];
    }
    std::vector<std::vector<Float> > temp(theta.size(), std::vector<Float>(2));
    mcmc::np::row_normalize(&temp, theta);
    for (int64_t k = 0; k < (int64_t)K; ++k) beta[k] = temp[k][1];
  }

  void set_step(uint64_t s) { step_count = s; }

  // a fresh random stream for the draws from here on (learner.cc:47-59
  // seeds rng_[i] with (seed + 1 + i, seed)); the held-out set and the state
  // already drawn stay as they are
  void reseed(unsigned int s) {
    delete rng_[0];
    rng_[0] = new mcmc::Random::Random(s + 1, s, false);
  }
  uint64_t get_step() const { return step_count; }
  float eps_t() { return get_eps_t(); }

  // one update_phi call; returns the neighbour set's iteration order and
  // the noise the call draws
  void call_update_phi(Vertex node, const int32_t* nbrs, int32_t n, float eps, int32_t* order,
                       float* noise, float* phi_out) {
    mcmc::NeighborSet set;
    for (int32_t q = 0; q < n; ++q) set.insert(nbrs[q]);
    int32_t q = 0;
    for (auto v : set) order[q++] = v;
    mcmc::Random::Random copy(*rng_[0]);
    std::vector<Float> nz = copy.randn(K);
    for (int64_t k = 0; k < (int64_t)K; ++k) noise[k] = nz[k];
    update_phi(node, set, eps);
    for (int64_t k = 0; k < (int64_t)K; ++k) phi_out[k] = phi[node][k];
  }

  void call_update_beta(const int32_t* ea, const int32_t* eb, int32_t n, float scale,
                        int32_t* order_a, int32_t* order_b, float* noise, float* theta_out,
                        float* beta_out) {
    mcmc::MinibatchSet mb;
    for (int32_t q = 0; q < n; ++q) mb.insert(Edge(std::min(ea[q], eb[q]), std::max(ea[q], eb[q])));
    int32_t q = 0;
    for (auto& e : mb) {
      order_a[q] = e.first;
      order_b[q] = e.second;
      ++q;
    }
    mcmc::Random::Random copy(*rng_[0]);
    auto nz = copy.randn(K, 2);
    for (int64_t k = 0; k < (int64_t)K; ++k) {
      noise[2 * k] = nz[k][0];
      noise[2 * k + 1] = nz[k][1];
    }
    update_beta(mb, scale);
    get_state(nullptr, nullptr, theta_out, beta_out);
  }

  float call_perplexity(float* ppx_out) {
    float v = cal_perplexity_held_out();
    for (size_t e = 0; e < ppx_per_heldout_edge_.size(); ++e) ppx_out[e] = ppx_per_heldout_edge_[e];
    return v;
  }

  int sample_minibatch(int32_t* ea, int32_t* eb, int32_t cap, int32_t* n_edges, float* scale) {
    mcmc::EdgeSample es = network.sample_mini_batch(mini_batch_size, strategy);
    int32_t q = 0;
    for (auto& e : *es.first) {
      if (q >= cap) {
        delete es.first;
        return -2;
      }
      ea[q] = e.first;
      eb[q] = e.second;
      ++q;
    }
    *n_edges = q;
    *scale = es.second;
    delete es.first;
    return 0;
  }

  void sample_neighbors(Vertex node, int32_t* out) {
    mcmc::NeighborSet set;
    sample_neighbor_nodes(&set, num_node_sample, node, rng_[0]);
    int32_t q = 0;
    for (auto v : set) out[q++] = v;
  }

  void run_iterations(int64_t n, int64_t interval_override) {
    max_iteration = step_count + n;
    if (interval_override > 0) interval = interval_override;
    run();
  }
};

thread_local std::string g_err;

template <class F>
int guarded(F f) {
  try {
    f();
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

void dump_set(const mcmc::EdgeMap& s, int32_t* a, int32_t* b, uint8_t* y) {
  int64_t q = 0;
  for (auto& kv : s) {
    a[q] = kv.first.first;
    b[q] = kv.first.second;
    y[q] = kv.second ? 1 : 0;
    ++q;
  }
}

}  // namespace

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

// Options(argv) then init(): LoadNetwork (graph from the input file, held-out
// and test sets by the reference's RNG) and the gamma initialisation.
void* ref_create(int argc, const char** argv) {
  RefSampler* s = nullptr;
  int rc = guarded([&] {
    std::vector<std::string> args(argv, argv + argc);
    mcmc::Options opts(args);
    s = new RefSampler(opts);
    s->init();
  });
  if (rc) {
    delete s;
    return nullptr;
  }
  return s;
}

void ref_destroy(void* h) { delete static_cast<RefSampler*>(h); }

void ref_sizes(void* h, int64_t* N, int64_t* K, int64_t* E, int64_t* H, int64_t* T, int64_t* nns,
               int64_t* mbs) {
  auto* s = static_cast<RefSampler*>(h);
  *N = s->num_nodes();
  *K = s->num_k();
  *E = s->num_edges();
  *H = (int64_t)s->held_out().size();
  *T = (int64_t)s->test_set().size();
  *nns = s->nns();
  *mbs = s->mbs();
}

void ref_held_out(void* h, int32_t* a, int32_t* b, uint8_t* y) {
  dump_set(static_cast<RefSampler*>(h)->held_out(), a, b, y);
}

void ref_test_set(void* h, int32_t* a, int32_t* b, uint8_t* y) {
  dump_set(static_cast<RefSampler*>(h)->test_set(), a, b, y);
}

// undirected edges (a < b) of the loaded graph; returns the count
int64_t ref_edges(void* h, int32_t* a, int32_t* b) {
  int64_t q = 0;
  for (auto e : static_cast<RefSampler*>(h)->graph()) {
    if (e.first < e.second) {
      a[q] = e.first;
      b[q] = e.second;
      ++q;
    }
  }
  return q;
}

void ref_get_state(void* h, float* phi, float* pi, float* theta, float* beta) {
  static_cast<RefSampler*>(h)->get_state(phi, pi, theta, beta);
}

void ref_set_state(void* h, const float* phi, const float* theta) {
  static_cast<RefSampler*>(h)->set_state(phi, theta);
}

void ref_set_step(void* h, uint64_t s) { static_cast<RefSampler*>(h)->set_step(s); }
void ref_reseed(void* h, uint32_t s) { static_cast<RefSampler*>(h)->reseed(s); }
uint64_t ref_get_step(void* h) { return static_cast<RefSampler*>(h)->get_step(); }
float ref_eps_t(void* h) { return static_cast<RefSampler*>(h)->eps_t(); }

int ref_update_phi(void* h, int32_t node, const int32_t* nbrs, int32_t n, float eps, int32_t* order,
                   float* noise, float* phi_out) {
  return guarded([&] {
    static_cast<RefSampler*>(h)->call_update_phi(node, nbrs, n, eps, order, noise, phi_out);
  });
}

int ref_update_beta(void* h, const int32_t* ea, const int32_t* eb, int32_t n, float scale,
                    int32_t* order_a, int32_t* order_b, float* noise, float* theta_out,
                    float* beta_out) {
  return guarded([&] {
    static_cast<RefSampler*>(h)->call_update_beta(ea, eb, n, scale, order_a, order_b, noise,
                                                  theta_out, beta_out);
  });
}

float ref_perplexity(void* h, float* ppx_out) {
  return static_cast<RefSampler*>(h)->call_perplexity(ppx_out);
}

int ref_sample_minibatch(void* h, int32_t* ea, int32_t* eb, int32_t cap, int32_t* n_edges,
                         float* scale) {
  int rc2 = 0;
  int rc = guarded([&] { rc2 = static_cast<RefSampler*>(h)->sample_minibatch(ea, eb, cap, n_edges, scale); });
  return rc ? rc : rc2;
}

int ref_sample_neighbors(void* h, int32_t node, int32_t* out) {
  return guarded([&] { static_cast<RefSampler*>(h)->sample_neighbors(node, out); });
}

// the reference's run() loop for n more iterations (perplexity every
// `interval` steps if interval > 0, else the configured interval)
int ref_run(void* h, int64_t n, int64_t interval) {
  return guarded([&] { static_cast<RefSampler*>(h)->run_iterations(n, interval); });
}

}  // extern "C"
