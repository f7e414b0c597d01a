/*
 * ammsb_oracle.h -- CPU oracle for the a-MMSB SG-MCMC hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the mcmc_for_ammsb_gb300
 * package, its CUDA library, its C-ABI) may link, load or call this code.
 * Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
 * reference legs use it, as the checker.
 *
 * Two kinds of functions live here:
 *   1. Literal restatements of the reference sampler's arithmetic
 *      (mcmc_sampler_stochastic.cc update_phi / update_beta, learner.h
 *      cal_edge_likelihood, learner.cc cal_perplexity), in the reference's
 *      own operation order, in float (the reference's default Float) and in
 *      double (for error statements).
 *   2. The sampling specification of this project: the reference's minibatch
 *      and neighbour semantics (network.cc:274-421, mcmc_sampler_stochastic.h
 *      :87-108) driven by a counter-based Philox4x32-10 stream instead of the
 *      reference's sequential xorshift128+ (random.cc:136-142).  The CUDA
 *      sampler must reproduce these draws bit for bit.
 */
#ifndef AMMSB_ORACLE_H_
#define AMMSB_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Philox4x32-10 (Salmon et al., SC'11) -------------------------------- */
void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                          uint32_t out[4]);

/* Stream tags (counter word 3, low byte). */
enum {
  OR_P_MB_FLAG = 1,
  OR_P_MB_NODE = 2,
  OR_P_MB_CAND = 3,
  OR_P_NBR = 4,
  OR_P_PHI_NOISE = 5,
  OR_P_THETA_NOISE = 6,
  OR_P_PHI_INIT = 7,
  OR_P_THETA_INIT = 8
};

/* 64-bit uniform draw #t of stream (tag, entity, step): two 32-bit words of
 * Philox block t/2, half t%2. */
uint64_t oracle_draw_u64(uint32_t seed, uint32_t chain, uint32_t tag,
                         uint32_t entity, uint32_t step, uint64_t t);

/* Uniform integer in [0, n) from a 64-bit draw x: floor(x * n / 2^64) (the
 * multiply-high map; the reference reduces rand() % range, random.cc:174). */
uint64_t oracle_uniform_below(uint64_t x, uint64_t n);

/* Standard normals of stream (tag, entity, step), element idx: Box-Muller on
 * 24-bit uniforms, four normals per Philox block. */
float oracle_normal(uint32_t seed, uint32_t chain, uint32_t tag,
                    uint32_t entity, uint32_t step, uint64_t idx);

/* Marsaglia-Tsang gamma(shape, scale) draw for element (entity, idx). */
double oracle_gamma(uint32_t seed, uint32_t chain, uint32_t tag,
                    uint32_t entity, uint64_t idx, double shape, double scale);

/* ---- graph queries --------------------------------------------------------*/
typedef struct {
  int64_t n;               /* vertices */
  const int64_t *row_ptr;  /* n+1 */
  const int32_t *col;      /* row_ptr[n], each row sorted ascending */
  const uint64_t *excl;    /* sorted keys (min<<32|max) of held-out + test */
  int64_t n_excl;
} oracle_graph;

int oracle_has_edge(const oracle_graph *g, int32_t a, int32_t b);
int oracle_is_excluded(const oracle_graph *g, int32_t a, int32_t b);

/* ---- sampling spec (Philox-driven restatement of the reference) ----------*/
typedef struct {
  int32_t flag;       /* 0: non-link stratum, 1: link stratum */
  int32_t n_edges;
  int32_t n_nodes;
  float scale;
  int32_t rounds;     /* non-link rounds or link attempts used */
} oracle_mb_info;

/* stratified-random-node (strategy 0), -links (1), -nonlinks (2).
 * edge_a/edge_b/edge_y get n_edges entries (slot of endpoint in nodes[]),
 * nodes gets n_nodes vertex ids; capacities are max_edges / max_nodes.
 * Returns 0 on success, negative on a capped loop or capacity overflow. */
int oracle_sample_minibatch(const oracle_graph *g, int strategy,
                            int64_t mini_batch_size, int64_t num_total_edges,
                            uint32_t seed, uint32_t chain, uint32_t step,
                            int32_t *edge_a, int32_t *edge_b, uint8_t *edge_y,
                            int32_t max_edges, int32_t *nodes,
                            int32_t max_nodes, oracle_mb_info *info);

/* The same with sampler.max-source (network.cc:355-407) for the link
 * stratum, and strategy 3 = random-edge (network.cc:237-268). */
int oracle_sample_minibatch_ex(const oracle_graph *g, int strategy,
                               int64_t mini_batch_size, int64_t max_source,
                               int64_t num_total_edges, uint32_t seed,
                               uint32_t chain, uint32_t step, int32_t *edge_a,
                               int32_t *edge_b, uint8_t *edge_y,
                               int32_t max_edges, int32_t *nodes,
                               int32_t max_nodes, oracle_mb_info *info);

/* n_out distinct neighbours of node (n_out = num_node_sample + 1), each
 * != node and not a held-out/test pair; y[t] = graph membership.
 * Returns number of candidate draws used, negative on cap. */
int64_t oracle_sample_neighbors(const oracle_graph *g, int32_t node,
                                int32_t n_out, uint32_t seed, uint32_t chain,
                                uint32_t step, int32_t *out, uint8_t *y);

/* Scale factors of the two strata (network.cc:341-342, 385-390). */
float oracle_nonlink_scale(int64_t N, int64_t m, int64_t num_total_edges);

/* eps_t = a (1 + t/b)^-c (mcmc_sampler_stochastic.h:112-115), in double then
 * rounded to float. */
float oracle_eps_t(double a, double b, double c, uint64_t step);
/* the reference's own float evaluation of the same formula */
float oracle_eps_t_ref(float a, float b, float c, uint64_t step);

/* ---- hot-path arithmetic, literal restatements --------------------------*/
/* update_phi for one node (mcmc_sampler_stochastic.cc:269-313).
 * pi: N x K row-major (stride K); phi_i: K (updated in place);
 * nbrs: n_nbrs ids in iteration order; y: per neighbour; noise: K. */
void oracle_update_phi_f32(int32_t K, const float *pi, float *phi_i,
                           int32_t i, const int32_t *nbrs, const uint8_t *y,
                           int32_t n_nbrs, const float *beta, float alpha,
                           float epsilon, float eps_t, int64_t N,
                           int64_t num_node_sample, const float *noise);
void oracle_update_phi_f64(int32_t K, const double *pi, double *phi_i,
                           int32_t i, const int32_t *nbrs, const uint8_t *y,
                           int32_t n_nbrs, const double *beta, double alpha,
                           double epsilon, double eps_t, int64_t N,
                           int64_t num_node_sample, const double *noise);

/* The update_phi gradient alone (grads[k] before the SGRLD step). */
void oracle_phi_grad_f64(int32_t K, const double *pi, const double *phi_i,
                         int32_t i, const int32_t *nbrs, const uint8_t *y,
                         int32_t n_nbrs, const double *beta, double epsilon,
                         double *grads);

/* np::normalize (np.h:39-56) */
void oracle_normalize_f32(int32_t K, const float *phi_i, float *pi_i);
void oracle_normalize_f64(int32_t K, const double *phi_i, double *pi_i);

/* update_beta (mcmc_sampler_stochastic.cc:200-267): gradient over the
 * minibatch edges (ea, eb vertex ids, ey), theta step with noise K x 2,
 * beta = theta1 / (theta0 + theta1).  grads_out (K x 2) optional. */
void oracle_update_beta_f32(int32_t K, const float *pi, const int32_t *ea,
                            const int32_t *eb, const uint8_t *ey,
                            int32_t n_edges, float *theta, float *beta,
                            const float *eta, float epsilon, float eps_t,
                            float scale, const float *noise, float *grads_out);
void oracle_update_beta_f64(int32_t K, const double *pi, const int32_t *ea,
                            const int32_t *eb, const uint8_t *ey,
                            int32_t n_edges, double *theta, double *beta,
                            const double *eta, double epsilon, double eps_t,
                            double scale, const double *noise,
                            double *grads_out);

/* The two halves of update_beta: the gradient over the given edges (K x 2,
 * in edge order) and the theta step from a gradient (sums of the halves
 * over disjoint edge sets give the whole minibatch's gradient). */
void oracle_beta_grads_f32(int32_t K, const float *pi, const int32_t *ea,
                           const int32_t *eb, const uint8_t *ey, int32_t n_edges,
                           const float *theta, const float *beta, float epsilon,
                           float *grads);
void oracle_theta_step_f32(int32_t K, float *theta, float *beta, const float *eta,
                           float eps_t, float scale, const float *noise,
                           const float *grads);

/* cal_edge_likelihood (learner.h:100-139) */
float oracle_edge_likelihood_f32(int32_t K, const float *pa, const float *pb,
                                 int y, const float *beta, float epsilon);
double oracle_edge_likelihood_f64(int32_t K, const double *pa,
                                  const double *pb, int y, const double *beta,
                                  double epsilon);

/* cal_perplexity (learner.cc:138-183) over held-out edges (ha, hb, hy) with
 * running averages ppx (updated) and average_count (caller increments).
 * f32: the reference's float accumulation.  f64acc: float likelihoods and
 * float running average (the device's storage types) with the log-sum in
 * double -- the semantics of the CUDA perplexity kernel. */
float oracle_perplexity_f32(int32_t K, const float *pi, const int32_t *ha,
                            const int32_t *hb, const uint8_t *hy, int64_t H,
                            const float *beta, float epsilon, float *ppx,
                            uint64_t average_count);
double oracle_perplexity_f64acc(int32_t K, const float *pi, const int32_t *ha,
                                const int32_t *hb, const uint8_t *hy,
                                int64_t H, const float *beta, float epsilon,
                                float *ppx, uint64_t average_count);
double oracle_perplexity_f64(int32_t K, const double *pi, const int32_t *ha,
                             const int32_t *hb, const uint8_t *hy, int64_t H,
                             const double *beta, double epsilon, double *ppx,
                             uint64_t average_count);

/* ---- whole iteration ---------------------------------------------------*/
typedef struct {
  int32_t K;
  int64_t N;
  int64_t num_total_edges;
  int32_t strategy;
  int64_t mini_batch_size;
  int64_t num_node_sample;
  float alpha, epsilon, eta0, eta1;
  double a, b, c;
  uint32_t seed, chain;
  int64_t max_source; /* sampler.max-source */
} oracle_params;

/* One SG-MCMC iteration at `step` (draws from the Philox spec), float
 * arithmetic in the reference's order: minibatch, neighbours, update_phi
 * (Jacobi: all reads see the old pi), pi normalisation, update_beta.
 * pi/phi: N x K; theta: K x 2 (float, as the reference); beta: K.
 * Returns 0 or a negative sampling error. */
int oracle_step_f32(const oracle_params *p, const oracle_graph *g,
                    uint32_t step, float *pi, float *phi, float *theta,
                    float *beta, oracle_mb_info *info);
/* The same iteration in double (same draws, eps_t in double): the FP64
 * trajectory reference. */
int oracle_step_f64(const oracle_params *p, const oracle_graph *g,
                    uint32_t step, double *pi, double *phi, double *theta,
                    double *beta, oracle_mb_info *info);

/* The same float iteration with the per-node work (neighbour sets,
 * update_phi) spread over `threads` host threads (OpenMP), as the
 * reference's distributed sampler spreads it (distr.cc:1142); results equal
 * oracle_step_f32's bit for bit (Jacobi: each node writes only its own phi
 * row).  max_edges: the strategy's minibatch edge capacity, or <= 0 to
 * compute it from the graph. */
int oracle_step_f32_threads(const oracle_params *p, const oracle_graph *g,
                            uint32_t step, float *pi, float *phi, float *theta,
                            float *beta, oracle_mb_info *info, int threads,
                            int64_t max_edges);

/* ---- workload inputs (ammsb_oracle_graph.c) -------------------------------*/
typedef struct {
  int64_t n, k_true;
  double zipf_s;
  int64_t size_min, size_max;
  double p1, p2, intra_degree, background_frac;
  uint32_t seed;
} oracle_gen_params;

/* Planted-community graph as a symmetric CSR with sorted rows; the arrays
 * are malloc'ed (release with oracle_free).  0 or -1. */
int oracle_generate_graph(const oracle_gen_params *p, int64_t **row_ptr,
                          int32_t **col);
/* p = (ratio * E truncated) / 2: the held-out and the test set each get p
 * links and p non-links. */
int64_t oracle_held_out_pairs(int64_t num_edges, double ratio);
/* Held-out and test sets (2p entries each, caller-allocated). 0 or -1. */
int oracle_make_held_out(int64_t n, const int64_t *row_ptr, const int32_t *col,
                         double ratio, uint32_t seed, int32_t *ha, int32_t *hb,
                         uint8_t *hy, int32_t *ta, int32_t *tb, uint8_t *ty);
/* A Gamma(1, 1) phi (N x K) and its row-normalised pi, on `threads`
 * host threads: the starting state of the benchmark's CPU legs. */
void oracle_init_state_threads(int64_t n, int32_t K, uint32_t seed, float *phi,
                               float *pi, int threads);
void oracle_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
