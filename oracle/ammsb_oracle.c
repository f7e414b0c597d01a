/*
 * ammsb_oracle.c -- CPU oracle for the a-MMSB SG-MCMC hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path.  The product never
 * links or calls this file.  Built with -ffp-contract=off so that float
 * results do not depend on whether the host compiler fuses multiply-adds.
 *
 * Reference files cited below are paths inside the reference project
 * (c++/src/mcmc/...).
 */
#include "ammsb_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* Learner::MCMC_NONZERO_GUARD, learner.h:26 */
#define NONZERO_GUARD_F 1.0e-24f
#define NONZERO_GUARD_D 1.0e-24

/* ------------------------------------------------------------------------ */
/* Philox4x32-10, Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as  */
/* easy as 1, 2, 3", SC'11.  Multipliers and Weyl key increments as given   */
/* in that paper.                                                           */
/* ------------------------------------------------------------------------ */
#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                          uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
    uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
    k0 += PHILOX_W0;
    k1 += PHILOX_W1;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

static void block(uint32_t seed, uint32_t chain, uint32_t tag, uint32_t entity,
                  uint32_t step, uint64_t blk, uint32_t out[4]) {
  uint32_t ctr[4] = {(uint32_t)blk, entity, step,
                     (tag & 0xffu) | ((uint32_t)(blk >> 32) << 8)};
  uint32_t key[2] = {seed, chain};
  oracle_philox4x32_10(ctr, key, out);
}

uint64_t oracle_draw_u64(uint32_t seed, uint32_t chain, uint32_t tag,
                         uint32_t entity, uint32_t step, uint64_t t) {
  uint32_t o[4];
  block(seed, chain, tag, entity, step, t >> 1, o);
  if (t & 1) return (uint64_t)o[2] | ((uint64_t)o[3] << 32);
  return (uint64_t)o[0] | ((uint64_t)o[1] << 32);
}

/* Uniform integer in [0, n) from a 64-bit draw: floor(x * n / 2^64). */
static inline uint64_t below(uint64_t x, uint64_t n) {
  return (uint64_t)(((unsigned __int128)x * (unsigned __int128)n) >> 64);
}

uint64_t oracle_uniform_below(uint64_t x, uint64_t n) { return below(x, n); }

float oracle_normal(uint32_t seed, uint32_t chain, uint32_t tag,
                    uint32_t entity, uint32_t step, uint64_t idx) {
  uint32_t o[4];
  block(seed, chain, tag, entity, step, idx >> 2, o);
  unsigned pair = (unsigned)((idx >> 1) & 1);
  uint32_t x0 = o[2 * pair], x1 = o[2 * pair + 1];
  /* 24-bit uniforms: exact in float on every platform */
  float u1 = ((float)(x0 >> 8) + 0.5f) * 5.9604644775390625e-08f; /* (0,1) */
  float u2 = (float)(x1 >> 8) * 5.9604644775390625e-08f;          /* [0,1) */
  float r = sqrtf(-2.0f * logf(u1));
  double ang = 2.0 * 3.14159265358979323846 * (double)u2;
  float t = (idx & 1) ? (float)sin(ang) : (float)cos(ang);
  return r * t;
}

/* Marsaglia & Tsang, "A simple method for generating gamma variables",
 * ACM TOMS 26(3), 2000: d = a - 1/3, c = 1/sqrt(9d), accept v = (1+cx)^3
 * with the squeeze 1 - 0.0331 x^4 and the log test.  Shape < 1 via
 * Gamma(a) = Gamma(a+1) U^(1/a).  Double precision throughout. */
double oracle_gamma(uint32_t seed, uint32_t chain, uint32_t tag,
                    uint32_t entity, uint64_t idx, double shape,
                    double scale) {
  uint32_t o[4];
  double a = shape, boost = 1.0;
  if (a < 1.0) {
    block(seed, chain, tag, entity, 0xffffffffu, idx, o);
    double u = ((double)o[3] + 0.5) * 2.3283064365386963e-10;
    boost = pow(u, 1.0 / a);
    a += 1.0;
  }
  double d = a - 1.0 / 3.0;
  double c = 1.0 / sqrt(9.0 * d);
  for (uint32_t attempt = 0; attempt < 64; ++attempt) {
    block(seed, chain, tag, entity, attempt, idx, o);
    double u1 = ((double)o[0] + 0.5) * 2.3283064365386963e-10;
    double u2 = (double)o[1] * 2.3283064365386963e-10;
    double x = sqrt(-2.0 * log(u1)) * cos(2.0 * 3.14159265358979323846 * u2);
    double v = 1.0 + c * x;
    if (v <= 0.0) continue;
    v = v * v * v;
    double u = ((double)o[2] + 0.5) * 2.3283064365386963e-10;
    if (u < 1.0 - 0.0331 * x * x * x * x) return d * v * boost * scale;
    if (log(u) < 0.5 * x * x + d * (1.0 - v + log(v)))
      return d * v * boost * scale;
  }
  return d * boost * scale;
}

/* ------------------------------------------------------------------------ */
/* graph queries: Edge::in(NetworkGraph) (data.h:56-58, 254-276) and        */
/* Edge::in(held_out_map / test_map)                                        */
/* ------------------------------------------------------------------------ */
int oracle_has_edge(const oracle_graph *g, int32_t a, int32_t b) {
  int64_t lo = g->row_ptr[a], hi = g->row_ptr[a + 1];
  while (lo < hi) {
    int64_t mid = lo + (hi - lo) / 2;
    if (g->col[mid] < b)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo < g->row_ptr[a + 1] && g->col[lo] == b;
}

int oracle_is_excluded(const oracle_graph *g, int32_t a, int32_t b) {
  uint32_t lo_v = (uint32_t)(a < b ? a : b), hi_v = (uint32_t)(a < b ? b : a);
  uint64_t key = ((uint64_t)lo_v << 32) | hi_v;
  int64_t lo = 0, hi = g->n_excl;
  while (lo < hi) {
    int64_t mid = lo + (hi - lo) / 2;
    if (g->excl[mid] < key)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo < g->n_excl && g->excl[lo] == key;
}

/* ------------------------------------------------------------------------ */
/* sampling spec                                                            */
/* ------------------------------------------------------------------------ */
float oracle_nonlink_scale(int64_t N, int64_t m, int64_t num_total_edges) {
  /* network.cc:341-342, with Float = float */
  float scale = (float)N * (float)N / (float)m;
  scale = (float)((double)scale * ((double)num_total_edges /
                                   ((double)N * ((double)N - 1.0) / 2.0 -
                                    (double)num_total_edges)));
  return scale;
}

float oracle_eps_t(double a, double b, double c, uint64_t step) {
  return (float)(a * pow(1.0 + (double)step / b, -c));
}

/* get_eps_t as the reference evaluates it with Float = float
 * (mcmc_sampler_stochastic.h:112-115): step_count / b in float, powf. */
float oracle_eps_t_ref(float a, float b, float c, uint64_t step) {
  return a * powf(1.0f + (float)step / b, -c);
}

#define NONLINK_CAND_CAP(m) (64 * (int64_t)(m) + 4096)
#define LINK_ATTEMPT_CAP 4096

static int in_list(const int32_t *list, int32_t n, int32_t v) {
  for (int32_t i = 0; i < n; ++i)
    if (list[i] == v) return 1;
  return 0;
}

/* stratified_random_node_sampling_nonlinks, network.cc:274-349: a source
 * node v and m distinct partners u with (v,u) not a graph edge, not held-out
 * and not test.  Candidates are scanned in draw order; the first m valid,
 * new ones are kept. */
static int sample_nonlinks(const oracle_graph *g, int64_t m, uint32_t seed,
                           uint32_t chain, uint32_t step, int32_t *ea,
                           int32_t *eb, uint8_t *ey, int32_t max_edges,
                           int32_t *nodes, int32_t max_nodes,
                           oracle_mb_info *info) {
  int64_t N = g->n;
  if (m > max_edges || m + 1 > max_nodes) return -2;
  int32_t v = (int32_t)below(oracle_draw_u64(seed, chain, OR_P_MB_NODE, 0, step, 0),
                              (uint64_t)N);
  nodes[0] = v;
  int32_t count = 0;
  int64_t t = 0;
  /* candidates t = 0, 1, ... in draw order; the first m valid, new ones are
   * kept; the scan gives up when NONLINK_CAND_CAP(m) candidates are used */
  while (count < m) {
    if (t >= NONLINK_CAND_CAP(m)) return -1;
    int32_t u = (int32_t)below(oracle_draw_u64(seed, chain, OR_P_MB_CAND, 0, step,
                                               (uint64_t)t),
                               (uint64_t)N);
    t++;
    if (u == v) continue;
    if (oracle_has_edge(g, v, u) || oracle_is_excluded(g, v, u)) continue;
    if (in_list(nodes + 1, count, u)) continue;
    nodes[count + 1] = u;
    ea[count] = 0;
    eb[count] = count + 1;
    ey[count] = 0;
    count++;
  }
  info->n_edges = count;
  info->n_nodes = count + 1;
  info->rounds = (int32_t)(t < 0x7fffffff ? t : 0x7fffffff); /* candidates used */
  return 0;
}

/* stratified_random_node_sampling_links, network.cc:355-407 with
 * sampler.max-source = 1: all training edges of one random node, redrawn
 * while that set is empty; scale = N. */
static int sample_links(const oracle_graph *g, uint32_t seed, uint32_t chain,
                        uint32_t step, int32_t *ea, int32_t *eb, uint8_t *ey,
                        int32_t max_edges, int32_t *nodes, int32_t max_nodes,
                        oracle_mb_info *info) {
  int64_t N = g->n;
  for (int32_t attempt = 0; attempt < LINK_ATTEMPT_CAP; ++attempt) {
    int32_t v = (int32_t)below(oracle_draw_u64(seed, chain, OR_P_MB_NODE, 0, step,
                                               (uint64_t)attempt),
                               (uint64_t)N);
    int32_t count = 0;
    for (int64_t p = g->row_ptr[v]; p < g->row_ptr[v + 1]; ++p) {
      int32_t u = g->col[p];
      if (oracle_is_excluded(g, v, u)) continue;
      if (count >= max_edges || count + 2 > max_nodes) return -2;
      nodes[count + 1] = u;
      ea[count] = 0;
      eb[count] = count + 1;
      ey[count] = 1;
      count++;
    }
    if (count > 0) {
      nodes[0] = v;
      info->n_edges = count;
      info->n_nodes = count + 1;
      info->rounds = attempt + 1;
      return 0;
    }
  }
  return -1;
}

/* Slot of vertex x among nodes[0 .. *n), appended when new (first
 * appearance order); -1 when nodes[] is full. */
static int32_t node_slot(int32_t *nodes, int32_t *n, int32_t max_nodes,
                         int32_t x) {
  for (int32_t i = 0; i < *n; ++i)
    if (nodes[i] == x) return i;
  if (*n >= max_nodes) return -1;
  nodes[*n] = x;
  return (*n)++;
}

/* stratified_random_node_sampling_links with sampler.max-source = S > 1,
 * network.cc:355-407: up to S random sources per attempt; from the second
 * on, a source whose degree would take the set past m ends the attempt;
 * the training edges of each source are added once each (an edge between
 * two sources is kept from the earlier one; a repeated source adds
 * nothing); redrawn while empty.  Source s of attempt a is draw a*S + s.
 * Nodes are numbered by first appearance, source before partner, so S = 1
 * gives the layout of sample_links.  scale = num_total_edges / |set|. */
static int sample_links_multi(const oracle_graph *g, int64_t m, int64_t S,
                              int64_t num_total_edges, uint32_t seed,
                              uint32_t chain, uint32_t step, int32_t *ea,
                              int32_t *eb, uint8_t *ey, int32_t max_edges,
                              int32_t *nodes, int32_t max_nodes,
                              oracle_mb_info *info) {
  int64_t N = g->n;
  int32_t *srcs = (int32_t *)malloc(sizeof(int32_t) * (size_t)S);
  for (int32_t attempt = 0; attempt < LINK_ATTEMPT_CAP; ++attempt) {
    int32_t count = 0, n_nodes = 0;
    for (int64_t s = 0; s < S; ++s) {
      int32_t v = (int32_t)below(oracle_draw_u64(seed, chain, OR_P_MB_NODE, 0, step,
                                                 (uint64_t)attempt * (uint64_t)S + (uint64_t)s),
                                 (uint64_t)N);
      int64_t deg = g->row_ptr[v + 1] - g->row_ptr[v];
      if (s > 0 && count + deg > m) break;
      int dup = in_list(srcs, (int32_t)s, v);
      srcs[s] = v;
      if (dup) continue;
      for (int64_t p = g->row_ptr[v]; p < g->row_ptr[v + 1]; ++p) {
        int32_t u = g->col[p];
        if (oracle_is_excluded(g, v, u)) continue;
        if (in_list(srcs, (int32_t)s, u)) continue;
        if (count >= max_edges) { free(srcs); return -2; }
        int32_t a = node_slot(nodes, &n_nodes, max_nodes, v);
        int32_t b = node_slot(nodes, &n_nodes, max_nodes, u);
        if (a < 0 || b < 0) { free(srcs); return -2; }
        ea[count] = a;
        eb[count] = b;
        ey[count] = 1;
        count++;
      }
    }
    if (count > 0) {
      free(srcs);
      info->n_edges = count;
      info->n_nodes = n_nodes;
      info->rounds = attempt + 1;
      info->scale = (float)num_total_edges / (float)count;
      return 0;
    }
  }
  free(srcs);
  return -1;
}

/* random_edge_sampling, network.cc:237-268: m distinct training edges.
 * Candidates t = 0, 1, ... are entries q of the symmetric CSR (each edge
 * appears twice, as in the reference's linked_edges), q uniform in [0, 2E);
 * the entry (a, b) is kept when a < b, (a, b) is neither held-out nor test
 * and not kept already.  When m >= E - |held-out| - |test| the whole
 * training set is the minibatch (sample_full_training_set, :215-234), in CSR
 * order.  Nodes are numbered by first appearance over (a0, b0, a1, b1, ...);
 * scale = (N - 1) N / 2 / |set| (double, then float). */
static int sample_random_edge(const oracle_graph *g, int64_t m, uint32_t seed,
                              uint32_t chain, uint32_t step, int32_t *ea,
                              int32_t *eb, uint8_t *ey, int32_t max_edges,
                              int32_t *nodes, int32_t max_nodes,
                              oracle_mb_info *info) {
  const int64_t N = g->n, E2 = g->row_ptr[N], E = E2 / 2;
  int32_t count = 0, n_nodes = 0;
  if (m >= E - g->n_excl) {
    for (int32_t a = 0; a < N; ++a)
      for (int64_t q = g->row_ptr[a]; q < g->row_ptr[a + 1]; ++q) {
        int32_t b = g->col[q];
        if (a >= b || oracle_is_excluded(g, a, b)) continue;
        if (count >= max_edges) return -2;
        int32_t sa = node_slot(nodes, &n_nodes, max_nodes, a);
        int32_t sb = node_slot(nodes, &n_nodes, max_nodes, b);
        if (sa < 0 || sb < 0) return -2;
        ea[count] = sa;
        eb[count] = sb;
        ey[count] = 1;
        count++;
      }
    info->rounds = 0;
  } else {
    if (m > max_edges) return -2;
    int64_t *kept = (int64_t *)malloc(sizeof(int64_t) * (size_t)(m > 0 ? m : 1));
    int64_t t = 0;
    while (count < m) {
      if (t >= NONLINK_CAND_CAP(m)) { free(kept); return -1; }
      int64_t q = (int64_t)below(oracle_draw_u64(seed, chain, OR_P_MB_CAND, 0, step,
                                                 (uint64_t)t),
                                 (uint64_t)E2);
      t++;
      int64_t lo = 0, hi = N; /* row of entry q: last a with row_ptr[a] <= q */
      while (hi - lo > 1) {
        int64_t mid = (lo + hi) / 2;
        if (g->row_ptr[mid] <= q) lo = mid; else hi = mid;
      }
      int32_t a = (int32_t)lo, b = g->col[q];
      if (a >= b || oracle_is_excluded(g, a, b)) continue;
      int seen = 0;
      for (int32_t i = 0; i < count && !seen; ++i) seen = kept[i] == q;
      if (seen) continue;
      int32_t sa = node_slot(nodes, &n_nodes, max_nodes, a);
      int32_t sb = node_slot(nodes, &n_nodes, max_nodes, b);
      if (sa < 0 || sb < 0) { free(kept); return -2; }
      kept[count] = q;
      ea[count] = sa;
      eb[count] = sb;
      ey[count] = 1;
      count++;
    }
    free(kept);
    info->rounds = (int32_t)(t < 0x7fffffff ? t : 0x7fffffff);
  }
  info->n_edges = count;
  info->n_nodes = n_nodes;
  info->scale = count > 0 ? (float)((double)(N - 1) * (double)N / 2.0 / (double)count) : 0.0f;
  return 0;
}

int oracle_sample_minibatch_ex(const oracle_graph *g, int strategy,
                               int64_t mini_batch_size, int64_t max_source,
                               int64_t num_total_edges, uint32_t seed,
                               uint32_t chain, uint32_t step, int32_t *edge_a,
                               int32_t *edge_b, uint8_t *edge_y,
                               int32_t max_edges, int32_t *nodes,
                               int32_t max_nodes, oracle_mb_info *info) {
  int flag;
  if (strategy == 3) {
    info->flag = 2;
    return sample_random_edge(g, mini_batch_size, seed, chain, step, edge_a,
                              edge_b, edge_y, max_edges, nodes, max_nodes, info);
  }
  if (strategy == 0) {
    /* network.cc:410-421: flag = randint(0, 1) */
    flag = (int)below(oracle_draw_u64(seed, chain, OR_P_MB_FLAG, 0, step, 0), 2u);
  } else if (strategy == 1) {
    flag = 1;
  } else if (strategy == 2) {
    flag = 0;
  } else {
    return -3;
  }
  info->flag = flag;
  if (flag == 0) {
    info->scale = oracle_nonlink_scale(g->n, mini_batch_size, num_total_edges);
    return sample_nonlinks(g, mini_batch_size, seed, chain, step, edge_a,
                           edge_b, edge_y, max_edges, nodes, max_nodes, info);
  }
  if (max_source > 1)
    return sample_links_multi(g, mini_batch_size, max_source, num_total_edges,
                              seed, chain, step, edge_a, edge_b, edge_y,
                              max_edges, nodes, max_nodes, info);
  info->scale = (float)g->n;
  return sample_links(g, seed, chain, step, edge_a, edge_b, edge_y, max_edges,
                      nodes, max_nodes, info);
}

int oracle_sample_minibatch(const oracle_graph *g, int strategy,
                            int64_t mini_batch_size, int64_t num_total_edges,
                            uint32_t seed, uint32_t chain, uint32_t step,
                            int32_t *edge_a, int32_t *edge_b, uint8_t *edge_y,
                            int32_t max_edges, int32_t *nodes,
                            int32_t max_nodes, oracle_mb_info *info) {
  return oracle_sample_minibatch_ex(g, strategy, mini_batch_size, 1,
                                    num_total_edges, seed, chain, step, edge_a,
                                    edge_b, edge_y, max_edges, nodes, max_nodes,
                                    info);
}

/* sample_neighbor_nodes, mcmc_sampler_stochastic.h:87-108: n_out distinct
 * ids, each != node and with (node, id) neither held-out nor test. */
int64_t oracle_sample_neighbors(const oracle_graph *g, int32_t node,
                                int32_t n_out, uint32_t seed, uint32_t chain,
                                uint32_t step, int32_t *out, uint8_t *y) {
  int64_t cap = 64 * (int64_t)n_out + 4096;
  int32_t count = 0;
  int64_t t = 0;
  while (count < n_out) {
    if (t >= cap) return -1;
    int32_t j = (int32_t)below(oracle_draw_u64(seed, chain, OR_P_NBR, (uint32_t)node, step,
                                               (uint64_t)t),
                               (uint64_t)g->n);
    t++;
    if (j == node) continue;
    if (oracle_is_excluded(g, node, j)) continue;
    if (in_list(out, count, j)) continue;
    out[count] = j;
    y[count] = (uint8_t)oracle_has_edge(g, node, j);
    count++;
  }
  return t;
}

/* ------------------------------------------------------------------------ */
/* hot-path arithmetic, in the reference's operation order                  */
/* ------------------------------------------------------------------------ */
#define REAL float
#define SFX(name) name##_f32
#define R(x) x##f
#define RSQRT sqrtf
#define RABS fabsf
#define RLOG logf
#define GUARD NONZERO_GUARD_F
#include "ammsb_oracle_impl.h"
#undef REAL
#undef SFX
#undef R
#undef RSQRT
#undef RABS
#undef RLOG
#undef GUARD

#define REAL double
#define SFX(name) name##_f64
#define R(x) x
#define RSQRT sqrt
#define RABS fabs
#define RLOG log
#define GUARD NONZERO_GUARD_D
#include "ammsb_oracle_impl.h"

/* update_phi gradient only, double (used for the differentiation check). */
void oracle_phi_grad_f64(int32_t K, const double *pi, const double *phi_i,
                         int32_t i, const int32_t *nbrs, const uint8_t *y,
                         int32_t n_nbrs, const double *beta, double epsilon,
                         double *grads) {
  double phi_i_sum = 0.0;
  for (int32_t k = 0; k < K; ++k) phi_i_sum += phi_i[k];
  double *probs = (double *)malloc(sizeof(double) * (size_t)K);
  for (int32_t k = 0; k < K; ++k) grads[k] = 0.0;
  for (int32_t n = 0; n < n_nbrs; ++n) {
    int32_t j = nbrs[n];
    if (j == i) continue;
    double e = y[n] ? epsilon : 1.0 - epsilon;
    double prob_sum = 0.0;
    for (int32_t k = 0; k < K; ++k) {
      double f = y[n] ? (beta[k] - epsilon) : (epsilon - beta[k]);
      probs[k] = pi[(int64_t)i * K + k] * (pi[(int64_t)j * K + k] * f + e);
      prob_sum += probs[k];
    }
    for (int32_t k = 0; k < K; ++k)
      grads[k] += (probs[k] / prob_sum) / phi_i[k] - 1.0 / phi_i_sum;
  }
  free(probs);
}

double oracle_perplexity_f64acc(int32_t K, const float *pi, const int32_t *ha,
                                const int32_t *hb, const uint8_t *hy,
                                int64_t H, const float *beta, float epsilon,
                                float *ppx, uint64_t average_count) {
  double sum = 0.0;
  for (int64_t e = 0; e < H; ++e) {
    float p = oracle_edge_likelihood_f32(K, pi + (int64_t)ha[e] * K,
                                         pi + (int64_t)hb[e] * K, hy[e], beta,
                                         epsilon);
    float cnt = (float)average_count;
    ppx[e] = (ppx[e] * (cnt - 1.0f) + p) / cnt;
    sum += log((double)ppx[e]);
  }
  return H ? -(sum / (double)H) : 0.0;
}

/* ------------------------------------------------------------------------ */
/* one whole iteration, mcmc_sampler_stochastic.cc:93-183 (loop body)       */
/* ------------------------------------------------------------------------ */
/* Edge capacity of one minibatch of the step's strategy (the reference's
 * max_minibatch_edges_for_strategy, network.cc:188-201, plus the full
 * training set of random-edge). */
static int64_t step_max_edges(const oracle_params *p, const oracle_graph *g) {
  int64_t maxdeg = 0;
  for (int64_t v = 0; v < g->n; ++v) {
    int64_t d = g->row_ptr[v + 1] - g->row_ptr[v];
    if (d > maxdeg) maxdeg = d;
  }
  int64_t me = p->mini_batch_size > maxdeg ? p->mini_batch_size : maxdeg;
  if (p->max_source > 1) me = p->mini_batch_size + maxdeg;
  if (p->strategy == 3 && g->row_ptr[g->n] / 2 > me) me = g->row_ptr[g->n] / 2;
  return me > 0 ? me : 1;
}

int oracle_step_f32(const oracle_params *p, const oracle_graph *g,
                    uint32_t step, float *pi, float *phi, float *theta,
                    float *beta, oracle_mb_info *info) {
  const int32_t K = p->K;
  int64_t max_edges = step_max_edges(p, g);
  int32_t *ea = (int32_t *)malloc(sizeof(int32_t) * (size_t)max_edges);
  int32_t *eb = (int32_t *)malloc(sizeof(int32_t) * (size_t)max_edges);
  uint8_t *ey = (uint8_t *)malloc((size_t)max_edges);
  int32_t *nodes = (int32_t *)malloc(sizeof(int32_t) * (size_t)(2 * max_edges + 1));
  int rc = oracle_sample_minibatch_ex(g, p->strategy, p->mini_batch_size,
                                      p->max_source, p->num_total_edges, p->seed,
                                      p->chain, step, ea, eb, ey, (int32_t)max_edges,
                                      nodes, (int32_t)(2 * max_edges + 1), info);
  if (rc != 0) {
    free(ea); free(eb); free(ey); free(nodes);
    return rc;
  }
  float eps_t = oracle_eps_t(p->a, p->b, p->c, step);
  int32_t n_out = (int32_t)p->num_node_sample + 1;
  int32_t *nb = (int32_t *)malloc(sizeof(int32_t) * (size_t)n_out);
  uint8_t *ny = (uint8_t *)malloc((size_t)n_out);
  float *noise = (float *)malloc(sizeof(float) * (size_t)K);
  for (int32_t s = 0; s < info->n_nodes; ++s) {
    int32_t i = nodes[s];
    if (oracle_sample_neighbors(g, i, n_out, p->seed, p->chain, step, nb, ny) <
        0) {
      rc = -4;
      break;
    }
    for (int32_t k = 0; k < K; ++k)
      noise[k] = oracle_normal(p->seed, p->chain, OR_P_PHI_NOISE, (uint32_t)i,
                               step, (uint64_t)k);
    /* phi[i] is read only by node i itself, so updating it in place keeps
     * the Jacobi semantics; pi is untouched until every node is done. */
    oracle_update_phi_f32(K, pi, phi + (int64_t)i * K, i, nb, ny, n_out, beta,
                          p->alpha, p->epsilon, eps_t, p->N, p->num_node_sample,
                          noise);
  }
  if (rc == 0) {
    for (int32_t s = 0; s < info->n_nodes; ++s) {
      int32_t i = nodes[s];
      oracle_normalize_f32(K, phi + (int64_t)i * K, pi + (int64_t)i * K);
    }
    int32_t *va = (int32_t *)malloc(sizeof(int32_t) * (size_t)info->n_edges);
    int32_t *vb = (int32_t *)malloc(sizeof(int32_t) * (size_t)info->n_edges);
    for (int32_t e = 0; e < info->n_edges; ++e) {
      va[e] = nodes[ea[e]];
      vb[e] = nodes[eb[e]];
    }
    float *tn = (float *)malloc(sizeof(float) * 2 * (size_t)K);
    for (int32_t k = 0; k < 2 * K; ++k)
      tn[k] = oracle_normal(p->seed, p->chain, OR_P_THETA_NOISE, 0, step,
                            (uint64_t)k);
    float eta[2] = {p->eta0, p->eta1};
    oracle_update_beta_f32(K, pi, va, vb, ey, info->n_edges, theta, beta, eta,
                           p->epsilon, eps_t, info->scale, tn, NULL);
    free(tn);
    free(va);
    free(vb);
  }
  free(noise);
  free(nb);
  free(ny);
  free(ea);
  free(eb);
  free(ey);
  free(nodes);
  return rc;
}

int oracle_step_f32_threads(const oracle_params *p, const oracle_graph *g,
                            uint32_t step, float *pi, float *phi, float *theta,
                            float *beta, oracle_mb_info *info, int threads,
                            int64_t max_edges) {
  const int32_t K = p->K;
  if (max_edges <= 0) max_edges = step_max_edges(p, g);
  int32_t *ea = (int32_t *)malloc(sizeof(int32_t) * (size_t)max_edges);
  int32_t *eb = (int32_t *)malloc(sizeof(int32_t) * (size_t)max_edges);
  uint8_t *ey = (uint8_t *)malloc((size_t)max_edges);
  int32_t *nodes = (int32_t *)malloc(sizeof(int32_t) * (size_t)(2 * max_edges + 1));
  int rc = oracle_sample_minibatch_ex(g, p->strategy, p->mini_batch_size,
                                      p->max_source, p->num_total_edges, p->seed,
                                      p->chain, step, ea, eb, ey, (int32_t)max_edges,
                                      nodes, (int32_t)(2 * max_edges + 1), info);
  if (rc != 0) {
    free(ea); free(eb); free(ey); free(nodes);
    return rc;
  }
  const float eps_t = oracle_eps_t(p->a, p->b, p->c, step);
  const int32_t n_out = (int32_t)p->num_node_sample + 1;
  const int32_t n_nodes = info->n_nodes;
  int failed = 0;
#pragma omp parallel num_threads(threads > 0 ? threads : 1) reduction(| : failed)
  {
    int32_t *nb = (int32_t *)malloc(sizeof(int32_t) * (size_t)n_out);
    uint8_t *ny = (uint8_t *)malloc((size_t)n_out);
    float *noise = (float *)malloc(sizeof(float) * (size_t)K);
#pragma omp for schedule(dynamic, 4)
    for (int32_t s = 0; s < n_nodes; ++s) {
      const int32_t i = nodes[s];
      if (oracle_sample_neighbors(g, i, n_out, p->seed, p->chain, step, nb, ny) < 0) {
        failed = 1;
        continue;
      }
      for (int32_t k = 0; k < K; ++k)
        noise[k] = oracle_normal(p->seed, p->chain, OR_P_PHI_NOISE, (uint32_t)i,
                                 step, (uint64_t)k);
      oracle_update_phi_f32(K, pi, phi + (int64_t)i * K, i, nb, ny, n_out, beta,
                            p->alpha, p->epsilon, eps_t, p->N, p->num_node_sample,
                            noise);
    }
    free(noise);
    free(nb);
    free(ny);
  }
  if (failed) rc = -4;
  if (rc == 0) {
    for (int32_t s = 0; s < n_nodes; ++s) {
      const int32_t i = nodes[s];
      oracle_normalize_f32(K, phi + (int64_t)i * K, pi + (int64_t)i * K);
    }
    int32_t *va = (int32_t *)malloc(sizeof(int32_t) * (size_t)(info->n_edges + 1));
    int32_t *vb = (int32_t *)malloc(sizeof(int32_t) * (size_t)(info->n_edges + 1));
    for (int32_t e = 0; e < info->n_edges; ++e) {
      va[e] = nodes[ea[e]];
      vb[e] = nodes[eb[e]];
    }
    float *tn = (float *)malloc(sizeof(float) * 2 * (size_t)K);
    for (int32_t k = 0; k < 2 * K; ++k)
      tn[k] = oracle_normal(p->seed, p->chain, OR_P_THETA_NOISE, 0, step,
                            (uint64_t)k);
    const float eta[2] = {p->eta0, p->eta1};
    oracle_update_beta_f32(K, pi, va, vb, ey, info->n_edges, theta, beta, eta,
                           p->epsilon, eps_t, info->scale, tn, NULL);
    free(tn);
    free(va);
    free(vb);
  }
  free(ea);
  free(eb);
  free(ey);
  free(nodes);
  return rc;
}

/* The same iteration in double: identical draws (the minibatch, the
 * neighbour sets and the float normals of the Philox spec, widened), double
 * arithmetic throughout, eps_t in double.  The FP64 trajectory reference of
 * the FP32 and BF16 device paths. */
int oracle_step_f64(const oracle_params *p, const oracle_graph *g,
                    uint32_t step, double *pi, double *phi, double *theta,
                    double *beta, oracle_mb_info *info) {
  const int32_t K = p->K;
  int64_t max_edges = step_max_edges(p, g);
  int32_t *ea = (int32_t *)malloc(sizeof(int32_t) * (size_t)max_edges);
  int32_t *eb = (int32_t *)malloc(sizeof(int32_t) * (size_t)max_edges);
  uint8_t *ey = (uint8_t *)malloc((size_t)max_edges);
  int32_t *nodes = (int32_t *)malloc(sizeof(int32_t) * (size_t)(2 * max_edges + 1));
  int rc = oracle_sample_minibatch_ex(g, p->strategy, p->mini_batch_size,
                                      p->max_source, p->num_total_edges, p->seed,
                                      p->chain, step, ea, eb, ey, (int32_t)max_edges,
                                      nodes, (int32_t)(2 * max_edges + 1), info);
  if (rc != 0) {
    free(ea); free(eb); free(ey); free(nodes);
    return rc;
  }
  const double eps_t = p->a * pow(1.0 + (double)step / p->b, -p->c);
  const int32_t n_out = (int32_t)p->num_node_sample + 1;
  int32_t *nb = (int32_t *)malloc(sizeof(int32_t) * (size_t)n_out);
  uint8_t *ny = (uint8_t *)malloc((size_t)n_out);
  double *noise = (double *)malloc(sizeof(double) * (size_t)K);
  for (int32_t s = 0; s < info->n_nodes && rc == 0; ++s) {
    const int32_t i = nodes[s];
    if (oracle_sample_neighbors(g, i, n_out, p->seed, p->chain, step, nb, ny) < 0) {
      rc = -4;
      break;
    }
    for (int32_t k = 0; k < K; ++k)
      noise[k] = (double)oracle_normal(p->seed, p->chain, OR_P_PHI_NOISE,
                                       (uint32_t)i, step, (uint64_t)k);
    oracle_update_phi_f64(K, pi, phi + (int64_t)i * K, i, nb, ny, n_out, beta,
                          (double)p->alpha, (double)p->epsilon, eps_t, p->N,
                          p->num_node_sample, noise);
  }
  if (rc == 0) {
    for (int32_t s = 0; s < info->n_nodes; ++s) {
      const int32_t i = nodes[s];
      oracle_normalize_f64(K, phi + (int64_t)i * K, pi + (int64_t)i * K);
    }
    int32_t *va = (int32_t *)malloc(sizeof(int32_t) * (size_t)(info->n_edges + 1));
    int32_t *vb = (int32_t *)malloc(sizeof(int32_t) * (size_t)(info->n_edges + 1));
    for (int32_t e = 0; e < info->n_edges; ++e) {
      va[e] = nodes[ea[e]];
      vb[e] = nodes[eb[e]];
    }
    double *tn = (double *)malloc(sizeof(double) * 2 * (size_t)K);
    for (int32_t k = 0; k < 2 * K; ++k)
      tn[k] = (double)oracle_normal(p->seed, p->chain, OR_P_THETA_NOISE, 0,
                                    step, (uint64_t)k);
    const double eta[2] = {(double)p->eta0, (double)p->eta1};
    oracle_update_beta_f64(K, pi, va, vb, ey, info->n_edges, theta, beta, eta,
                           (double)p->epsilon, eps_t, (double)info->scale, tn,
                           NULL);
    free(tn);
    free(va);
    free(vb);
  }
  free(noise);
  free(nb);
  free(ny);
  free(ea);
  free(eb);
  free(ey);
  free(nodes);
  return rc;
}
