/*
 * ammsb_gpu.h -- C ABI of the GB300 a-MMSB SG-MCMC sampler (libammsb_gpu.so).
 *
 * The reference has no plugin or FFI surface: its hot path sits behind the
 * C++ class mcmc::learning::MCMCSamplerStochastic (learner.h:45 run(),
 * mcmc_sampler_stochastic.h:72-85), constructed from mcmc::Options
 * (options.h:129-315) and driven by apps/main/main.cc:69-76 as
 *   MCMCSamplerStochastic s(args); s.init(); s.run();
 * This header is that boundary as plain C: a handle owns the sampler state
 * resident in GPU memory; host arrays passed in are borrowed for the call.
 *
 * Conventions
 *   - every function returns AMMSB_OK (0) or a negative AMMSB_E* status;
 *     ammsb_last_error() gives the message.  No C++ exception crosses the ABI
 *     (the reference throws MCMCException, exception.h:12-28).
 *   - a handle is bound to one CUDA device and one stream and is not
 *     thread-safe, like the reference's single-threaded sequential sampler.
 *   - vertex ids are int32 (mcmc::Vertex, data.h:42); edges are unordered
 *     pairs (a, b); sets store a < b as the reference's Edge(min, max).
 */
#ifndef AMMSB_GPU_H_
#define AMMSB_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AMMSB_OK 0
#define AMMSB_E_ARG (-1)       /* invalid argument (InvalidArgumentException) */
#define AMMSB_E_CUDA (-2)      /* CUDA runtime error */
#define AMMSB_E_SAMPLING (-3)  /* a capped rejection loop gave up */
#define AMMSB_E_CAPACITY (-4)  /* minibatch exceeds its buffer (BufferSizeException) */
#define AMMSB_E_STATE (-5)     /* call order / state error */
#define AMMSB_E_UNSUPPORTED (-6)

/* mcmc.strategy values, types.h:11-16 */
#define AMMSB_STRATIFIED_RANDOM_NODE 0
#define AMMSB_STRATIFIED_RANDOM_NODE_LINKS 1
#define AMMSB_STRATIFIED_RANDOM_NODE_NONLINKS 2
#define AMMSB_RANDOM_EDGE 3

/* storage type of pi (GB300 option; the reference stores Float = float) */
#define AMMSB_PI_F32 0
#define AMMSB_PI_BF16 1

/* Element types of the edge log-likelihood and its adjoint. */
#define AMMSB_REAL_F32 0
#define AMMSB_REAL_F64 1

/* The sampler's option surface, options.h:142-185 (mcmc.* flags).  Zero
 * values take the reference's derived defaults at ammsb_create():
 * a := b^-c (options.h:257-259), alpha := 1/K (options.h:260-262),
 * held_out_ratio := 0.1 (learner.cc:88-92), interval := 50 (seq cc:15-19),
 * stats_print_interval := 64Ki (cc:20-24), num_node_sample := N/50 and
 * mini_batch_size := N/10 (cc:35-44). */
typedef struct ammsb_options {
  double alpha;                 /* mcmc.alpha, default 0 (=> 1/K) */
  double eta0;                  /* mcmc.eta0, default 1 */
  double eta1;                  /* mcmc.eta1, default 1 */
  double epsilon;               /* mcmc.epsilon, default 1e-7 */
  double a;                     /* mcmc.a, default 0 (=> b^-c) */
  double b;                     /* mcmc.b, default 1024 */
  double c;                     /* mcmc.c, default 0.5 */
  int64_t K;                    /* mcmc.K, default 300 */
  int64_t mini_batch_size;      /* mcmc.mini-batch-size, default 0 */
  int64_t num_node_sample;      /* mcmc.num-node-sample, default 0 */
  int32_t strategy;             /* mcmc.strategy, default stratified-random-node */
  int64_t sampler_max_source;   /* mcmc.sampler.max-source, default 1 */
  int64_t max_iteration;        /* mcmc.max-iteration, default 10000000 */
  int64_t interval;             /* mcmc.interval, default 0 (=> 50) */
  int64_t stats_print_interval; /* mcmc.stats, default 0 (=> 65536) */
  int64_t num_updates;          /* mcmc.num-updates, default 1000 (unused, kept) */
  double held_out_ratio;        /* mcmc.held-out-ratio, default 0 (=> 0.1) */
  int32_t random_seed;          /* mcmc.seed, default 42 */
  double convergence_threshold; /* mcmc.convergence, default 1e-12 */
  /* GB300 options (no reference counterpart) */
  int32_t pi_dtype;             /* AMMSB_PI_F32 (default) or AMMSB_PI_BF16 */
  int32_t chain;                /* Philox key word 1: independent chain id */
  int32_t device;               /* CUDA device ordinal, default 0 */
  int32_t use_graph;            /* capture the iteration in a CUDA graph (1) */
  int32_t verbose;              /* info lines on stderr like learner.cc:105-120 */
  int32_t pipeline;             /* 1 (default): the draws of the next two
                                   iterations run on a second stream during the
                                   update; 0: run()'s loop order on one stream,
                                   draws then update (cc:126-170) */
} ammsb_options;

/* Undirected graph as symmetric CSR: row v lists the neighbours of v in
 * ascending order; row_ptr[n] = 2E.  Replaces NetworkGraph (data.h:135-313). */
typedef struct ammsb_graph {
  int64_t n;
  const int64_t *row_ptr; /* n + 1 */
  const int32_t *col;     /* row_ptr[n] */
} ammsb_graph;

/* Held-out or test set: EdgeMap{Edge -> bool is_edge} (data.h:131) as
 * arrays; a[i] < b[i]; iteration order is array order. */
typedef struct ammsb_edge_set {
  int64_t count;
  const int32_t *a;
  const int32_t *b;
  const uint8_t *y;
} ammsb_edge_set;

typedef struct ammsb_handle ammsb_handle;

/* Fills the reference defaults of options.h:144-185. */
void ammsb_options_default(ammsb_options *opt);

/* Learner::Learner + Network::Init + Learner::Init + the sampler constructor
 * (learner.cc:13-84, network.cc:31-84, mcmc_sampler_stochastic.cc:9-44):
 * validates options, derives defaults, uploads the graph and the held-out
 * and test sets, allocates the state in GPU memory. */
int ammsb_create(const ammsb_options *opt, const ammsb_graph *graph,
                 const ammsb_edge_set *held_out, const ammsb_edge_set *test,
                 ammsb_handle **out);
void ammsb_destroy(ammsb_handle *h);
const char *ammsb_last_error(const ammsb_handle *h);
/* Message of the last ammsb_create() failure on this thread. */
const char *ammsb_create_error(void);

/* MCMCSamplerStochastic::init (cc:29-79): theta ~ Gamma(eta0, eta1) (K x 2),
 * beta = theta[:,1] / sum, phi ~ Gamma(1, 1) (N x K), pi = row-normalised
 * phi.  Draws follow the Philox streams of ammsb_rng.h. */
int ammsb_init_state(ammsb_handle *h);
/* Loads a given state instead: phi N x K float, theta K x 2 double. */
int ammsb_set_state(ammsb_handle *h, const float *phi, const double *theta);

/* n_iters iterations of the loop body of run() (cc:131-174): minibatch,
 * neighbour sets, update_phi, pi, update_beta, step_count++.  No
 * perplexity.  With use_graph the iterations are launched as CUDA graphs
 * (up to 16 iterations per launch, the draws of the next ones overlapped);
 * the chain is the same bit for bit either way. */
int ammsb_step(ammsb_handle *h, int64_t n_iters);

/* One iteration with every draw supplied by the caller (parity hook):
 * minibatch edges as slots into nodes[] with y, the step's scale, node ids,
 * neighbour ids + y per node (n_nodes x (num_node_sample+1)), phi noise
 * (n_nodes x K), theta noise (K x 2), and the step index used for eps_t.
 * Does not advance the internal step counter. */
int ammsb_step_fed(ammsb_handle *h, uint32_t step, int32_t n_edges,
                   const int32_t *edge_slot_a, const int32_t *edge_slot_b,
                   const uint8_t *edge_y, float scale, int32_t n_nodes,
                   const int32_t *nodes, const int32_t *nbrs,
                   const uint8_t *nbr_y, const float *phi_noise,
                   const float *theta_noise);

/* One rank's phases of a sharded iteration.  They replace the distributed
 * sampler's per-iteration split (mcmc_sampler_stochastic_distr.cc:630-708:
 * minibatch nodes owned by node % ranks, distr.cc:1626-1632; the updated pi
 * rows written to the shared store; the beta gradient summed over ranks,
 * distr.cc:1430-1442): every rank holds all of pi, updates the phi rows of
 * the nodes it owns, and the caller moves rows and sums between ranks.
 *   ammsb_shard_draw    the minibatch and neighbour sets of iteration
 *                       step_count, the same on every rank (they depend only
 *                       on seed, chain and step); ammsb_get_last_minibatch
 *                       reads them;
 *   ammsb_shard_update  update_phi of the owned slots (ascending indices into
 *                       the drawn nodes); writes their new pi rows (FP32,
 *                       n_owned x K) to rows_out;
 *   ammsb_shard_commit  every drawn node's new pi row (FP32, n_nodes x K in
 *                       slot order, gathered from all ranks) committed into
 *                       pi, then the beta-gradient sums R (K x 2: sum of
 *                       f_k / P over the y = 0 and the y = 1 edges) over the
 *                       owned edges (ascending indices into the drawn edges)
 *                       written to R_out;
 *   ammsb_shard_theta   the theta step (update_beta, cc:241-266) from the sums
 *                       added over all ranks; the iteration is done and
 *                       step_count advances.
 * The calls must come in this order; each synchronises the handle's stream.
 * Host arrays throughout.  A single rank that owns every node and edge
 * takes the same iteration as ammsb_step, up to the order in which the
 * beta sums are added. */
int ammsb_shard_draw(ammsb_handle *h);
int ammsb_shard_update(ammsb_handle *h, int32_t n_owned, const int32_t *slots,
                       float *rows_out);
int ammsb_shard_commit(ammsb_handle *h, const float *rows_all,
                       int32_t n_owned_edges, const int32_t *edge_idx,
                       double *R_out);
int ammsb_shard_theta(ammsb_handle *h, const double *R_total);

/* Learner::cal_perplexity_held_out (learner.cc:128, 138-183): running
 * average per held-out edge, -mean log; advances average_count. */
int ammsb_perplexity(ammsb_handle *h, double *out);

/* MCMCSamplerStochastic::run (cc:93-183): perplexity every interval steps
 * (printed in the reference's line format on stdout), convergence test
 * (learner.cc:130-136), until max_iteration.  Returns the last perplexity. */
int ammsb_run(ammsb_handle *h, double *last_perplexity);

/* State readers (host destination arrays). */
int ammsb_get_pi(ammsb_handle *h, float *dst);       /* N x K */
int ammsb_get_phi(ammsb_handle *h, float *dst);      /* N x K */
int ammsb_get_theta(ammsb_handle *h, double *dst);   /* K x 2 */
int ammsb_get_beta(ammsb_handle *h, float *dst);     /* K */
int ammsb_get_ppx(ammsb_handle *h, float *dst);      /* held-out count */
int ammsb_get_step(ammsb_handle *h, uint64_t *step_count,
                   uint64_t *average_count);
int ammsb_set_step(ammsb_handle *h, uint64_t step_count);

/* Draws of the last ammsb_step() iteration, for sampling parity.
 * sizes: n_edges <= max_edges, n_nodes <= max_nodes; nbrs/nbr_y hold
 * n_nodes x (num_node_sample + 1). */
int ammsb_get_last_minibatch(ammsb_handle *h, int32_t *flag, int32_t *n_edges,
                             int32_t *n_nodes, float *scale,
                             int32_t *edge_slot_a, int32_t *edge_slot_b,
                             uint8_t *edge_y, int32_t *nodes, int32_t *nbrs,
                             uint8_t *nbr_y);
/* Buffer capacities of the handle. */
int ammsb_get_sizes(ammsb_handle *h, int64_t *N, int64_t *K,
                    int64_t *max_edges, int64_t *max_nodes,
                    int64_t *num_node_sample, int64_t *held_out_count);
/* Options after the derived defaults were applied. */
int ammsb_get_options(ammsb_handle *h, ammsb_options *out);

/* Device-side timing of one iteration's phases (milliseconds, CUDA events
 * on the handle's stream): sample_mini_batch, sample_neighbor_nodes,
 * update_phi, update_pi + beta gradients, theta.  Mirrors the reference's
 * per-phase Timers (cc:95-102). */
int ammsb_profile_step(ammsb_handle *h, double *ms5);

/* Raw stream of the handle (cudaStream_t as void*), for callers that
 * order their own work against it. */
void *ammsb_stream(ammsb_handle *h);

/* Device-side running totals since the last init/set_state: sampled edge
 * evaluations (sum over iterations of minibatch nodes x (num_node_sample
 * + 1), the unit of the edge-evals/s metric) and sampled iterations. */
int ammsb_get_counters(ammsb_handle *h, uint64_t *edge_evals,
                       uint64_t *iterations);

/* Autotuner of the update_phi kernel (no reference counterpart): times
 * every built shape of the kernel that covers this handle's rows -- lanes
 * per node and vectors per lane (the K-tile), sub-groups per node (warps per
 * node), and the ring kernel's depth for wide rows -- `reps`
 * launches each on a non-link minibatch of the handle's own graph against a
 * scratch copy of phi (the chain's state and its draws are untouched), and
 * keeps the fastest.  Choices are cached per (device, pi type, row width,
 * neighbours, minibatch capacity) for the process; AMMSB_TUNE_FRESH times
 * again.  Needs a state (ammsb_init_state / ammsb_set_state). */
#define AMMSB_TUNE_FRESH 1
int ammsb_autotune(ammsb_handle *h, int32_t reps, int32_t flags);
/* The update_phi configuration in use: out[0..4] = ring kernel (0/1),
 * lanes per node, vectors per lane, sub-groups per node, ring depth. */
int ammsb_get_kernel_config(ammsb_handle *h, int32_t *out);

/* Batches of independent chains (no reference counterpart): the
 * iterations of many handles -- each with its own graph, held-out set,
 * state, options and update_phi configuration -- advanced together, one
 * CUDA graph launch per iteration for all of them.  Each kernel of the
 * iteration runs once for all chains sharing its compiled shape (the chain
 * is the grid's y index), so chains of different sizes and row widths take
 * a handful of launches per iteration instead of five each.  A chain goes
 * through exactly the states it goes through when stepped on its own (same
 * kernels, same draws); its step counter advances with the batch.  The
 * handles must outlive the batch and must not be stepped concurrently with
 * it; stepping a handle on its own between batch steps is allowed (the
 * batch then draws again from each chain's own step counter). */
typedef struct ammsb_batch ammsb_batch;
int ammsb_batch_create(ammsb_handle *const *handles, int32_t n,
                       ammsb_batch **out);
void ammsb_batch_destroy(ammsb_batch *b);
/* n_iters iterations of every chain (ammsb_step semantics per chain). */
int ammsb_batch_step(ammsb_batch *b, int64_t n_iters);
/* Number of update_phi launches per iteration (distinct kernel shapes). */
int32_t ammsb_batch_groups(const ammsb_batch *b);
void *ammsb_batch_stream(ammsb_batch *b);
const char *ammsb_batch_last_error(const ammsb_batch *b);
const char *ammsb_batch_create_error(void);

/* Checkpoint and resume.  No counterpart in the reference's sequential
 * sampler (its state lives only in memory).  ammsb_save_checkpoint writes
 * the whole chain to `path`: phi, the stored pi bit for bit (F32 or BF16),
 * theta, beta, the held-out running averages, step_count, average_count, the
 * perplexity history of the convergence test (learner.cc:130-136) and the
 * Philox key (seed, chain).  Every draw is a function of (seed, chain,
 * step), so a handle created with the same options and data that loads the
 * checkpoint continues the trajectory bit for bit.  ammsb_load_checkpoint
 * rejects (AMMSB_E_ARG) a file whose pi type, N, K, held-out set, seed or
 * chain differ from the handle's.  Both synchronise the handle's stream. */
int ammsb_save_checkpoint(ammsb_handle *h, const char *path);
int ammsb_load_checkpoint(ammsb_handle *h, const char *path);

/* Held-out perplexity without any device allocation.  No counterpart in
 * the reference: it serves callers that cannot call cudaMalloc (a host
 * program whose runtime owns every device allocation, or that must not
 * allocate after start-up) and hold the sampler state in device memory they
 * obtained themselves.  Same kernel and result as ammsb_perplexity, but no
 * handle: pi (n_rows rows of row_stride elements, 16-byte aligned rows, F32
 * or BF16), beta, the held-out pairs and the running averages ppx (updated)
 * are caller-owned device arrays; *out (host) receives -mean log of the
 * running averages.  Only the first K elements of a row are read: what the
 * row padding holds does not matter.  A pair naming a row outside
 * [0, n_rows) is skipped on the device, before any row is read, and the
 * call returns AMMSB_E_ARG (the other pairs' running averages are
 * updated).  Its scratch is a fixed 256 KB __device__ array, so held_count
 * is limited to 4,194,304 (AMMSB_E_CAPACITY beyond).  The array is shared
 * by every call on a device and keeps the last call's contents: calls whose
 * kernels overlap on the GPU race.  The first call on a device looks up the
 * array's address with that device current.  Runs on `stream` (a
 * cudaStream_t, 0 for the legacy default stream), copies its result into
 * host memory and synchronises the stream before returning, so it cannot
 * be called on a stream that is being captured into a CUDA graph. */
int ammsb_perplexity_noalloc(const void *pi, int32_t pi_dtype, int64_t K,
                             int64_t row_stride, int64_t n_rows,
                             const float *beta, double epsilon,
                             const int32_t *held_a, const int32_t *held_b,
                             const uint8_t *held_y, int64_t held_count,
                             float *ppx, uint64_t average_count, void *stream,
                             double *out);

/* ------------------------------------------------------------------------ */
/* Minibatch edge log-likelihood and its adjoint (the SGRLD drift).        */
/* ------------------------------------------------------------------------ */
/* L = sum over pairs q = (a, b, y) of log p_q, with
 *   p_q = sum_k pi_ak pi_bk (f_qk - e_q) + e_q,  pi_a = phi_a / sum(phi_a),
 *   f = y ? beta : 1 - beta,  e = y ? epsilon : 1 - epsilon,
 *   beta_k = theta_k1 / (theta_k0 + theta_k1):
 * the probability update_beta normalises by (prob_sum,
 * mcmc_sampler_stochastic.cc:212-240) of a source row given as phi and a
 * neighbour row given as pi (cal_edge_likelihood, learner.h:100-139, leaves
 * out eps * (1 - sum_k pi_ak pi_bk) for a link).  Its gradient in phi is the
 * update_phi gradient
 * (mcmc_sampler_stochastic.cc:274-296, neighbour pi held fixed) and in theta
 * the update_beta gradient (cc:212-240): the hand-derived terms the
 * reference uses as its SGRLD drift.  All arrays are device memory of
 * element type dtype: phi_src n_src rows (stride ld_phi), pi_nbr n_nbr rows
 * (stride ld_pi), theta K x 2.  Pairs are grouped by source: the pairs of
 * source a are q in [src_ptr[a], src_ptr[a+1]), with neighbour row
 * pair_nbr[q] and label pair_y[q].  The forward writes *loss (device) and
 * keeps p_q and the row sums in `workspace` (caller-owned device memory of
 * ammsb_edge_loglik_workspace_size bytes); the backward reads them back, so
 * the two calls share one workspace and the same inputs.  Index errors in
 * the pair arrays skip the pair and set bit 1 of the workspace's status
 * word, a non-positive row sum or probability sets bit 2 (read with
 * ammsb_edge_loglik_status).  Deterministic: every sum runs in a fixed
 * order.  Kernels are queued on `stream`; nothing is synchronised. */
size_t ammsb_edge_loglik_workspace_size(int32_t dtype, int64_t K,
                                        int64_t n_src, int64_t n_pairs);
int ammsb_edge_loglik_forward(int32_t dtype, int64_t K, const void *phi_src,
                              int64_t ld_phi, const void *pi_nbr,
                              int64_t ld_pi, int64_t n_nbr, const void *theta,
                              double epsilon, const int64_t *src_ptr,
                              int64_t n_src, const int32_t *pair_nbr,
                              const uint8_t *pair_y, int64_t n_pairs,
                              void *loss, void *workspace, void *stream);
/* grad_loss: device scalar dL.  Writes grad_phi_src (n_src rows, stride
 * ld_phi), grad_theta (K x 2) and, when grad_pi_nbr is not null, grad_pi_nbr
 * (n_nbr rows, stride ld_pi), which needs the pairs grouped by neighbour
 * too: the pairs of neighbour row b are nbr_pairs[r], r in
 * [nbr_ptr[b], nbr_ptr[b+1]), and pair_src[q] is the source of pair q. */
int ammsb_edge_loglik_backward(int32_t dtype, int64_t K, const void *phi_src,
                               int64_t ld_phi, const void *pi_nbr,
                               int64_t ld_pi, int64_t n_nbr,
                               const void *theta, double epsilon,
                               const int64_t *src_ptr, int64_t n_src,
                               const int32_t *pair_nbr, const uint8_t *pair_y,
                               int64_t n_pairs, const int32_t *pair_src,
                               const int64_t *nbr_ptr,
                               const int32_t *nbr_pairs, const void *grad_loss,
                               void *grad_phi_src, void *grad_pi_nbr,
                               void *grad_theta, void *workspace,
                               void *stream);
/* Status word of a workspace (bits above); synchronises `stream`. */
int ammsb_edge_loglik_status(const void *workspace, void *stream,
                             int32_t *flags);

/* ------------------------------------------------------------------------ */
/* Host-side data preparation (no GPU use).                                 */
/* ------------------------------------------------------------------------ */

/* Synthetic planted-community graph: n nodes, k_true communities with sizes
 * drawn Zipf(zipf_s) clipped to [size_min, size_max] and rescaled to cover
 * the memberships; each node joins 1/2/3 communities with probabilities
 * p1/p2/(1-p1-p2); each community of size s gets round(intra_degree * s / 2)
 * random member pairs; background_frac * that many uniform pairs are added;
 * self-loops dropped, duplicates merged.  Philox-seeded. */
typedef struct ammsb_gen_params {
  int64_t n;
  int64_t k_true;
  double zipf_s;
  int64_t size_min, size_max;
  double p1, p2;
  double intra_degree;
  double background_frac;
  uint32_t seed;
} ammsb_gen_params;

typedef struct ammsb_graph_buf ammsb_graph_buf;

/* Builds a graph; *out owns its arrays until ammsb_graph_free. */
int ammsb_generate_graph(const ammsb_gen_params *p, ammsb_graph_buf **out);
/* CSR from an edge list (any order, duplicates and self-loops dropped). */
int ammsb_graph_from_edges(int64_t n, int64_t n_edges, const int32_t *a,
                           const int32_t *b, ammsb_graph_buf **out);
/* Reads a relativity/SNAP text file (relativity.cc:20-200): four header
 * lines, then "a b" per line.  contiguous != 0 keeps ids as given
 * (N = max id + 1); otherwise ids are renumbered in ascending order. */
int ammsb_read_relativity(const char *path, int contiguous,
                          ammsb_graph_buf **out);
/* Writes the graph in that format (each undirected edge once, a < b). */
int ammsb_write_relativity(const ammsb_graph_buf *g, const char *path);
void ammsb_graph_view(const ammsb_graph_buf *g, ammsb_graph *view);
void ammsb_graph_free(ammsb_graph_buf *g);

/* Held-out and test sets (network.cc:503-614): held_out_size =
 * ratio * E; p = held_out_size / 2 random links plus p random non-links for
 * each set, test disjoint from held-out.  Philox-seeded. */
typedef struct ammsb_split_buf ammsb_split_buf;
int ammsb_make_held_out(const ammsb_graph_buf *g, double held_out_ratio,
                        uint32_t seed, ammsb_split_buf **out);
void ammsb_split_view(const ammsb_split_buf *s, ammsb_edge_set *held_out,
                      ammsb_edge_set *test);
void ammsb_split_free(ammsb_split_buf *s);

/* Preprocessed networks: Network::save (network.cc:136-145) writes a loaded
 * network into a directory and Network::Init with input class
 * "preprocessed" (network.cc:49-65) reads it back instead of the text
 * graph and the random held-out / test draws.  Here the directory holds
 * graph.bin (symmetric CSR), held-out.bin (held-out ratio and pairs),
 * test.bin and aux.bin (N, E, largest degree), an own little-endian
 * binary layout in place of the reference's gzip'ed sparse-hash dumps.
 * ammsb_save_preprocessed creates the directory if needed (one level) and
 * overwrites the files; ammsb_load_preprocessed checks the files' tags and
 * sizes, the CSR (sorted rows, symmetric, ids in range) and the pairs,
 * returning AMMSB_E_ARG for anything else, and hands back owned buffers
 * (ammsb_graph_view / ammsb_split_view read them). */
int ammsb_save_preprocessed(const ammsb_graph *g, const ammsb_edge_set *held_out,
                            const ammsb_edge_set *test, double held_out_ratio,
                            const char *dirname);
int ammsb_load_preprocessed(const char *dirname, ammsb_graph_buf **graph_out,
                            ammsb_split_buf **split_out, double *held_out_ratio);

#ifdef __cplusplus
}
#endif
#endif
