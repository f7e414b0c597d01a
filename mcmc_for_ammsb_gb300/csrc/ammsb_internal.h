// ammsb_internal.h -- the sampler handle and the helpers shared by the
// host-side translation units (ammsb_gpu.cu: one chain; ammsb_batch.cu:
// many chains per launch).  Not part of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/ammsb_gpu.h"
#include "ammsb_kernels.cuh"

using namespace ammsb;

constexpr int kRing = 4;  // minibatch buffer sets per handle

// Launches of the iteration that may start before the kernel ahead of them
// has finished (programmatic dependent launch): update_phi after the
// previous iteration's theta step, the commit after update_phi, the theta
// step after the commit.
enum : int { kPdlPhi = 1, kPdlCommit = 2, kPdlTheta = 4 };

struct KernelCfg {
  int lpn, vpl, split, npb;  // update_phi
  int ring;                  // wide rows: the shared-memory ring kernel
  int ring_stages;           // its ring depth
  int ring_few;              // a 16-warp variant takes iterations of few nodes
  int ring_grid;             // CTAs of the many-node ring launch (0: one per node slot)
  int pdl;                   // programmatic dependent launches: kPdl* bits
  int graph_pairs;           // pairs of iterations per long graph launch (<= 1: none)
  int ppx_lpn, ppx_vpl;      // perplexity
  int kq;                    // commit_beta
};

struct ammsb_handle {
  ammsb_options opt{};
  int device = 0;
  cudaStream_t stream = nullptr;  // the handle's stream: updates, perplexity, copies
  cudaStream_t side = nullptr;    // draws of the next iteration, overlapped with the update
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  Model m{};
  DevGraph g{};
  Buffers b{};        // shared state pointers (bufs[s] add the minibatch buffers)
  Buffers bufs[kRing]{};  // ring of minibatch buffer sets (draws run two iterations ahead)
  DevCounters* gc = nullptr;
  int slot = 0;   // ring slot of the next iteration
  int ahead = 0;  // iterations from `slot` on whose draws are made or queued (0..2)
  int last = -1;            // buffer set of the last applied iteration
  KernelCfg cfg{};
  int64_t E = 0, H = 0, T = 0;
  int pi_bytes = 4;
  // device allocations
  std::vector<void*> allocs;
  int32_t* d_ha = nullptr;
  int32_t* d_hb = nullptr;
  uint8_t* d_hy = nullptr;
  float* d_ppx = nullptr;
  double* d_ppx_part = nullptr;
  double* d_ppx_out = nullptr;
  int ppx_blocks = 1;
  float* d_fed_phi_noise = nullptr;
  float* d_fed_theta_noise = nullptr;
  int32_t* d_err_init = nullptr;
  int ncommit = 1;
  int nbr_blocks = 1, phi_blocks = 1;
  size_t phi_smem = 0, phi_smem_wide = 0, nbr_smem = 0, mb_smem = 0;
  // host mirrors
  uint64_t step_count = 1;     // learner.cc:37
  uint64_t average_count = 1;  // learner.cc:30
  std::vector<double> ppx_history;
  bool state_ready = false;
  // captured iterations per ring slot: one iteration, and two iterations
  // with the draws of the following two made alongside
  cudaGraphExec_t graph1[kRing] = {}, graph2[kRing] = {};
  cudaGraphExec_t graphL[kRing] = {};  // cfg.graph_pairs pipelined pairs of iterations in one launch
  // run()'s per-phase timers (mcmc_sampler_stochastic.cc:93-102), printed
  // as PrintStats does (cc:185-198): wall time and ticks per timer
  struct Timer {
    double seconds = 0.0;
    uint64_t ticks = 0;
  };
  enum { kTOuter, kTPerplexity, kTMiniBatch, kTNodes, kTNeighbors, kTPhi, kTPi, kTBeta, kTimers };
  Timer timers[kTimers];
  bool timing = false;  // run() launches the timed captures below
  // the same iterations with CUDA events between the phases: per launch of
  // n iterations, 1 + 3n events on the update stream, then 1 + 2n on the
  // draws' stream; one event set per (n, slot)
  cudaGraphExec_t graph1t[kRing] = {}, graph2t[kRing] = {};
  cudaEvent_t ev_phase[2][kRing][12] = {};
  struct Pending {
    int n, s;
  };
  std::vector<Pending> pending;  // timed launches whose events are not read yet
  uint64_t evals_read = 0;       // edge evaluations counted into the timers' ticks
  // a sharded iteration in progress (ammsb_shard_*): the drawn buffer set
  // and the device arrays of its phases
  int shard_drawn = -1;
  int shard_phase = 0;  // 1 drawn, 2 owned rows updated, 3 committed
  int32_t* d_shard_idx = nullptr;  // max(max_nodes, max_edges) slot / edge indices
  double* d_shard_R = nullptr;     // K x 2 beta-gradient sums
  std::string err;
};

#define CK(call)                                                              \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) {                                                  \
      h->err = std::string(#call) + ": " + cudaGetErrorString(e_);            \
      return AMMSB_E_CUDA;                                                    \
    }                                                                         \
  } while (0)

// Shapes of the register-path update_phi kernel that are built: (lanes per
// node, 16-byte vectors per lane, sub-groups splitting the neighbours).  The
// lanes x vectors product is the K-tile a node's row is cut into; lanes x
// split is the number of threads (warps-per-node x 32) that work on a node.
#define AMMSB_PHI_REG_SHAPES(X)                                                         \
  X(1, 1, 1) X(2, 1, 1) X(4, 1, 1) X(8, 1, 1) X(16, 1, 1) X(32, 1, 1) X(32, 1, 2)       \
  X(32, 1, 4) X(32, 2, 1) X(32, 2, 2) X(32, 2, 4) X(32, 4, 1) X(32, 4, 2) X(32, 4, 4)   \
  X(32, 8, 1) X(32, 8, 2) X(32, 8, 4) X(16, 1, 2) X(8, 1, 2) X(8, 1, 4) X(16, 2, 1)     \
  X(8, 2, 1) X(8, 4, 1) X(4, 2, 1) X(4, 4, 1) X(4, 1, 8) X(2, 1, 8) X(1, 1, 8)

// Iterations with at most kRingFewNodes nodes (the link stratum) take a
// kRingSplitWide-warp variant of the ring update_phi kernel.
constexpr int kRingFewNodes = 64;
constexpr int kRingSplitWide = 16;

// Ring depths the ring update_phi kernel is built for.
#define AMMSB_PHI_RING_STAGES(X) X(3) X(4) X(6)

namespace ammsb_detail {
// Raises a kernel's dynamic shared memory limit to at least `bytes` and
// never lowers it: the limit belongs to the kernel, not to a handle, and
// handles of different sizes share kernels.
template <typename F>
cudaError_t raise_smem_limit(F* kernel, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> set;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  size_t& cur = set[std::make_pair(dev, reinterpret_cast<const void*>(kernel))];
  if (bytes <= cur) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur = bytes;
  return e;
}

// Reads the device error word of a handle (synchronises its stream).
int check_device_err(ammsb_handle* h);
// Drops draws made ahead of time and points the next draw at step_count.
int invalidate_prefetch(ammsb_handle* h);
}  // namespace ammsb_detail
