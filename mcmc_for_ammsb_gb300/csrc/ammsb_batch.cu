// ammsb_batch.cu -- many independent chains advanced together, one CUDA
// graph launch per iteration for all of them.
//
// Each chain is an ammsb_handle of its own (its graph, held-out set, state,
// options and update_phi configuration).  The batch launches every kernel
// of the iteration once for all chains that share the kernel's compiled
// shape: blockIdx.y selects the chain, whose model, graph and buffer sets
// come from a device array of ChainArgs.  Chains of different row widths,
// minibatch sizes and graphs therefore run in a handful of launches per
// iteration instead of five per chain, and the whole iteration of all
// chains -- the update of iteration t and, on a second stream, the draws of
// t + 1 -- is captured as one graph per buffer parity.  Every chain keeps
// its own step counter and Philox key, so a chain advanced in a batch goes
// through exactly the states it goes through on its own.
#include <algorithm>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "ammsb_internal.h"
#include "ammsb_phi_ring.cuh"

namespace {

// One launch of the update phase: the chains sharing a kernel shape.
struct PhiGroup {
  int dtype;
  KernelCfg cfg;
  bool full;  // ring kernel: every lane's vectors inside the row
  std::vector<int> chains;
  ChainArgs* d = nullptr;  // the group's chains, in order
  int gx = 1;
  size_t smem = 0;
  size_t smem_wide = 0;  // ring kernel: its 16-warp variant
};

struct CommitGroup {
  int dtype, kq;
  std::vector<int> chains;
  ChainArgs* d = nullptr;
  int gx = 1;
};

constexpr int kRingSplitB = 4;

template <typename PiT, int L, int V, int S>
cudaError_t phi_reg_chains(const PhiGroup& g, int p, cudaStream_t st) {
  constexpr int NPB = 128 / (L * S) > 0 ? 128 / (L * S) : 1;
  k_update_phi_chains<PiT, L, V, S, NPB><<<dim3(g.gx, (unsigned)g.chains.size()), NPB * S * L, g.smem, st>>>(
      g.d, p);
  return cudaGetLastError();
}

template <typename PiT, int V, int STAGES, bool FULL>
cudaError_t phi_ring_chains(const PhiGroup& g, int p, cudaStream_t st, bool configure) {
  // the same pair of launches as one chain: a 16-warp variant for the
  // iterations of few nodes, the 4-warp kernel for the others
  constexpr int WS = sizeof(PiT) == 2 ? 4 : 2;
  auto kern = k_update_phi_ring_chains<PiT, V, kRingSplitB, STAGES, FULL>;
  auto wide = k_update_phi_ring_chains<PiT, V, kRingSplitWide, WS, FULL>;
  // every chain of the group configured the variant (its shared memory is
  // then the largest of theirs), or none did
  const bool use_wide = g.cfg.ring_few && g.smem_wide > 0 && g.smem_wide <= 200 * 1024;
  if (configure) {
    cudaError_t e = ammsb_detail::raise_smem_limit(kern, g.smem);
    if (e == cudaSuccess && use_wide) e = ammsb_detail::raise_smem_limit(wide, g.smem_wide);
    return e;
  }
  const unsigned n = (unsigned)g.chains.size();
  if (use_wide) {
    wide<<<dim3(kRingFewNodes, n), kRingSplitWide * 32, g.smem_wide, st>>>(g.d, p, 0, kRingFewNodes);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    kern<<<dim3(g.gx, n), kRingSplitB * 32, g.smem, st>>>(g.d, p, kRingFewNodes, INT32_MAX);
  } else {
    kern<<<dim3(g.gx, n), kRingSplitB * 32, g.smem, st>>>(g.d, p, 0, INT32_MAX);
  }
  return cudaGetLastError();
}

template <typename PiT, int V>
cudaError_t phi_ring_chains_v(const PhiGroup& g, int p, cudaStream_t st, bool configure) {
#define RING_CASE(S)                                                                           \
  if (g.cfg.ring_stages == S)                                                                  \
    return g.full ? phi_ring_chains<PiT, V, S, true>(g, p, st, configure)                      \
                  : phi_ring_chains<PiT, V, S, false>(g, p, st, configure);
  AMMSB_PHI_RING_STAGES(RING_CASE)
#undef RING_CASE
  return cudaErrorInvalidConfiguration;
}

template <typename PiT>
cudaError_t phi_chains(const PhiGroup& g, int p, cudaStream_t st, bool configure) {
  const KernelCfg& c = g.cfg;
  if (c.ring) {
    switch (c.vpl) {
      case 1: return phi_ring_chains_v<PiT, 1>(g, p, st, configure);
      case 2: return phi_ring_chains_v<PiT, 2>(g, p, st, configure);
      case 4: return phi_ring_chains_v<PiT, 4>(g, p, st, configure);
      case 8: return phi_ring_chains_v<PiT, 8>(g, p, st, configure);
      default: return cudaErrorInvalidConfiguration;
    }
  }
  if (configure) {
    if (g.smem <= 48 * 1024) return cudaSuccess;
#define REG_CFG(L, V, S)                                                                        \
  if (c.lpn == L && c.vpl == V && c.split == S)                                                 \
    return ammsb_detail::raise_smem_limit(                                                      \
        k_update_phi_chains<PiT, L, V, S, (128 / (L * S) > 0 ? 128 / (L * S) : 1)>, g.smem);
    AMMSB_PHI_REG_SHAPES(REG_CFG)
#undef REG_CFG
    return cudaErrorInvalidConfiguration;
  }
#define REG_CASE(L, V, S) \
  if (c.lpn == L && c.vpl == V && c.split == S) return phi_reg_chains<PiT, L, V, S>(g, p, st);
  AMMSB_PHI_REG_SHAPES(REG_CASE)
#undef REG_CASE
  return cudaErrorInvalidConfiguration;
}

template <typename PiT>
cudaError_t commit_chains(const CommitGroup& g, int p, cudaStream_t st) {
  const dim3 grid(g.gx, (unsigned)g.chains.size());
  switch (g.kq) {
    case 1: k_commit_beta_chains<PiT, 1><<<grid, 128, 0, st>>>(g.d, p); break;
    case 2: k_commit_beta_chains<PiT, 2><<<grid, 128, 0, st>>>(g.d, p); break;
    case 4: k_commit_beta_chains<PiT, 4><<<grid, 128, 0, st>>>(g.d, p); break;
    case 8: k_commit_beta_chains<PiT, 8><<<grid, 128, 0, st>>>(g.d, p); break;
    default: return cudaErrorInvalidConfiguration;
  }
  return cudaGetLastError();
}

}  // namespace

struct ammsb_batch {
  int device = 0;
  std::vector<ammsb_handle*> h;
  cudaStream_t stream = nullptr, side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_done = nullptr;
  // update_phi groups after the first run side by side on their own streams
  std::vector<cudaStream_t> gstream;
  std::vector<cudaEvent_t> gevent;
  cudaEvent_t ev_groups = nullptr;
  ChainArgs* d_all = nullptr;
  std::vector<void*> allocs;
  std::vector<PhiGroup> phi;
  std::vector<CommitGroup> commit;
  int theta_gx = 1;
  int nbr_gx = 1;
  size_t mb_smem = 0, nbr_smem = 0;
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  cudaGraphExec_t execL[2] = {nullptr, nullptr};  // graph_iters iterations per launch
  int graph_iters = 8;
  int parity = 0;
  bool prefetched = false;
  std::vector<uint64_t> expect_step;  // each chain's step_count after the last batch step
  std::string err;
};

namespace {

thread_local std::string g_batch_create_error;

#define BK(call)                                                       \
  do {                                                                 \
    cudaError_t e_ = (call);                                           \
    if (e_ != cudaSuccess) {                                           \
      bt->err = std::string(#call) + ": " + cudaGetErrorString(e_);   \
      return AMMSB_E_CUDA;                                             \
    }                                                                  \
  } while (0)

cudaError_t launch_update_chains(ammsb_batch* bt, int p) {
  // the update_phi groups touch disjoint chains: they run concurrently
  // (parallel branches of the captured graph), then join before the commits
  const size_t ng = bt->phi.size();
  cudaError_t e = cudaSuccess;
  if (ng > 1 && (e = cudaEventRecord(bt->ev_groups, bt->stream)) != cudaSuccess) return e;
  for (size_t gi = 0; gi < ng; ++gi) {
    const PhiGroup& g = bt->phi[gi];
    cudaStream_t st = gi == 0 ? bt->stream : bt->gstream[gi - 1];
    if (gi > 0 && (e = cudaStreamWaitEvent(st, bt->ev_groups, 0)) != cudaSuccess) return e;
    e = (g.dtype == AMMSB_PI_BF16) ? phi_chains<__nv_bfloat16>(g, p, st, false)
                                   : phi_chains<float>(g, p, st, false);
    if (e != cudaSuccess) return e;
    if (gi > 0 && (e = cudaEventRecord(bt->gevent[gi - 1], st)) != cudaSuccess) return e;
  }
  for (size_t gi = 1; gi < ng; ++gi)
    if ((e = cudaStreamWaitEvent(bt->stream, bt->gevent[gi - 1], 0)) != cudaSuccess) return e;
  for (const CommitGroup& g : bt->commit) {
    cudaError_t e = (g.dtype == AMMSB_PI_BF16) ? commit_chains<__nv_bfloat16>(g, p, bt->stream)
                                               : commit_chains<float>(g, p, bt->stream);
    if (e != cudaSuccess) return e;
  }
  k_theta_chains<<<dim3(bt->theta_gx, (unsigned)bt->h.size()), 1024, 0, bt->stream>>>(bt->d_all, p);
  return cudaGetLastError();
}

cudaError_t launch_sampling_chains(ammsb_batch* bt, int p, cudaStream_t st) {
  const unsigned n = (unsigned)bt->h.size();
  k_sample_minibatch_chains<<<dim3(1, n), 1024, bt->mb_smem, st>>>(bt->d_all, p);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_sample_neighbors_chains<8><<<dim3(bt->nbr_gx, n), 256, bt->nbr_smem, st>>>(bt->d_all, p);
  return cudaGetLastError();
}

cudaError_t launch_pipelined_chains(ammsb_batch* bt, int p) {
  cudaError_t e = cudaEventRecord(bt->ev_fork, bt->stream);
  if (e != cudaSuccess) return e;
  if ((e = cudaStreamWaitEvent(bt->side, bt->ev_fork, 0)) != cudaSuccess) return e;
  if ((e = launch_update_chains(bt, p)) != cudaSuccess) return e;
  if ((e = launch_sampling_chains(bt, 1 - p, bt->side)) != cudaSuccess) return e;
  if ((e = cudaEventRecord(bt->ev_join, bt->side)) != cudaSuccess) return e;
  return cudaStreamWaitEvent(bt->stream, bt->ev_join, 0);
}

template <typename T>
cudaError_t dev_upload(ammsb_batch* bt, T** out, const std::vector<T>& v) {
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, std::max<size_t>(sizeof(T) * v.size(), 16));
  if (e != cudaSuccess) return e;
  bt->allocs.push_back(p);
  *out = static_cast<T*>(p);
  return cudaMemcpy(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice);
}

}  // namespace

extern "C" {

const char* ammsb_batch_create_error(void) { return g_batch_create_error.c_str(); }

const char* ammsb_batch_last_error(const ammsb_batch* bt) { return bt ? bt->err.c_str() : "null batch"; }

void ammsb_batch_destroy(ammsb_batch* bt) {
  if (!bt) return;
  cudaSetDevice(bt->device);
  if (bt->stream) cudaStreamSynchronize(bt->stream);
  if (bt->side) cudaStreamSynchronize(bt->side);
  for (auto* set : {bt->exec, bt->execL})
    for (int q = 0; q < 2; ++q)
      if (set[q]) cudaGraphExecDestroy(set[q]);
  for (void* p : bt->allocs) cudaFree(p);
  for (cudaEvent_t ev : {bt->ev_fork, bt->ev_join, bt->ev_done, bt->ev_groups})
    if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t ev : bt->gevent) cudaEventDestroy(ev);
  for (cudaStream_t st : bt->gstream) cudaStreamDestroy(st);
  if (bt->side) cudaStreamDestroy(bt->side);
  if (bt->stream) cudaStreamDestroy(bt->stream);
  delete bt;
}

int ammsb_batch_create(ammsb_handle* const* handles, int32_t n, ammsb_batch** out) {
  g_batch_create_error.clear();
  if (!handles || n < 1 || !out) {
    g_batch_create_error = "need at least one handle";
    return AMMSB_E_ARG;
  }
  *out = nullptr;
  auto* bt = new ammsb_batch();
  auto bail = [&](int code) {
    g_batch_create_error = bt->err;
    ammsb_batch_destroy(bt);
    return code;
  };
  for (int i = 0; i < n; ++i) {
    ammsb_handle* h = handles[i];
    if (!h) {
      bt->err = "null handle";
      return bail(AMMSB_E_ARG);
    }
    for (int j = 0; j < i; ++j)
      if (handles[j] == h) {
        bt->err = "a handle appears twice";
        return bail(AMMSB_E_ARG);
      }
    if (i > 0 && h->device != handles[0]->device) {
      bt->err = "all chains must be on one device";
      return bail(AMMSB_E_ARG);
    }
    bt->h.push_back(h);
  }
  bt->device = handles[0]->device;
  if (const char* env = std::getenv("AMMSB_BATCH_GRAPH_ITERS"))  // even; 1 = one iteration per launch
    bt->graph_iters = std::max(1, std::min(64, std::atoi(env) & ~1));
  int prio_lo = 0, prio_hi = 0;  // the draws ahead at the higher priority, as for one chain
  if (cudaSetDevice(bt->device) != cudaSuccess ||
      cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi) != cudaSuccess ||
      cudaStreamCreateWithFlags(&bt->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithPriority(&bt->side, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
      cudaEventCreateWithFlags(&bt->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&bt->ev_join, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&bt->ev_done, cudaEventDisableTiming) != cudaSuccess) {
    bt->err = "stream/event creation failed";
    return bail(AMMSB_E_CUDA);
  }
  std::vector<ChainArgs> args(n);
  for (int i = 0; i < n; ++i) {
    ammsb_handle* h = bt->h[i];
    ChainArgs& a = args[i];
    a.m = h->m;
    a.g = h->g;
    a.b[0] = h->bufs[0];
    a.b[1] = h->bufs[1];
    a.ncommit = h->ncommit;
    a.smem_hash = h->mb_smem > 0 ? 1 : 0;
    bt->mb_smem = std::max(bt->mb_smem, h->mb_smem);
    bt->nbr_smem = std::max(bt->nbr_smem, h->nbr_smem);
    bt->nbr_gx = std::max(bt->nbr_gx, h->nbr_blocks);
    bt->theta_gx = std::max(bt->theta_gx, (h->m.K + 31) / 32);
  }
  if (dev_upload(bt, &bt->d_all, args) != cudaSuccess) {
    bt->err = "upload of the chain table failed";
    return bail(AMMSB_E_CUDA);
  }
  // group the update_phi launches by compiled shape, the commits by K-tile
  std::map<std::tuple<int, int, int, int, int, int, int>, int> pg;
  std::map<std::pair<int, int>, int> cg;
  for (int i = 0; i < n; ++i) {
    ammsb_handle* h = bt->h[i];
    const KernelCfg& c = h->cfg;
    const int ev = (h->opt.pi_dtype == AMMSB_PI_BF16) ? 8 : 4;
    const bool full = (h->m.Kp / ev == 32 * c.vpl);
    auto key = std::make_tuple((int)h->opt.pi_dtype, c.ring, c.lpn, c.vpl, c.split,
                               c.ring ? c.ring_stages : 0, c.ring ? (int)full : 0);
    auto it = pg.find(key);
    if (it == pg.end()) {
      PhiGroup g;
      g.dtype = h->opt.pi_dtype;
      g.cfg = c;
      g.full = full;
      it = pg.emplace(key, (int)bt->phi.size()).first;
      bt->phi.push_back(g);
    }
    PhiGroup& g = bt->phi[it->second];
    g.chains.push_back(i);
    if (c.ring) {
      g.gx = std::max(g.gx, h->m.max_nodes);
      g.smem = std::max(g.smem, h->phi_smem);
      g.smem_wide = std::max(g.smem_wide, h->phi_smem_wide);
    } else {
      const int npb = std::max(1, 128 / (c.lpn * c.split));
      g.gx = std::max(g.gx, std::max(1, std::min((h->m.max_nodes + npb - 1) / npb, 152 * 32)));
      const size_t smem = ((size_t)npb * c.split * h->m.Kp + npb * c.split +
                           npb * std::max(1, c.split * c.lpn / 32)) * sizeof(float);
      g.smem = std::max(g.smem, smem);
    }
    auto ck = std::make_pair((int)h->opt.pi_dtype, c.kq);
    auto jt = cg.find(ck);
    if (jt == cg.end()) {
      CommitGroup g2;
      g2.dtype = h->opt.pi_dtype;
      g2.kq = c.kq;
      jt = cg.emplace(ck, (int)bt->commit.size()).first;
      bt->commit.push_back(g2);
    }
    CommitGroup& g2 = bt->commit[jt->second];
    g2.chains.push_back(i);
    g2.gx = std::max(g2.gx, h->ncommit + h->m.nbb);
  }
  for (PhiGroup& g : bt->phi) {
    std::vector<ChainArgs> a;
    for (int i : g.chains) a.push_back(args[i]);
    if (dev_upload(bt, &g.d, a) != cudaSuccess) {
      bt->err = "upload of a group table failed";
      return bail(AMMSB_E_CUDA);
    }
    cudaError_t e = (g.dtype == AMMSB_PI_BF16) ? phi_chains<__nv_bfloat16>(g, 0, bt->stream, true)
                                               : phi_chains<float>(g, 0, bt->stream, true);
    if (e != cudaSuccess) {
      bt->err = std::string("update_phi group configuration: ") + cudaGetErrorString(e);
      return bail(AMMSB_E_CUDA);
    }
  }
  if (cudaEventCreateWithFlags(&bt->ev_groups, cudaEventDisableTiming) != cudaSuccess) {
    bt->err = "event creation failed";
    return bail(AMMSB_E_CUDA);
  }
  for (size_t gi = 1; gi < bt->phi.size(); ++gi) {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
      bt->err = "stream creation failed";
      return bail(AMMSB_E_CUDA);
    }
    bt->gstream.push_back(st);
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
      bt->err = "event creation failed";
      return bail(AMMSB_E_CUDA);
    }
    bt->gevent.push_back(ev);
  }
  for (CommitGroup& g : bt->commit) {
    std::vector<ChainArgs> a;
    for (int i : g.chains) a.push_back(args[i]);
    if (dev_upload(bt, &g.d, a) != cudaSuccess) {
      bt->err = "upload of a group table failed";
      return bail(AMMSB_E_CUDA);
    }
  }
  if ((bt->mb_smem > 48 * 1024 &&
       ammsb_detail::raise_smem_limit(k_sample_minibatch_chains, bt->mb_smem) != cudaSuccess) ||
      (bt->nbr_smem > 48 * 1024 &&
       ammsb_detail::raise_smem_limit(k_sample_neighbors_chains<8>, bt->nbr_smem) != cudaSuccess)) {
    bt->err = "sampler shared memory configuration failed";
    return bail(AMMSB_E_CUDA);
  }
  bt->expect_step.assign(n, 0);
  *out = bt;
  return AMMSB_OK;
}

int32_t ammsb_batch_groups(const ammsb_batch* bt) { return bt ? (int32_t)bt->phi.size() : -1; }

int ammsb_batch_step(ammsb_batch* bt, int64_t n_iters) {
  if (!bt || n_iters < 0) return AMMSB_E_ARG;
  BK(cudaSetDevice(bt->device));
  for (ammsb_handle* h : bt->h)
    if (!h->state_ready) {
      bt->err = "every chain needs a state (ammsb_init_state / ammsb_set_state)";
      return AMMSB_E_STATE;
    }
  if (n_iters == 0) return AMMSB_OK;
  // chains stepped on their own since the last batch step lose the batch's
  // draws made ahead: start from each chain's own step counter again
  bool in_sync = bt->prefetched;
  for (size_t i = 0; i < bt->h.size() && in_sync; ++i) {
    ammsb_handle* h = bt->h[i];
    in_sync = h->ahead >= 1 && h->slot == bt->parity && h->step_count == bt->expect_step[i];
  }
  for (ammsb_handle* h : bt->h) BK(cudaStreamSynchronize(h->stream));
  if (!in_sync) {
    for (ammsb_handle* h : bt->h) {
      int rc = ammsb_detail::invalidate_prefetch(h);
      if (rc) {
        bt->err = h->err;
        return rc;
      }
      h->slot = 0;
      BK(cudaStreamSynchronize(h->stream));
    }
    bt->parity = 0;
    BK(launch_sampling_chains(bt, 0, bt->stream));
    bt->prefetched = true;
  }
  // graph_iters iterations per graph launch while that many are left (an
  // even count: the launch ends on the parity it started from), then one
  for (int64_t it = 0; it < n_iters;) {
    const int p = bt->parity;
    const int L = (bt->graph_iters > 1 && n_iters - it >= bt->graph_iters) ? bt->graph_iters : 1;
    cudaGraphExec_t& g = (L > 1) ? bt->execL[p] : bt->exec[p];
    if (!g) {
      cudaGraph_t graph;
      BK(cudaStreamBeginCapture(bt->stream, cudaStreamCaptureModeThreadLocal));
      cudaError_t e = cudaSuccess;
      for (int j = 0; j < L && e == cudaSuccess; ++j) e = launch_pipelined_chains(bt, p ^ (j & 1));
      cudaError_t e2 = cudaStreamEndCapture(bt->stream, &graph);
      if (e != cudaSuccess || e2 != cudaSuccess) {
        bt->err = std::string("graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2);
        return AMMSB_E_CUDA;
      }
      BK(cudaGraphInstantiate(&g, graph, cudaGraphInstantiateFlagUseNodePriority));
      cudaGraphDestroy(graph);
    }
    BK(cudaGraphLaunch(g, bt->stream));
    bt->parity ^= (L & 1);
    it += L;
  }
  BK(cudaEventRecord(bt->ev_done, bt->stream));
  for (size_t i = 0; i < bt->h.size(); ++i) {
    ammsb_handle* h = bt->h[i];
    BK(cudaStreamWaitEvent(h->stream, bt->ev_done, 0));  // later work on the chain's own stream
    h->step_count += (uint64_t)n_iters;
    h->slot = bt->parity;
    h->ahead = 1;  // the batch draws one iteration ahead, into buffer sets 0 and 1
    h->last = bt->parity ^ 1;
    bt->expect_step[i] = h->step_count;
  }
  BK(cudaStreamSynchronize(bt->stream));
  for (ammsb_handle* h : bt->h) {
    int rc = ammsb_detail::check_device_err(h);
    if (rc) {
      bt->err = h->err;
      return rc;
    }
  }
  return AMMSB_OK;
}

void* ammsb_batch_stream(ammsb_batch* bt) { return bt ? (void*)bt->stream : nullptr; }

}  // extern "C"
