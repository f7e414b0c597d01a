// ammsb_gpu.cu -- host driver of the GB300 a-MMSB sampler and its C ABI
// (include/ammsb_gpu.h).  The handle plays the role of the reference's
// MCMCSamplerStochastic object (mcmc_sampler_stochastic.h:32-140): it owns
// phi, pi, theta, beta and the held-out running averages, all resident in
// GPU memory, and runs the iteration as a captured CUDA graph of the
// kernels in ammsb_kernels.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <tuple>
#include <vector>

#include "ammsb_internal.h"
#include "ammsb_phi_ring.cuh"

namespace {
thread_local std::string g_create_error;

int next_pow2(int64_t v) {
  int64_t p = 1;
  while (p < v) p <<= 1;
  return (int)p;
}

// Host gamma draw of the same stream layout as gamma_draw() (theta init).
double host_gamma(const Stream& s, uint32_t tag, uint32_t entity, uint64_t idx,
                  double shape, double scale) {
  double a = shape, boost = 1.0;
  if (a < 1.0) {
    U32x4 o = s.block(tag, entity, 0xffffffffu, idx);
    double u = ((double)o.w + 0.5) * 2.3283064365386963e-10;
    boost = std::pow(u, 1.0 / a);
    a += 1.0;
  }
  const double d = a - 1.0 / 3.0, c = 1.0 / std::sqrt(9.0 * d);
  for (uint32_t attempt = 0; attempt < 64; ++attempt) {
    U32x4 o = s.block(tag, entity, attempt, idx);
    double u1 = ((double)o.x + 0.5) * 2.3283064365386963e-10;
    double u2 = (double)o.y * 2.3283064365386963e-10;
    double x = std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * 3.14159265358979323846 * u2);
    double v = 1.0 + c * x;
    if (v <= 0.0) continue;
    v = v * v * v;
    double u = ((double)o.z + 0.5) * 2.3283064365386963e-10;
    if (u < 1.0 - 0.0331 * x * x * x * x) return d * v * boost * scale;
    if (std::log(u) < 0.5 * x * x + d * (1.0 - v + std::log(v))) return d * v * boost * scale;
  }
  return d * boost * scale;
}

}  // namespace

namespace {

template <typename T>
int dev_alloc(ammsb_handle* h, T** p, size_t count) {
  void* q = nullptr;
  size_t bytes = std::max<size_t>(count * sizeof(T), 16);
  CK(cudaMalloc(&q, bytes));
  CK(cudaMemsetAsync(q, 0, bytes, h->stream));
  h->allocs.push_back(q);
  *p = static_cast<T*>(q);
  return AMMSB_OK;
}

// ---- kernel dispatch -------------------------------------------------------
template <typename PiT, int LPN, int VPL, int SPLIT>
cudaError_t launch_phi_t(ammsb_handle* h, const Buffers& b) {
  constexpr int NPB = 128 / (LPN * SPLIT) > 0 ? 128 / (LPN * SPLIT) : 1;
  int blocks = (h->m.max_nodes + NPB - 1) / NPB;
  blocks = std::max(1, std::min(blocks, 152 * 32));
  size_t smem = ((size_t)NPB * SPLIT * h->m.Kp + NPB * SPLIT + NPB * std::max(1, SPLIT * LPN / 32)) * sizeof(float);
  k_update_phi<PiT, LPN, VPL, SPLIT, NPB><<<blocks, NPB * SPLIT * LPN, smem, h->stream>>>(h->m, b);
  return cudaGetLastError();
}

#ifndef AMMSB_RING_SPLIT
#define AMMSB_RING_SPLIT 4
#endif
constexpr int kRingSplit = AMMSB_RING_SPLIT;  // warps per node of the many-node ring kernel

// Launches `k` on stream `s`; with `pdl` as a programmatic dependent launch
// (it may start once every CTA of the kernel ahead of it in the stream has
// triggered, and waits on the device before reading that kernel's results).
template <typename... P, typename... A>
cudaError_t launch_k(void (*k)(P...), int grid, int block, size_t smem, cudaStream_t s, bool pdl,
                     A&&... args) {
  cudaLaunchConfig_t lc{};
  lc.gridDim = dim3(grid);
  lc.blockDim = dim3(block);
  lc.dynamicSmemBytes = smem;
  lc.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  lc.attrs = at;
  lc.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&lc, k, std::forward<A>(args)...);
}

// `pdl`: the launch directly follows k_theta in the stream and its draws
// were complete before that kernel started; the update kernels then start
// as programmatic dependent launches, the many-node kernel first, which
// overlaps its first row copies and node prologue with the theta step.
template <typename PiT, int VPL, int STAGES, bool FULL>
cudaError_t launch_phi_ring_t(ammsb_handle* h, const Buffers& b, bool configure, bool pdl = false) {
  auto kern = k_update_phi_ring<PiT, VPL, kRingSplit, STAGES, FULL>;
  constexpr int WS = sizeof(PiT) == 2 ? 4 : 2;  // ring depth of the 16-warp variant
  auto wide = k_update_phi_ring<PiT, VPL, kRingSplitWide, WS, FULL>;
  const size_t smem = PhiRingSmem<PiT, VPL, kRingSplit, STAGES>::bytes(h->m.Kp, h->m.n_out);
  const size_t smem_w = PhiRingSmem<PiT, VPL, kRingSplitWide, WS>::bytes(h->m.Kp, h->m.n_out);
  const bool use_wide = h->cfg.ring_few && smem_w <= 200 * 1024;
  if (configure) {
    cudaError_t e = ammsb_detail::raise_smem_limit(kern, smem);
    if (e != cudaSuccess) return e;
    if (use_wide && (e = ammsb_detail::raise_smem_limit(wide, smem_w)) != cudaSuccess) return e;
    h->phi_smem = smem;
    h->phi_smem_wide = use_wide ? smem_w : 0;
    return cudaSuccess;
  }
  // the many-node kernel walks the node slots grid-stride: one CTA per slot
  // unless a smaller grid is asked for
  const int grid = h->cfg.ring_grid > 0 ? std::min(h->cfg.ring_grid, h->m.max_nodes) : h->m.max_nodes;
  const int grid_w = std::min(kRingFewNodes, h->m.max_nodes);
  const Model& m = h->m;
  if (pdl) {
    cudaError_t e = launch_k(kern, grid, kRingSplit * 32, smem, h->stream, true, m, b,
                             use_wide ? kRingFewNodes : 0, INT32_MAX);
    if (e != cudaSuccess || !use_wide) return e;
    return launch_k(wide, grid_w, kRingSplitWide * 32, smem_w, h->stream, true, m, b, 0, kRingFewNodes);
  }
  if (use_wide) {
    wide<<<grid_w, kRingSplitWide * 32, smem_w, h->stream>>>(m, b, 0, kRingFewNodes);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    kern<<<grid, kRingSplit * 32, smem, h->stream>>>(m, b, kRingFewNodes, INT32_MAX);
  } else {
    kern<<<grid, kRingSplit * 32, smem, h->stream>>>(m, b, 0, INT32_MAX);
  }
  return cudaGetLastError();
}

// ring depths the ring kernel is built for; FULL when every lane's
// vectors lie inside the row
template <typename PiT, int VPL>
cudaError_t launch_phi_ring_v(ammsb_handle* h, const Buffers& b, bool configure, bool pdl) {
  constexpr int EV = PiTraits<PiT>::kPerVec;
  const bool full = (h->m.Kp / EV == 32 * VPL);
#define RING_CASE(S)                                                                        \
  if (h->cfg.ring_stages == S)                                                              \
    return full ? launch_phi_ring_t<PiT, VPL, S, true>(h, b, configure, pdl)                \
                : launch_phi_ring_t<PiT, VPL, S, false>(h, b, configure, pdl);
  AMMSB_PHI_RING_STAGES(RING_CASE)
#undef RING_CASE
  return cudaErrorInvalidConfiguration;
}

template <typename PiT>
cudaError_t launch_phi_ring(ammsb_handle* h, const Buffers& b, bool configure, bool pdl = false) {
  switch (h->cfg.vpl) {
    case 1: return launch_phi_ring_v<PiT, 1>(h, b, configure, pdl);
    case 2: return launch_phi_ring_v<PiT, 2>(h, b, configure, pdl);
    case 4: return launch_phi_ring_v<PiT, 4>(h, b, configure, pdl);
    case 8: return launch_phi_ring_v<PiT, 8>(h, b, configure, pdl);
    default: return cudaErrorInvalidConfiguration;
  }
}

template <typename PiT>
cudaError_t launch_phi(ammsb_handle* h, const Buffers& b, bool pdl = false) {
  const KernelCfg& c = h->cfg;
  if (c.ring) return launch_phi_ring<PiT>(h, b, false, pdl && (c.pdl & kPdlPhi));
#define PHI_CASE(L, V, S) \
  if (c.lpn == L && c.vpl == V && c.split == S) return launch_phi_t<PiT, L, V, S>(h, b);
  AMMSB_PHI_REG_SHAPES(PHI_CASE)
#undef PHI_CASE
  return cudaErrorInvalidConfiguration;
}

// `pdl`: as a programmatic dependent launch after update_phi
template <typename PiT>
cudaError_t launch_commit(ammsb_handle* h, const Buffers& b, bool pdl = false) {
  const int grid = h->ncommit + h->m.nbb;
  switch (h->cfg.kq) {
    case 1: return launch_k(k_commit_beta<PiT, 1>, grid, 128, 0, h->stream, pdl, h->m, b, h->ncommit);
    case 2: return launch_k(k_commit_beta<PiT, 2>, grid, 128, 0, h->stream, pdl, h->m, b, h->ncommit);
    case 4: return launch_k(k_commit_beta<PiT, 4>, grid, 128, 0, h->stream, pdl, h->m, b, h->ncommit);
    case 8: return launch_k(k_commit_beta<PiT, 8>, grid, 128, 0, h->stream, pdl, h->m, b, h->ncommit);
    default: return cudaErrorInvalidConfiguration;
  }
}

template <typename PiT>
cudaError_t launch_ppx(ammsb_handle* h, float count) {
  const PiT* pi = reinterpret_cast<const PiT*>(h->b.pi);
  const int nb = h->ppx_blocks;
#define PPX_CASE(L, V)                                                                         \
  if (h->cfg.ppx_lpn == L && h->cfg.ppx_vpl == V) {                                            \
    k_perplexity<PiT, L, V><<<nb, 256, 0, h->stream>>>(h->m, pi, h->b.beta, h->d_ha, h->d_hb, \
                                                       h->d_hy, h->H, h->d_ppx, count,        \
                                                       h->d_ppx_part, h->m.N, nullptr);       \
    return cudaGetLastError();                                                                 \
  }
  PPX_CASE(1, 1) PPX_CASE(2, 1) PPX_CASE(4, 1) PPX_CASE(8, 1) PPX_CASE(16, 1) PPX_CASE(32, 1)
  PPX_CASE(32, 2) PPX_CASE(32, 4) PPX_CASE(32, 8)
#undef PPX_CASE
  return cudaErrorInvalidConfiguration;
}

cudaError_t launch_normalize(ammsb_handle* h) {
  const int blocks = (int)std::min<int64_t>((h->m.N + 7) / 8, 152 * 64);
  if (h->opt.pi_dtype == AMMSB_PI_BF16)
    k_normalize_rows<__nv_bfloat16><<<blocks, 256, 0, h->stream>>>(
        h->m, h->b.phi, reinterpret_cast<__nv_bfloat16*>(h->b.pi));
  else
    k_normalize_rows<float><<<blocks, 256, 0, h->stream>>>(h->m, h->b.phi,
                                                           reinterpret_cast<float*>(h->b.pi));
  return cudaGetLastError();
}

// Records `ev` on `s` when timing (ev != nullptr).  Inside a stream
// capture an external record becomes an event-record node of the graph, so
// the event is recorded every time the graph runs (a plain record would only
// mark a dependency of the capture).
inline cudaError_t mark(cudaEvent_t ev, cudaStream_t s) {
  return ev ? cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal) : cudaSuccess;
}

// The iteration's kernels in order; `b` carries the fed-noise pointers when
// called from ammsb_step_fed (which skips the two sampling kernels).  With
// `ev`, events are recorded after update_phi, the commit and theta, and
// every kernel waits for the one ahead to finish; without, the commit and
// theta step start as programmatic dependent launches (cfg.pdl).  `pdl`:
// the previous iteration's theta step is the kernel ahead in the stream and
// this iteration's draws are complete (update_phi may then start early).
cudaError_t launch_update_phase(ammsb_handle* h, const Buffers& b, const cudaEvent_t* ev = nullptr,
                                bool pdl = false) {
  const int early = ev ? 0 : h->cfg.pdl;
  cudaError_t e = (h->opt.pi_dtype == AMMSB_PI_BF16) ? launch_phi<__nv_bfloat16>(h, b, pdl)
                                                      : launch_phi<float>(h, b, pdl);
  if (e != cudaSuccess || (e = mark(ev ? ev[0] : nullptr, h->stream)) != cudaSuccess) return e;
  e = (h->opt.pi_dtype == AMMSB_PI_BF16) ? launch_commit<__nv_bfloat16>(h, b, early & kPdlCommit)
                                          : launch_commit<float>(h, b, early & kPdlCommit);
  if (e != cudaSuccess || (e = mark(ev ? ev[1] : nullptr, h->stream)) != cudaSuccess) return e;
  e = launch_k(k_theta, (h->m.K + 31) / 32, 1024, 0, h->stream, early & kPdlTheta, h->m, b);
  if (e != cudaSuccess) return e;
  return mark(ev ? ev[2] : nullptr, h->stream);
}

// Draws of one iteration (minibatch + neighbour sets) into buffer set b;
// with `ev`, events after each of the two kernels.
cudaError_t launch_sampling_phase(ammsb_handle* h, const Buffers& b, cudaStream_t s,
                                  const cudaEvent_t* ev = nullptr) {
  k_sample_minibatch<<<1, 1024, h->mb_smem, s>>>(h->m, h->g, b, h->mb_smem > 0);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || (e = mark(ev ? ev[0] : nullptr, s)) != cudaSuccess) return e;
  k_sample_neighbors<8><<<h->nbr_blocks, 256, h->nbr_smem, s>>>(h->m, h->g, b);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  return mark(ev ? ev[1] : nullptr, s);
}

// `n` (1 or 2) pipelined iterations from ring slot s: the updates of slots
// s .. s+n-1 on the handle's stream, concurrently with the draws of the
// iterations two ahead (slots s+2 .. s+n+1) on the side stream (fork/join by
// events; inside a capture these become graph edges).  Draws depend only on
// the step index, so they can run ahead; taking two iterations per join
// lets the short updates of link-stratum iterations and the longer draws of
// the non-link ones even out.
// With `ev` (run()'s timers): events ev[0] before the first update and
// ev[1 + 3i ..] after each phase of update i on the update stream, then
// ev[1 + 3n] before the first draws and ev[2 + 3n + 2i ..] after each of
// draws i on the draws' stream.
// `first_pdl`: the previous pair's theta step is the kernel ahead of the
// first update (a long graph of several pairs), which may then start early
// too.
cudaError_t launch_pipelined(ammsb_handle* h, int s, int n, const cudaEvent_t* ev = nullptr,
                             bool first_pdl = false) {
  cudaError_t e = cudaEventRecord(h->ev_fork, h->stream);
  if (e != cudaSuccess) return e;
  if ((e = cudaStreamWaitEvent(h->side, h->ev_fork, 0)) != cudaSuccess) return e;
  if ((e = mark(ev ? ev[0] : nullptr, h->stream)) != cudaSuccess) return e;
  // the second update follows the first one's theta step directly (its
  // draws were joined before this launch)
  for (int i = 0; i < n; ++i)
    if ((e = launch_update_phase(h, h->bufs[(s + i) % kRing], ev ? ev + 1 + 3 * i : nullptr,
                                 (i > 0 || first_pdl) && !ev)) != cudaSuccess)
      return e;
  if ((e = mark(ev ? ev[1 + 3 * n] : nullptr, h->side)) != cudaSuccess) return e;
  for (int i = 0; i < n; ++i)
    if ((e = launch_sampling_phase(h, h->bufs[(s + 2 + i) % kRing], h->side,
                                   ev ? ev + 2 + 3 * n + 2 * i : nullptr)) != cudaSuccess)
      return e;
  if ((e = cudaEventRecord(h->ev_join, h->side)) != cudaSuccess) return e;
  return cudaStreamWaitEvent(h->stream, h->ev_join, 0);
}

// `n` (1 or 2) iterations from ring slot s in run()'s loop order on the
// handle's stream, each drawn right before its update (the pipeline
// option off).  With `ev`: per iteration i, events ev[6i] before the draws,
// ev[6i + 1], ev[6i + 2] after each draw kernel and ev[6i + 3 ..] after
// each update phase.
cudaError_t launch_serial(ammsb_handle* h, int s, int n, const cudaEvent_t* ev = nullptr) {
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < n; ++i) {
    const Buffers& b = h->bufs[(s + i) % kRing];
    if ((e = mark(ev ? ev[6 * i] : nullptr, h->stream)) != cudaSuccess) return e;
    if ((e = launch_sampling_phase(h, b, h->stream, ev ? ev + 6 * i + 1 : nullptr)) != cudaSuccess) return e;
    if ((e = launch_update_phase(h, b, ev ? ev + 6 * i + 3 : nullptr)) != cudaSuccess) return e;
  }
  return e;
}

// Adds the phase durations of a finished timed launch (n iterations from
// slot s) to run()'s timers; waits for the launch's events.
int read_phase_events(ammsb_handle* h, int n, int s) {
  const cudaEvent_t* ev = h->ev_phase[n - 1][s];
  if (!h->opt.pipeline) {  // launch_serial's layout: 6 events per iteration
    CK(cudaEventSynchronize(ev[6 * n - 1]));
    const int order[5] = {ammsb_handle::kTMiniBatch, ammsb_handle::kTNeighbors, ammsb_handle::kTPhi,
                          ammsb_handle::kTPi, ammsb_handle::kTBeta};
    for (int i = 0; i < n; ++i)
      for (int q = 0; q < 5; ++q) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, ev[6 * i + q], ev[6 * i + q + 1]));
        h->timers[order[q]].seconds += ms * 1e-3;
      }
    h->timers[ammsb_handle::kTMiniBatch].ticks += (uint64_t)n;
    h->timers[ammsb_handle::kTPi].ticks += (uint64_t)n;
    h->timers[ammsb_handle::kTBeta].ticks += (uint64_t)n;
    return AMMSB_OK;
  }
  const cudaEvent_t* sv = ev + 1 + 3 * n;
  CK(cudaEventSynchronize(ev[3 * n]));
  CK(cudaEventSynchronize(sv[2 * n]));
  auto add = [&](int t, cudaEvent_t a, cudaEvent_t b) -> int {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, a, b));
    h->timers[t].seconds += ms * 1e-3;
    return AMMSB_OK;
  };
  for (int i = 0; i < n; ++i) {
    int rc = add(ammsb_handle::kTPhi, ev[3 * i], ev[3 * i + 1]);
    if (!rc) rc = add(ammsb_handle::kTPi, ev[3 * i + 1], ev[3 * i + 2]);
    if (!rc) rc = add(ammsb_handle::kTBeta, ev[3 * i + 2], ev[3 * i + 3]);
    if (!rc) rc = add(ammsb_handle::kTMiniBatch, sv[2 * i], sv[2 * i + 1]);
    if (!rc) rc = add(ammsb_handle::kTNeighbors, sv[2 * i + 1], sv[2 * i + 2]);
    if (rc) return rc;
  }
  h->timers[ammsb_handle::kTMiniBatch].ticks += (uint64_t)n;
  h->timers[ammsb_handle::kTPi].ticks += (uint64_t)n;
  h->timers[ammsb_handle::kTBeta].ticks += (uint64_t)n;
  return AMMSB_OK;
}

// Reads every pending timed launch (all of them, or those up to and
// including the one that used event set (n, s)).
int drain_phase_events(ammsb_handle* h, int n = 0, int s = -1) {
  size_t upto = h->pending.size();
  if (s >= 0) {
    upto = 0;
    for (size_t q = 0; q < h->pending.size(); ++q)
      if (h->pending[q].n == n && h->pending[q].s == s) upto = q + 1;
  }
  for (size_t q = 0; q < upto; ++q) {
    int rc = read_phase_events(h, h->pending[q].n, h->pending[q].s);
    if (rc) return rc;
  }
  h->pending.erase(h->pending.begin(), h->pending.begin() + (long)upto);
  return AMMSB_OK;
}

// Node ticks of sample_neighbor_nodes and update_phi (the reference ticks
// them once per minibatch node): the edge evaluations the device counted
// since the last call, over n_out.
int count_node_ticks(ammsb_handle* h) {
  DevCounters gc;
  CK(cudaMemcpyAsync(&gc, h->gc, sizeof(gc), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  const uint64_t nodes = (gc.evals - h->evals_read) / (uint64_t)h->m.n_out;
  h->timers[ammsb_handle::kTNeighbors].ticks += nodes;
  h->timers[ammsb_handle::kTPhi].ticks += nodes;
  h->evals_read = gc.evals;
  return AMMSB_OK;
}

// PrintStats (mcmc_sampler_stochastic.cc:185-198) in the reference Timer's
// tabular layout (timer.cc:18-53): name, total seconds, ticks, microseconds
// per tick; "<unused>" for a timer that never ticked.
void print_stats(const ammsb_handle* h) {
  static const char* names[ammsb_handle::kTimers] = {
      "  outer", "  perplexity", "  sample_mini_batch", "  nodes_in_mini_batch",
      "  sample_neighbor_nodes", "  update_phi", "  update_pi", "  update_beta"};
  std::printf("%-37s%13s%9s%15s\n", "timer", "total (s)", "ticks", "per tick (us)");
  for (int t = 0; t < ammsb_handle::kTimers; ++t) {
    const auto& x = h->timers[t];
    if (x.ticks == 0) {
      std::printf("%-36s<unused>\n", names[t]);
    } else {
      // the total is whole milliseconds, as the reference truncates it
      std::printf("%-36s %12.3f %8llu %14.3f\n", names[t], std::floor(x.seconds * 1e3) / 1e3,
                  (unsigned long long)x.ticks, x.seconds * 1e6 / (double)x.ticks);
    }
  }
  std::fflush(stdout);
}

int check_device_err(ammsb_handle* h) {
  DevCounters gc;
  CK(cudaMemcpyAsync(&gc, h->gc, sizeof(gc), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (gc.err) {
    h->err = "device error bits " + std::to_string(gc.err) +
             " (1 minibatch cap, 2 neighbour cap, 4 capacity, 8 init cap)";
    if (gc.err & kErrCapacity) return AMMSB_E_CAPACITY;
    return AMMSB_E_SAMPLING;
  }
  return AMMSB_OK;
}

// Drops draws made ahead of time (their step no longer follows) and points
// the device's next draw at the host's step_count.
int invalidate_prefetch(ammsb_handle* h) {
  if (h->ahead == 0) return AMMSB_OK;
  h->ahead = 0;
  uint32_t s = (uint32_t)h->step_count;
  CK(cudaMemcpyAsync(&h->gc->next_step, &s, sizeof(s), cudaMemcpyHostToDevice, h->stream));
  return AMMSB_OK;
}

int reset_counters(ammsb_handle* h) {
  h->step_count = 1;
  h->average_count = 1;
  h->ppx_history.clear();
  h->slot = 0;
  h->ahead = 0;
  h->last = -1;
  DevCounters gc{};
  gc.next_step = 1;
  CK(cudaMemcpyAsync(h->gc, &gc, sizeof(gc), cudaMemcpyHostToDevice, h->stream));
  for (int p = 0; p < kRing; ++p) CK(cudaMemsetAsync(h->bufs[p].st, 0, sizeof(DevState), h->stream));
  CK(cudaMemsetAsync(h->d_ppx, 0, sizeof(float) * std::max<int64_t>(h->H, 1), h->stream));
  return AMMSB_OK;
}

void choose_config(ammsb_handle* h) {
  const int ev = (h->opt.pi_dtype == AMMSB_PI_BF16) ? 8 : 4;
  const int nvec = h->m.Kp / ev;
  KernelCfg c{};
  if (nvec <= 32) {
    c.lpn = std::min(32, next_pow2(nvec));
    c.vpl = 1;
  } else {
    c.lpn = 32;
    c.vpl = next_pow2((nvec + 31) / 32);
  }
  // rows narrower than a warp: sub-groups split a node's neighbours until
  // the node has a warp (K = 32 BF16: 4 lanes x 8 sub-groups), so that a
  // minibatch of a few hundred nodes still spreads over the SMs
  c.split = (c.lpn == 32) ? (c.vpl >= 2 ? 4 : 2) : std::min(8, 32 / c.lpn);
  c.ring = (c.lpn == 32) ? 1 : 0;
  c.ring_stages = (h->opt.pi_dtype == AMMSB_PI_BF16) ? 4 : 3;  // fastest ring depths on GB300
  c.ring_few = 1;
  if (const char* env = std::getenv("AMMSB_PHI_FEW")) c.ring_few = std::atoi(env) != 0;
  // the many-node ring launch: 16 CTAs per SM (four waves of the four that
  // fit an SM), each walking its node slots; a link-stratum iteration, which
  // leaves this launch idle, then starts 2,432 empty CTAs on a GB300 instead
  // of one per node slot (4,097 at m = 4,096): 0.6% less time per BF16
  // iteration on the 4M-node workload; fewer CTAs (12 or 14 per SM) were
  // slower (uneven node counts per CTA)
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device) != cudaSuccess || sms < 1)
    sms = 152;
  c.ring_grid = 16 * sms;
  if (const char* env = std::getenv("AMMSB_PHI_GRID")) c.ring_grid = std::max(0, std::atoi(env));
  // early starts of update_phi after theta and of theta after the commit:
  // 1.7% less time per BF16 iteration on the 4M-node workload (1.6% on the
  // 100k-node one); the commit's early start measured no gain
  c.pdl = kPdlPhi | kPdlTheta;
  if (const char* env = std::getenv("AMMSB_PDL")) c.pdl = std::atoi(env) & (kPdlPhi | kPdlCommit | kPdlTheta);
  c.graph_pairs = 8;
  if (const char* env = std::getenv("AMMSB_GRAPH_PAIRS")) c.graph_pairs = std::max(1, std::min(64, std::atoi(env)));
  if (const char* env = std::getenv("AMMSB_PHI_KERNEL")) {  // "ring" or "regs"
    if (std::strcmp(env, "regs") == 0) c.ring = 0;
  }
  if (const char* env = std::getenv("AMMSB_PHI_RING")) {  // ring stages
    int st = 0;
    if (std::sscanf(env, "%d", &st) == 1) c.ring_stages = st;
  }
  c.npb = std::max(1, 128 / (c.lpn * c.split));
  c.ppx_lpn = c.lpn;
  c.ppx_vpl = c.vpl;
  c.kq = std::max(1, next_pow2((h->m.Kp + 127) / 128));
  h->cfg = c;
}

}  // namespace

namespace ammsb_detail {
int check_device_err(ammsb_handle* h) { return ::check_device_err(h); }
int invalidate_prefetch(ammsb_handle* h) { return ::invalidate_prefetch(h); }
}  // namespace ammsb_detail

extern "C" {

void ammsb_options_default(ammsb_options* o) {
  std::memset(o, 0, sizeof(*o));
  o->alpha = 0.0;
  o->eta0 = 1.0;
  o->eta1 = 1.0;
  o->epsilon = 0.0000001;
  o->a = 0.0;
  o->b = 1024;
  o->c = 0.5;
  o->K = 300;
  o->mini_batch_size = 0;
  o->num_node_sample = 0;
  o->strategy = AMMSB_STRATIFIED_RANDOM_NODE;
  o->sampler_max_source = 1;
  o->max_iteration = 10000000;
  o->interval = 0;
  o->stats_print_interval = 0;
  o->num_updates = 1000;
  o->held_out_ratio = 0.0;
  o->random_seed = 42;
  o->convergence_threshold = 0.000000000001;
  o->pi_dtype = AMMSB_PI_F32;
  o->chain = 0;
  o->device = 0;
  o->use_graph = 1;
  o->verbose = 0;
  o->pipeline = 1;
}

const char* ammsb_create_error(void) { return g_create_error.c_str(); }

const char* ammsb_last_error(const ammsb_handle* h) { return h ? h->err.c_str() : "null handle"; }

void ammsb_destroy(ammsb_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  for (auto* set : {h->graph1, h->graph2, h->graph1t, h->graph2t, h->graphL})
    for (int s = 0; s < kRing; ++s)
      if (set[s]) cudaGraphExecDestroy(set[s]);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->side) cudaStreamSynchronize(h->side);
  for (auto& per_n : h->ev_phase)
    for (auto& set : per_n)
      for (auto& e : set)
        if (e) cudaEventDestroy(e);
  for (void* p : h->allocs) cudaFree(p);
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  if (h->side) cudaStreamDestroy(h->side);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

int ammsb_create(const ammsb_options* opt_in, const ammsb_graph* graph,
                 const ammsb_edge_set* held_out, const ammsb_edge_set* test,
                 ammsb_handle** out) {
  g_create_error.clear();
  auto fail = [](const std::string& msg, int code) {
    g_create_error = msg;
    return code;
  };
  if (!opt_in || !graph || !out) return fail("null argument", AMMSB_E_ARG);
  *out = nullptr;
  ammsb_options o = *opt_in;
  const int64_t N = graph->n;
  if (N < 2 || N > INT32_MAX || !graph->row_ptr || (!graph->col && graph->row_ptr[N] > 0))
    return fail("graph: need 2 <= n <= 2^31-1 and CSR arrays", AMMSB_E_ARG);
  if (o.K < 1 || o.K > 1024) return fail("K must be in [1, 1024]", AMMSB_E_ARG);
  if (o.strategy < 0 || o.strategy > 3) return fail("Invalid sampling strategy", AMMSB_E_ARG);
  if (o.sampler_max_source < 1 || o.sampler_max_source > 2048)
    return fail("sampler.max-source must be in [1, 2048]", AMMSB_E_ARG);
  if (o.pi_dtype != AMMSB_PI_F32 && o.pi_dtype != AMMSB_PI_BF16)
    return fail("pi_dtype must be AMMSB_PI_F32 or AMMSB_PI_BF16", AMMSB_E_ARG);
  // derived defaults: options.h:257-262, learner.cc:88-92, cc:15-24, 35-44
  if (o.a == 0.0) o.a = std::pow(o.b, -o.c);
  if (o.alpha == 0.0) o.alpha = 1.0 / (double)o.K;
  if (o.held_out_ratio == 0.0) o.held_out_ratio = 0.1;
  if (o.interval == 0) o.interval = 50;
  if (o.stats_print_interval == 0) o.stats_print_interval = 64 * 1024;
  if (o.num_node_sample == 0) o.num_node_sample = N / 50;
  if (o.mini_batch_size == 0) o.mini_batch_size = N / 10;
  if (o.num_node_sample < 1 || o.num_node_sample + 1 > N - 1)
    return fail("num_node_sample must be in [1, N-2]", AMMSB_E_ARG);
  if (o.mini_batch_size < 1 || o.mini_batch_size > (1 << 24) ||
      (o.strategy != AMMSB_RANDOM_EDGE && o.mini_batch_size > N - 1))
    return fail("mini_batch_size must be in [1, 2^24] (and <= N-1 for node strategies)", AMMSB_E_ARG);
  if (o.b <= 0 || o.epsilon <= 0 || o.epsilon >= 1) return fail("invalid b or epsilon", AMMSB_E_ARG);

  // validate the CSR: monotone row_ptr, ids in range, sorted rows, no self loops
  const int64_t nnz = graph->row_ptr[N];
  if (graph->row_ptr[0] != 0 || nnz < 0 || (nnz & 1)) return fail("graph: bad row_ptr", AMMSB_E_ARG);
  int64_t maxdeg = 0;
  for (int64_t v = 0; v < N; ++v) {
    const int64_t r0 = graph->row_ptr[v], r1 = graph->row_ptr[v + 1];
    if (r1 < r0 || r1 > nnz) return fail("graph: row_ptr not monotone", AMMSB_E_ARG);
    maxdeg = std::max(maxdeg, r1 - r0);
    for (int64_t q = r0; q < r1; ++q) {
      const int32_t c = graph->col[q];
      if (c < 0 || c >= N || c == v || (q > r0 && graph->col[q - 1] >= c))
        return fail("graph: rows must be sorted, in range, without self-loops", AMMSB_E_ARG);
    }
  }
  auto check_set = [&](const ammsb_edge_set* s) {
    if (!s || s->count == 0) return true;
    if (s->count < 0 || !s->a || !s->b || !s->y) return false;
    for (int64_t i = 0; i < s->count; ++i)
      if (s->a[i] < 0 || s->b[i] < 0 || s->a[i] >= N || s->b[i] >= N || s->a[i] == s->b[i])
        return false;
    return true;
  };
  if (!check_set(held_out) || !check_set(test)) return fail("held-out/test sets: bad pairs", AMMSB_E_ARG);

  auto* h = new ammsb_handle();
  h->opt = o;
  h->device = o.device;
  h->E = nnz / 2;
  h->H = held_out ? held_out->count : 0;
  h->T = test ? test->count : 0;
  auto bail = [&](int code) {
    g_create_error = h->err;
    ammsb_destroy(h);
    return code;
  };
  if (cudaSetDevice(o.device) != cudaSuccess) {
    h->err = "cudaSetDevice failed (no CUDA device?)";
    return bail(AMMSB_E_CUDA);
  }
  // the draws of the iterations ahead get the higher priority, so their
  // short launches go in as the update's CTAs retire (graphs keep it: they
  // are instantiated with node priorities)
  int prio_lo = 0, prio_hi = 0;
  cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithPriority(&h->side, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) != cudaSuccess) {
    h->err = "cudaStreamCreate / cudaEventCreate failed";
    return bail(AMMSB_E_CUDA);
  }
  const int K = (int)o.K;
  h->pi_bytes = (o.pi_dtype == AMMSB_PI_BF16) ? 2 : 4;
  const int Kp = (o.pi_dtype == AMMSB_PI_BF16) ? ((K + 7) / 8) * 8 : ((K + 3) / 4) * 4;
  Model& m = h->m;
  m.K = K;
  m.Kp = Kp;
  m.N = N;
  m.alpha = (float)o.alpha;
  m.epsilon = (float)o.epsilon;
  m.Nn = (1.0f * (float)N) / (float)o.num_node_sample;
  m.eta0 = (float)o.eta0;
  m.eta1 = (float)o.eta1;
  m.a = o.a;
  m.b = o.b;
  m.c = o.c;
  m.seed = (uint32_t)o.random_seed;
  m.chain = (uint32_t)o.chain;
  m.n_out = (int32_t)o.num_node_sample + 1;
  // minibatch capacities (network.cc:172-201): one source's star for the
  // stratified strategies; m + max degree with several link sources; m
  // edges for random-edge, or the whole training set when m reaches it
  // (E - |held-out| - |test|, network.cc:238-241)
  const bool multi_src = o.sampler_max_source > 1;
  const bool rand_edge = o.strategy == AMMSB_RANDOM_EDGE;
  m.full_set = (rand_edge && o.mini_batch_size >= h->E - h->H - h->T) ? 1 : 0;
  int64_t max_edges = std::max<int64_t>(o.mini_batch_size, std::max<int64_t>(maxdeg, 1));
  if (multi_src) max_edges = o.mini_batch_size + std::max<int64_t>(maxdeg, 1);
  if (rand_edge) max_edges = m.full_set ? std::max<int64_t>(h->E, 1) : o.mini_batch_size;
  if (max_edges > (1 << 28)) {
    h->err = "minibatch capacity too large";
    return bail(AMMSB_E_CAPACITY);
  }
  if (rand_edge && nnz >= (int64_t)INT32_MAX) {
    h->err = "random-edge needs fewer than 2^30 edges";
    return bail(AMMSB_E_UNSUPPORTED);
  }
  m.max_edges = (int32_t)max_edges;
  m.max_nodes = (multi_src || rand_edge) ? (int32_t)std::min<int64_t>(N, 2 * max_edges + 1)
                                         : (int32_t)(max_edges + 1);
  m.max_source = (int32_t)o.sampler_max_source;
  m.n_entries = nnz;
  m.mini_batch_size = (int32_t)o.mini_batch_size;
  m.strategy = o.strategy;
  {  // network.cc:341-342 with Float = float
    float scale = (float)N * (float)N / (float)o.mini_batch_size;
    scale = (float)((double)scale * ((double)h->E / ((double)N * ((double)N - 1.0) / 2.0 - (double)h->E)));
    m.nonlink_scale = scale;
    m.link_scale = (float)N;  // network.cc:386-387, max-source 1
  }
  m.nbb = (int)std::min<int64_t>(kMaxBetaBlocks, std::max<int64_t>(1, (max_edges + 3) / 4));
  choose_config(h);
  if (h->cfg.vpl > 8) {
    h->err = "K too large for the row kernels";
    return bail(AMMSB_E_ARG);
  }

  Buffers& b = h->b;
  DevGraph& g = h->g;
  int rc = AMMSB_OK;
  int64_t* d_row = nullptr;
  int32_t* d_col = nullptr;
#define TRY(x)                   \
  do {                           \
    rc = (x);                    \
    if (rc != AMMSB_OK) return bail(rc); \
  } while (0)
  TRY(dev_alloc(h, &d_row, N + 1));
  TRY(dev_alloc(h, &d_col, std::max<int64_t>(nnz, 1)));
  if (cudaMemcpyAsync(d_row, graph->row_ptr, sizeof(int64_t) * (N + 1), cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
      (nnz > 0 && cudaMemcpyAsync(d_col, graph->col, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, h->stream) != cudaSuccess)) {
    h->err = "graph upload failed";
    return bail(AMMSB_E_CUDA);
  }
  g.n = N;
  g.row_ptr = d_row;
  g.col = d_col;
  {  // held-out + test exclusion hash
    const int64_t nex = h->H + h->T;
    const int cap = next_pow2(std::max<int64_t>(16, 2 * nex));
    std::vector<unsigned long long> keys(cap, kEmptyKey);
    auto insert = [&](const ammsb_edge_set* s) {
      if (!s) return;
      for (int64_t i = 0; i < s->count; ++i) {
        unsigned long long k = pair_key(s->a[i], s->b[i]);
        uint32_t slot = hash64(k) & (uint32_t)(cap - 1);
        while (keys[slot] != kEmptyKey && keys[slot] != k) slot = (slot + 1) & (uint32_t)(cap - 1);
        keys[slot] = k;
      }
    };
    insert(held_out);
    insert(test);
    unsigned long long* d_ex = nullptr;
    TRY(dev_alloc(h, &d_ex, cap));
    if (cudaMemcpyAsync(d_ex, keys.data(), sizeof(unsigned long long) * cap, cudaMemcpyHostToDevice, h->stream) != cudaSuccess) {
      h->err = "exclusion upload failed";
      return bail(AMMSB_E_CUDA);
    }
    g.excl = d_ex;
    g.excl_mask = (uint32_t)(cap - 1);
  }
  // held-out set for perplexity
  TRY(dev_alloc(h, &h->d_ha, std::max<int64_t>(h->H, 1)));
  TRY(dev_alloc(h, &h->d_hb, std::max<int64_t>(h->H, 1)));
  TRY(dev_alloc(h, &h->d_hy, std::max<int64_t>(h->H, 1)));
  TRY(dev_alloc(h, &h->d_ppx, std::max<int64_t>(h->H, 1)));
  if (h->H > 0) {
    if (cudaMemcpyAsync(h->d_ha, held_out->a, sizeof(int32_t) * h->H, cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
        cudaMemcpyAsync(h->d_hb, held_out->b, sizeof(int32_t) * h->H, cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
        cudaMemcpyAsync(h->d_hy, held_out->y, h->H, cudaMemcpyHostToDevice, h->stream) != cudaSuccess) {
      h->err = "held-out upload failed";
      return bail(AMMSB_E_CUDA);
    }
  }
  {
    const int gpb = 256 / h->cfg.ppx_lpn;
    h->ppx_blocks = (int)std::max<int64_t>(1, std::min<int64_t>((h->H + gpb - 1) / gpb, 152 * 8));
  }
  TRY(dev_alloc(h, &h->d_ppx_part, 2 * (size_t)h->ppx_blocks));
  TRY(dev_alloc(h, &h->d_ppx_out, 1));
  // model state
  void* d_pi = nullptr;
  {
    void* q = nullptr;
    const size_t bytes = (size_t)N * Kp * h->pi_bytes;
    if (cudaMalloc(&q, bytes) != cudaSuccess) {
      h->err = "cudaMalloc pi failed";
      return bail(AMMSB_E_CUDA);
    }
    h->allocs.push_back(q);
    cudaMemsetAsync(q, 0, bytes, h->stream);
    d_pi = q;
  }
  b.pi = d_pi;
  TRY(dev_alloc(h, &b.phi, (size_t)N * Kp));
  TRY(dev_alloc(h, &b.stage, (size_t)m.max_nodes * Kp));
  TRY(dev_alloc(h, &b.beta, (size_t)Kp));
  TRY(dev_alloc(h, &b.theta, 2 * (size_t)K));
  for (int p = 0; p < kRing; ++p) {  // the ring of minibatch buffer sets
    Buffers& bp = h->bufs[p];
    TRY(dev_alloc(h, &bp.nodes, (size_t)m.max_nodes));
    TRY(dev_alloc(h, &bp.ea, (size_t)m.max_edges));
    TRY(dev_alloc(h, &bp.eb, (size_t)m.max_edges));
    TRY(dev_alloc(h, &bp.ey, (size_t)m.max_edges));
    TRY(dev_alloc(h, &bp.nbr, (size_t)m.max_nodes * m.n_out));
    TRY(dev_alloc(h, &bp.st, 1));
  }
  // a minibatch round examines up to max(remaining, 4096) candidates while
  // the dedup hash stays at most half full
  TRY(dev_alloc(h, &b.cand, (size_t)std::max<int64_t>(o.mini_batch_size, 4096)));
  // ... and numbers the nodes of a general edge list (random-edge, several
  // link sources) in the same table: at most max_nodes distinct vertices
  int64_t hneed = std::max<int64_t>(8192, 2 * o.mini_batch_size);
  if (multi_src || rand_edge) hneed = std::max<int64_t>(hneed, 2 * (int64_t)m.max_nodes);
  const int hcap = next_pow2(hneed);
  TRY(dev_alloc(h, &b.htab_key, (size_t)hcap));
  TRY(dev_alloc(h, &b.htab_idx, (size_t)hcap));
  b.hmask = (uint32_t)(hcap - 1);
  // the dedup hash lives in shared memory when it fits (up to 16Ki entries)
  if (hcap <= 16384 &&
      ammsb_detail::raise_smem_limit(k_sample_minibatch, 2 * sizeof(uint32_t) * hcap) == cudaSuccess)
    h->mb_smem = 2 * sizeof(uint32_t) * (size_t)hcap;
  TRY(dev_alloc(h, &b.beta_part, (size_t)m.nbb * 2 * Kp));
  TRY(dev_alloc(h, &h->gc, 1));
  b.gc = h->gc;
  TRY(dev_alloc(h, &h->d_err_init, 1));
  TRY(dev_alloc(h, &h->d_fed_phi_noise, (size_t)m.max_nodes * K));
  TRY(dev_alloc(h, &h->d_fed_theta_noise, 2 * (size_t)K));
  b.fed_phi_noise = nullptr;
  b.fed_theta_noise = nullptr;
  for (int p = 0; p < kRing; ++p) {  // shared state + this set's minibatch arrays
    Buffers own = h->bufs[p];
    h->bufs[p] = b;
    h->bufs[p].nodes = own.nodes;
    h->bufs[p].ea = own.ea;
    h->bufs[p].eb = own.eb;
    h->bufs[p].ey = own.ey;
    h->bufs[p].nbr = own.nbr;
    h->bufs[p].st = own.st;
  }
  b.nodes = nullptr;
  b.ea = b.eb = nullptr;
  b.ey = nullptr;
  b.nbr = nullptr;
  b.st = nullptr;
#undef TRY
  // commit blocks (4 rows each, grid-strided): two per SM, so an iteration
  // of few nodes does not launch a thousand idle blocks
  h->ncommit = (int)std::max<int64_t>(1, std::min<int64_t>((m.max_nodes + 3) / 4, 152 * 2));
  // neighbour blocks (8 warps, one node each, grid-strided): a warp more
  // than the nodes, so the last one, which computes eps_t, has none
  h->nbr_blocks = (int)std::max<int64_t>(1, std::min<int64_t>((m.max_nodes + 8) / 8, 152 * 8));
  h->m.nbr_set_cap = next_pow2(std::max<int64_t>(64, 2 * (int64_t)m.n_out));
  h->nbr_smem = (size_t)8 * h->m.nbr_set_cap * sizeof(int32_t);
  if (h->nbr_smem > 48 * 1024) {
    if (ammsb_detail::raise_smem_limit(k_sample_neighbors<8>, h->nbr_smem) != cudaSuccess) {
      h->err = "num_node_sample too large for the neighbour kernel";
      return bail(AMMSB_E_ARG);
    }
  }
  if (h->cfg.ring) {
    cudaError_t e = (o.pi_dtype == AMMSB_PI_BF16) ? launch_phi_ring<__nv_bfloat16>(h, h->b, true)
                                                   : launch_phi_ring<float>(h, h->b, true);
    if (e != cudaSuccess) {
      h->err = std::string("update_phi shared memory configuration: ") + cudaGetErrorString(e);
      return bail(AMMSB_E_CUDA);
    }
  }
  if (reset_counters(h) != AMMSB_OK) return bail(AMMSB_E_CUDA);
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) {
    h->err = std::string("create: ") + cudaGetErrorString(cudaGetLastError());
    return bail(AMMSB_E_CUDA);
  }
  if (o.verbose) {
    std::fprintf(stderr, "N %lld E %lld K %d\nminibatch size %lld epsilon %g alpha %g iterations %lld\n",
                 (long long)N, (long long)h->E, K, (long long)o.mini_batch_size, o.epsilon, o.alpha,
                 (long long)o.max_iteration);
    std::fprintf(stderr, "num_node_sample %lld\na %g b %g c %g eta (%g,%g)\n",
                 (long long)o.num_node_sample, o.a, o.b, o.c, o.eta0, o.eta1);
    std::fprintf(stderr, "update_phi lanes/node %d vec/lane %d split %d %s; pi %s\n", h->cfg.lpn,
                 h->cfg.vpl, h->cfg.split, h->cfg.ring ? "shared-memory ring" : "register path",
                 o.pi_dtype == AMMSB_PI_BF16 ? "bf16" : "f32");
  }
  *out = h;
  return AMMSB_OK;
}

int ammsb_init_state(ammsb_handle* h) {
  if (!h) return AMMSB_E_ARG;
  CK(cudaSetDevice(h->device));
  const int K = h->m.K;
  const Stream rs{h->m.seed, h->m.chain};
  std::vector<double> theta(2 * (size_t)K);
  std::vector<float> beta(h->m.Kp, 0.f);
  for (int k = 0; k < K; ++k) {  // theta = gamma(eta0, eta1, K, 2), cc:54
    theta[2 * k] = host_gamma(rs, kTagThetaInit, 0, 2ull * k, h->opt.eta0, h->opt.eta1);
    theta[2 * k + 1] = host_gamma(rs, kTagThetaInit, 0, 2ull * k + 1, h->opt.eta0, h->opt.eta1);
    beta[k] = (float)(theta[2 * k + 1] / (theta[2 * k] + theta[2 * k + 1]));
  }
  CK(cudaMemcpyAsync(h->b.theta, theta.data(), sizeof(double) * 2 * K, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->b.beta, beta.data(), sizeof(float) * h->m.Kp, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemsetAsync(h->d_err_init, 0, sizeof(int32_t), h->stream));
  const int64_t total = h->m.N * (int64_t)h->m.Kp;
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 152 * 64));
  k_init_phi<<<blocks, 256, 0, h->stream>>>(h->m, h->b.phi, 1.0, 1.0, h->d_err_init);  // cc:66
  CK(cudaGetLastError());
  CK(launch_normalize(h));
  int rc = reset_counters(h);
  if (rc) return rc;
  int32_t err = 0;
  CK(cudaMemcpyAsync(&err, h->d_err_init, sizeof(err), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (err) {
    h->err = "gamma initialisation hit its rejection cap";
    return AMMSB_E_SAMPLING;
  }
  h->state_ready = true;
  return AMMSB_OK;
}

int ammsb_set_state(ammsb_handle* h, const float* phi, const double* theta) {
  if (!h || !phi || !theta) return AMMSB_E_ARG;
  CK(cudaSetDevice(h->device));
  const int K = h->m.K, Kp = h->m.Kp;
  for (int64_t x = 0; x < h->m.N * (int64_t)K; ++x)
    if (!(phi[x] > 0.f) || !std::isfinite(phi[x])) {
      h->err = "phi must be positive and finite";
      return AMMSB_E_ARG;
    }
  std::vector<float> beta(Kp, 0.f);
  for (int k = 0; k < K; ++k) {
    if (!(theta[2 * k] > 0) || !(theta[2 * k + 1] > 0)) {
      h->err = "theta must be positive";
      return AMMSB_E_ARG;
    }
    beta[k] = (float)(theta[2 * k + 1] / (theta[2 * k] + theta[2 * k + 1]));
  }
  CK(cudaMemcpy2DAsync(h->b.phi, sizeof(float) * Kp, phi, sizeof(float) * K, sizeof(float) * K, h->m.N,
                       cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->b.theta, theta, sizeof(double) * 2 * K, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->b.beta, beta.data(), sizeof(float) * Kp, cudaMemcpyHostToDevice, h->stream));
  CK(launch_normalize(h));
  int rc = reset_counters(h);
  if (rc) return rc;
  CK(cudaStreamSynchronize(h->stream));
  h->state_ready = true;
  return AMMSB_OK;
}

int ammsb_set_step(ammsb_handle* h, uint64_t step_count) {
  if (!h || step_count < 1 || step_count > 0xffffffffull) return AMMSB_E_ARG;
  CK(cudaSetDevice(h->device));
  h->step_count = step_count;
  h->ahead = 0;
  uint32_t s = (uint32_t)step_count;
  CK(cudaMemcpyAsync(&h->gc->next_step, &s, sizeof(s), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return AMMSB_OK;
}

int ammsb_step(ammsb_handle* h, int64_t n_iters) {
  if (!h || n_iters < 0) return AMMSB_E_ARG;
  if (!h->state_ready) {
    h->err = "call ammsb_init_state or ammsb_set_state first";
    return AMMSB_E_STATE;
  }
  CK(cudaSetDevice(h->device));
  if (n_iters == 0) return AMMSB_OK;
  // the draws of the next two iterations, where they are not made yet
  while (h->opt.pipeline && h->ahead < 2) {
    CK(launch_sampling_phase(h, h->bufs[(h->slot + h->ahead) % kRing], h->stream));
    ++h->ahead;
  }
  auto launch = [&](int s, int n, const cudaEvent_t* ev) {
    return h->opt.pipeline ? launch_pipelined(h, s, n, ev) : launch_serial(h, s, n, ev);
  };
  int64_t left = n_iters;
  while (left > 0) {
    // long graphs: graph_pairs pipelined pairs per launch, so that every
    // update but the launch's first follows a theta step inside the graph
    // (and may start early), with fewer graph launches
    const int L = h->cfg.graph_pairs;
    if (L > 1 && h->opt.use_graph && h->opt.pipeline && !h->timing && left >= 2 * (int64_t)L) {
      const int s = h->slot;
      cudaGraphExec_t& g = h->graphL[s];
      if (!g) {
        cudaGraph_t graph;
        CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaSuccess;
        for (int j = 0; j < L && e == cudaSuccess; ++j) e = launch_pipelined(h, (s + 2 * j) % kRing, 2, nullptr, j > 0);
        cudaError_t e2 = cudaStreamEndCapture(h->stream, &graph);
        if (e != cudaSuccess || e2 != cudaSuccess) {
          h->err = std::string("graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2);
          return AMMSB_E_CUDA;
        }
        CK(cudaGraphInstantiate(&g, graph, cudaGraphInstantiateFlagUseNodePriority));
        cudaGraphDestroy(graph);
      }
      CK(cudaGraphLaunch(g, h->stream));
      h->last = (s + 2 * L - 1) % kRing;
      h->slot = (s + 2 * L) % kRing;
      left -= 2 * L;
      continue;
    }
    const int n = left >= 2 ? 2 : 1;
    const int s = h->slot;
    // run()'s timers: the launch records events between the phases; the
    // events of an earlier launch with the same event set are read first
    const cudaEvent_t* ev = nullptr;
    if (h->timing) {
      cudaEvent_t* set = h->ev_phase[n - 1][s];
      if (!set[0])
        for (int q = 0; q < 12; ++q) CK(cudaEventCreate(&set[q]));
      int rc = drain_phase_events(h, n, s);
      if (rc) return rc;
      ev = set;
    }
    if (h->opt.use_graph) {
      cudaGraphExec_t& g = h->timing ? ((n == 2) ? h->graph2t[s] : h->graph1t[s])
                                     : ((n == 2) ? h->graph2[s] : h->graph1[s]);
      if (!g) {
        cudaGraph_t graph;
        CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = launch(s, n, ev);
        cudaError_t e2 = cudaStreamEndCapture(h->stream, &graph);
        if (e != cudaSuccess || e2 != cudaSuccess) {
          h->err = std::string("graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2);
          return AMMSB_E_CUDA;
        }
        CK(cudaGraphInstantiate(&g, graph, cudaGraphInstantiateFlagUseNodePriority));
        cudaGraphDestroy(graph);
      }
      CK(cudaGraphLaunch(g, h->stream));
    } else {
      CK(launch(s, n, ev));
    }
    if (h->timing) h->pending.push_back({n, s});
    h->last = (s + n - 1) % kRing;
    h->slot = (s + n) % kRing;
    left -= n;
  }
  h->step_count += (uint64_t)n_iters;
  return AMMSB_OK;
}

int ammsb_step_fed(ammsb_handle* h, uint32_t step, int32_t n_edges, const int32_t* edge_slot_a,
                   const int32_t* edge_slot_b, const uint8_t* edge_y, float scale, int32_t n_nodes,
                   const int32_t* nodes, const int32_t* nbrs, const uint8_t* nbr_y,
                   const float* phi_noise, const float* theta_noise) {
  if (!h || n_edges < 0 || n_nodes < 1 || !nodes || !nbrs || !nbr_y || !phi_noise || !theta_noise ||
      (n_edges > 0 && (!edge_slot_a || !edge_slot_b || !edge_y)))
    return AMMSB_E_ARG;
  if (!h->state_ready) {
    h->err = "call ammsb_init_state or ammsb_set_state first";
    return AMMSB_E_STATE;
  }
  if (n_edges > h->m.max_edges || n_nodes > h->m.max_nodes) {
    h->err = "fed minibatch exceeds the handle's buffers";
    return AMMSB_E_CAPACITY;
  }
  const int n_out = h->m.n_out, K = h->m.K;
  for (int32_t s = 0; s < n_nodes; ++s)
    if (nodes[s] < 0 || nodes[s] >= h->m.N) {
      h->err = "fed node id out of range";
      return AMMSB_E_ARG;
    }
  for (int32_t e = 0; e < n_edges; ++e)
    if (edge_slot_a[e] < 0 || edge_slot_a[e] >= n_nodes || edge_slot_b[e] < 0 || edge_slot_b[e] >= n_nodes) {
      h->err = "fed edge slot out of range";
      return AMMSB_E_ARG;
    }
  std::vector<uint32_t> packed((size_t)n_nodes * n_out);
  for (size_t q = 0; q < packed.size(); ++q) {
    if (nbrs[q] < 0 || nbrs[q] >= h->m.N) {
      h->err = "fed neighbour id out of range";
      return AMMSB_E_ARG;
    }
    packed[q] = (uint32_t)nbrs[q] | ((nbr_y[q] ? 1u : 0u) << 31);
  }
  CK(cudaSetDevice(h->device));
  int rc0 = invalidate_prefetch(h);
  if (rc0) return rc0;
  const Buffers& bp = h->bufs[h->slot];
  CK(cudaMemcpyAsync(bp.nodes, nodes, sizeof(int32_t) * n_nodes, cudaMemcpyHostToDevice, h->stream));
  if (n_edges > 0) {
    CK(cudaMemcpyAsync(bp.ea, edge_slot_a, sizeof(int32_t) * n_edges, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(bp.eb, edge_slot_b, sizeof(int32_t) * n_edges, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(bp.ey, edge_y, n_edges, cudaMemcpyHostToDevice, h->stream));
  }
  CK(cudaMemcpyAsync(bp.nbr, packed.data(), sizeof(uint32_t) * packed.size(), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->d_fed_phi_noise, phi_noise, sizeof(float) * (size_t)n_nodes * K, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->d_fed_theta_noise, theta_noise, sizeof(float) * 2 * K, cudaMemcpyHostToDevice, h->stream));
  DevState st{};
  st.step = step;
  st.eps = (float)(h->m.a * std::pow(1.0 + (double)step / h->m.b, -h->m.c));
  st.scale = scale;
  st.flag = -1;
  st.n_edges = n_edges;
  st.n_nodes = n_nodes;
  CK(cudaMemcpyAsync(bp.st, &st, sizeof(st), cudaMemcpyHostToDevice, h->stream));
  Buffers fb = bp;
  fb.fed_phi_noise = h->d_fed_phi_noise;
  fb.fed_theta_noise = h->d_fed_theta_noise;
  CK(launch_update_phase(h, fb));
  h->last = h->slot;
  return check_device_err(h);
}

int ammsb_perplexity(ammsb_handle* h, double* out) {
  if (!h || !out) return AMMSB_E_ARG;
  if (!h->state_ready) {
    h->err = "call ammsb_init_state or ammsb_set_state first";
    return AMMSB_E_STATE;
  }
  CK(cudaSetDevice(h->device));
  const float count = (float)h->average_count;
  if (h->H > 0) {
    CK(h->opt.pi_dtype == AMMSB_PI_BF16 ? launch_ppx<__nv_bfloat16>(h, count) : launch_ppx<float>(h, count));
  }
  k_ppx_final<<<1, kPpxFinalThreads, 0, h->stream>>>(h->d_ppx_part, h->H > 0 ? h->ppx_blocks : 0, h->H, h->d_ppx_out);
  CK(cudaGetLastError());
  double v = 0.0;
  CK(cudaMemcpyAsync(&v, h->d_ppx_out, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  int rc = check_device_err(h);  // synchronises
  if (rc) return rc;
  h->average_count++;
  *out = v;
  return AMMSB_OK;
}

int ammsb_run(ammsb_handle* h, double* last) {
  if (!h) return AMMSB_E_ARG;
  if (!h->state_ready) {
    int rc = ammsb_init_state(h);
    if (rc) return rc;
  }
  using clk = std::chrono::steady_clock;
  const auto t0 = std::chrono::system_clock::now();
  double ppx = 0.0;
  auto converged = [&]() {  // learner.cc:130-136
    const size_t n = h->ppx_history.size();
    if (n < 2) return false;
    return std::fabs(h->ppx_history[n - 1] - h->ppx_history[n - 2]) / h->ppx_history[n - 2] <=
           h->opt.convergence_threshold;
  };
  // the timers (cc:95-102) start from zero and time this run
  for (auto& t : h->timers) t = ammsb_handle::Timer{};
  h->pending.clear();
  {
    int rc = count_node_ticks(h);  // node ticks count from here
    if (rc) return rc;
    h->timers[ammsb_handle::kTNeighbors].ticks = h->timers[ammsb_handle::kTPhi].ticks = 0;
  }
  h->timing = true;
  auto finish = [&](int rc) {
    h->timing = false;
    return rc;
  };
  const uint64_t stats_every = (uint64_t)h->opt.stats_print_interval;
  const uint64_t first_step = h->step_count;
  auto outer_start = clk::now();
  // the outer timer: wall time of the iterations (perplexity included), one
  // tick per iteration; brought up to date at every stats print
  auto stats = [&]() -> int {
    int rc = drain_phase_events(h);
    if (!rc) rc = count_node_ticks(h);
    if (rc) return rc;
    const auto now = clk::now();
    h->timers[ammsb_handle::kTOuter].seconds += std::chrono::duration<double>(now - outer_start).count();
    h->timers[ammsb_handle::kTOuter].ticks = h->step_count - first_step;
    outer_start = now;
    print_stats(h);
    outer_start = clk::now();  // printing is not an iteration's time
    return AMMSB_OK;
  };
  while (h->step_count < (uint64_t)h->opt.max_iteration && !converged()) {
    if ((h->step_count - 1) % (uint64_t)h->opt.interval == 0) {
      const auto p0 = clk::now();
      int rc = ammsb_perplexity(h, &ppx);
      if (rc) return finish(rc);
      h->timers[ammsb_handle::kTPerplexity].seconds +=
          std::chrono::duration<double>(clk::now() - p0).count();
      h->timers[ammsb_handle::kTPerplexity].ticks += 1;
      const double secs =
          std::chrono::duration<double>(std::chrono::system_clock::now() - t0).count();
      std::printf("average_count is: %llu step count: %llu time: %.3f perplexity for hold out set: %.12f\n",
                  (unsigned long long)h->average_count, (unsigned long long)h->step_count, secs, ppx);
      std::fflush(stdout);
      h->ppx_history.push_back(ppx);
    }
    // run up to the next perplexity point or stats print, whichever is first
    const uint64_t interval = (uint64_t)h->opt.interval;
    uint64_t until = ((h->step_count - 1) / interval + 1) * interval + 1;
    until = std::min<uint64_t>(until, (h->step_count / stats_every + 1) * stats_every);
    until = std::min<uint64_t>(until, (uint64_t)h->opt.max_iteration);
    const int64_t n = (int64_t)(until - h->step_count);
    int rc = ammsb_step(h, std::max<int64_t>(n, 1));
    if (rc) return finish(rc);
    if (h->step_count % stats_every == 0 && (rc = stats()) != AMMSB_OK) return finish(rc);  // cc:177-179
  }
  int rc = check_device_err(h);
  if (!rc) rc = stats();  // cc:182
  if (rc) return finish(rc);
  if (last) *last = ppx;
  return finish(AMMSB_OK);
}

int ammsb_get_pi(ammsb_handle* h, float* dst) {
  if (!h || !dst) return AMMSB_E_ARG;
  CK(cudaSetDevice(h->device));
  const int K = h->m.K, Kp = h->m.Kp;
  const int64_t N = h->m.N;
  if (h->opt.pi_dtype == AMMSB_PI_F32) {
    CK(cudaMemcpy2DAsync(dst, sizeof(float) * K, h->b.pi, sizeof(float) * Kp, sizeof(float) * K, N,
                         cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
  } else {
    std::vector<uint16_t> tmp((size_t)N * K);
    CK(cudaMemcpy2DAsync(tmp.data(), 2 * K, h->b.pi, 2 * Kp, 2 * K, N, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (size_t x = 0; x < tmp.size(); ++x) {
      uint32_t u = (uint32_t)tmp[x] << 16;
      std::memcpy(dst + x, &u, 4);
    }
  }
  return AMMSB_OK;
}

int ammsb_get_phi(ammsb_handle* h, float* dst) {
  if (!h || !dst) return AMMSB_E_ARG;
  CK(cudaSetDevice(h->device));
  const int K = h->m.K, Kp = h->m.Kp;
  CK(cudaMemcpy2DAsync(dst, sizeof(float) * K, h->b.phi, sizeof(float) * Kp, sizeof(float) * K, h->m.N,
                       cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return AMMSB_OK;
}

int ammsb_get_theta(ammsb_handle* h, double* dst) {
  if (!h || !dst) return AMMSB_E_ARG;
  CK(cudaSetDevice(h->device));
  CK(cudaMemcpyAsync(dst, h->b.theta, sizeof(double) * 2 * h->m.K, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return AMMSB_OK;
}

int ammsb_get_beta(ammsb_handle* h, float* dst) {
  if (!h || !dst) return AMMSB_E_ARG;
  CK(cudaSetDevice(h->device));
  CK(cudaMemcpyAsync(dst, h->b.beta, sizeof(float) * h->m.K, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return AMMSB_OK;
}

int ammsb_get_ppx(ammsb_handle* h, float* dst) {
  if (!h || !dst) return AMMSB_E_ARG;
  CK(cudaSetDevice(h->device));
  if (h->H > 0) CK(cudaMemcpyAsync(dst, h->d_ppx, sizeof(float) * h->H, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return AMMSB_OK;
}

int ammsb_get_step(ammsb_handle* h, uint64_t* step_count, uint64_t* average_count) {
  if (!h) return AMMSB_E_ARG;
  if (step_count) *step_count = h->step_count;
  if (average_count) *average_count = h->average_count;
  return AMMSB_OK;
}

int ammsb_get_last_minibatch(ammsb_handle* h, int32_t* flag, int32_t* n_edges, int32_t* n_nodes,
                             float* scale, int32_t* ea, int32_t* eb, uint8_t* ey, int32_t* nodes,
                             int32_t* nbrs, uint8_t* nbr_y) {
  if (!h) return AMMSB_E_ARG;
  CK(cudaSetDevice(h->device));
  if (h->last < 0) {
    h->err = "no iteration has run yet";
    return AMMSB_E_STATE;
  }
  const Buffers& bl = h->bufs[h->last];
  DevState st;
  DevCounters gc;
  CK(cudaMemcpyAsync(&st, bl.st, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(&gc, h->gc, sizeof(gc), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (flag) *flag = st.flag;
  if (n_edges) *n_edges = st.n_edges;
  if (n_nodes) *n_nodes = st.n_nodes;
  if (scale) *scale = st.scale;
  if (st.n_edges > 0) {
    if (ea) CK(cudaMemcpyAsync(ea, bl.ea, sizeof(int32_t) * st.n_edges, cudaMemcpyDeviceToHost, h->stream));
    if (eb) CK(cudaMemcpyAsync(eb, bl.eb, sizeof(int32_t) * st.n_edges, cudaMemcpyDeviceToHost, h->stream));
    if (ey) CK(cudaMemcpyAsync(ey, bl.ey, st.n_edges, cudaMemcpyDeviceToHost, h->stream));
  }
  if (st.n_nodes > 0) {
    if (nodes) CK(cudaMemcpyAsync(nodes, bl.nodes, sizeof(int32_t) * st.n_nodes, cudaMemcpyDeviceToHost, h->stream));
    if (nbrs || nbr_y) {
      std::vector<uint32_t> packed((size_t)st.n_nodes * h->m.n_out);
      CK(cudaMemcpyAsync(packed.data(), bl.nbr, sizeof(uint32_t) * packed.size(), cudaMemcpyDeviceToHost, h->stream));
      CK(cudaStreamSynchronize(h->stream));
      for (size_t q = 0; q < packed.size(); ++q) {
        if (nbrs) nbrs[q] = (int32_t)(packed[q] & 0x7fffffffu);
        if (nbr_y) nbr_y[q] = (uint8_t)(packed[q] >> 31);
      }
    }
  }
  CK(cudaStreamSynchronize(h->stream));
  if (gc.err) {
    h->err = "device error bits " + std::to_string(gc.err);
    return (gc.err & kErrCapacity) ? AMMSB_E_CAPACITY : AMMSB_E_SAMPLING;
  }
  return AMMSB_OK;
}

int ammsb_get_sizes(ammsb_handle* h, int64_t* N, int64_t* K, int64_t* max_edges, int64_t* max_nodes,
                    int64_t* num_node_sample, int64_t* held_out_count) {
  if (!h) return AMMSB_E_ARG;
  if (N) *N = h->m.N;
  if (K) *K = h->m.K;
  if (max_edges) *max_edges = h->m.max_edges;
  if (max_nodes) *max_nodes = h->m.max_nodes;
  if (num_node_sample) *num_node_sample = h->opt.num_node_sample;
  if (held_out_count) *held_out_count = h->H;
  return AMMSB_OK;
}

int ammsb_get_options(ammsb_handle* h, ammsb_options* out) {
  if (!h || !out) return AMMSB_E_ARG;
  *out = h->opt;
  return AMMSB_OK;
}

int ammsb_profile_step(ammsb_handle* h, double* ms5) {
  if (!h || !ms5) return AMMSB_E_ARG;
  if (!h->state_ready) {
    h->err = "call ammsb_init_state or ammsb_set_state first";
    return AMMSB_E_STATE;
  }
  CK(cudaSetDevice(h->device));
  int rc0 = invalidate_prefetch(h);
  if (rc0) return rc0;
  const Buffers& bp = h->bufs[h->slot];
  cudaEvent_t ev[6];
  for (auto& e : ev) CK(cudaEventCreate(&e));
  CK(cudaEventRecord(ev[0], h->stream));
  k_sample_minibatch<<<1, 1024, h->mb_smem, h->stream>>>(h->m, h->g, bp, h->mb_smem > 0);
  CK(cudaEventRecord(ev[1], h->stream));
  k_sample_neighbors<8><<<h->nbr_blocks, 256, h->nbr_smem, h->stream>>>(h->m, h->g, bp);
  CK(cudaEventRecord(ev[2], h->stream));
  CK(h->opt.pi_dtype == AMMSB_PI_BF16 ? launch_phi<__nv_bfloat16>(h, bp) : launch_phi<float>(h, bp));
  CK(cudaEventRecord(ev[3], h->stream));
  CK(h->opt.pi_dtype == AMMSB_PI_BF16 ? launch_commit<__nv_bfloat16>(h, bp) : launch_commit<float>(h, bp));
  CK(cudaEventRecord(ev[4], h->stream));
  k_theta<<<(h->m.K + 31) / 32, 1024, 0, h->stream>>>(h->m, bp);
  CK(cudaGetLastError());
  CK(cudaEventRecord(ev[5], h->stream));
  CK(cudaEventSynchronize(ev[5]));
  for (int i = 0; i < 5; ++i) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]));
    ms5[i] = ms;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  h->step_count += 1;
  h->last = h->slot;
  return check_device_err(h);
}

// ---------------------------------------------------------------------------
// Autotuner of update_phi: warps-per-node and K-tile.  Every built shape of
// the kernels that covers this handle's row (lanes x vectors per lane within
// 2x of the row's 16-byte vectors; the ring kernel at each ring depth
// for wide rows) is timed with CUDA events on a non-link minibatch of this
// handle's graph, against a scratch copy of phi so the chain's state is not
// touched; the fastest becomes the handle's configuration.  Choices are
// cached per (device, pi type, row width, neighbours, minibatch capacity).
// ---------------------------------------------------------------------------
}  // extern "C"

namespace {

std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int, int>, KernelCfg> g_tune_cache;

std::vector<KernelCfg> phi_candidates(const ammsb_handle* h) {
  const int ev = (h->opt.pi_dtype == AMMSB_PI_BF16) ? 8 : 4;
  const int nvec = h->m.Kp / ev;
  std::vector<KernelCfg> out;
  KernelCfg base = h->cfg;
  base.ring = 0;
#define CAND(L, V, S)                                                      \
  if ((L) * (V) >= nvec && (L) * (V) < 2 * nvec + ((L) == 1 ? 1 : 0)) {  \
    KernelCfg c = base;                                                    \
    c.lpn = L;                                                             \
    c.vpl = V;                                                             \
    c.split = S;                                                           \
    out.push_back(c);                                                      \
  }
  AMMSB_PHI_REG_SHAPES(CAND)
#undef CAND
  if (nvec >= 32) {
    const int vpl = next_pow2((nvec + 31) / 32);
    if (vpl <= 8) {
#define TCAND(S)          \
  {                       \
    KernelCfg c = base;   \
    c.ring = 1;            \
    c.lpn = 32;           \
    c.vpl = vpl;          \
    c.split = 4;          \
    c.ring_stages = S;     \
    out.push_back(c);     \
  }
      AMMSB_PHI_RING_STAGES(TCAND)
#undef TCAND
    }
  }
  return out;
}

int apply_phi_cfg(ammsb_handle* h, const KernelCfg& c) {
  h->cfg = c;
  h->cfg.npb = std::max(1, 128 / (c.lpn * c.split));
  if (c.ring) {
    cudaError_t e = (h->opt.pi_dtype == AMMSB_PI_BF16) ? launch_phi_ring<__nv_bfloat16>(h, h->b, true)
                                                       : launch_phi_ring<float>(h, h->b, true);
    if (e != cudaSuccess) {
      h->err = std::string("update_phi configuration: ") + cudaGetErrorString(e);
      return AMMSB_E_CUDA;
    }
  }
  for (auto* gs : {h->graph1, h->graph2, h->graph1t, h->graph2t, h->graphL})  // the captured iterations used the old kernels
    for (int i = 0; i < kRing; ++i)
      if (gs[i]) {
        cudaGraphExecDestroy(gs[i]);
        gs[i] = nullptr;
      }
  return AMMSB_OK;
}

}  // namespace

extern "C" {

int ammsb_autotune(ammsb_handle* h, int32_t reps, int32_t flags) {
  if (!h || reps < 1) return AMMSB_E_ARG;
  if (!h->state_ready) {
    h->err = "call ammsb_init_state or ammsb_set_state first";
    return AMMSB_E_STATE;
  }
  CK(cudaSetDevice(h->device));
  const auto key = std::make_tuple(h->device, (int)h->opt.pi_dtype, h->m.Kp, h->m.n_out, h->m.max_nodes);
  if (!(flags & AMMSB_TUNE_FRESH)) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) return apply_phi_cfg(h, it->second);
  }
  CK(cudaStreamSynchronize(h->stream));
  // a non-link minibatch and its neighbour sets into buffer set 0
  Model mt = h->m;
  mt.strategy = AMMSB_STRATIFIED_RANDOM_NODE_NONLINKS;
  const Buffers& b0 = h->bufs[0];
  k_sample_minibatch<<<1, 1024, h->mb_smem, h->stream>>>(mt, h->g, b0, h->mb_smem > 0);
  CK(cudaGetLastError());
  k_sample_neighbors<8><<<h->nbr_blocks, 256, h->nbr_smem, h->stream>>>(h->m, h->g, b0);
  CK(cudaGetLastError());
  float* scratch = nullptr;
  const size_t phi_bytes = sizeof(float) * (size_t)h->m.N * h->m.Kp;
  CK(cudaMalloc(&scratch, phi_bytes));
  Buffers bt = b0;
  bt.phi = scratch;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = AMMSB_OK;
  const std::vector<KernelCfg> cands = phi_candidates(h);
  KernelCfg best = h->cfg;
  float best_ms = 1e30f;
  auto run = [&]() -> cudaError_t {
    if (cudaMemcpyAsync(scratch, h->b.phi, phi_bytes, cudaMemcpyDeviceToDevice, h->stream) ||
        cudaEventCreate(&e0) || cudaEventCreate(&e1))
      return cudaGetLastError();
    for (const KernelCfg& c : cands) {
      if (apply_phi_cfg(h, c) != AMMSB_OK) continue;  // shape not launchable here
      auto launch = [&]() {
        return (h->opt.pi_dtype == AMMSB_PI_BF16) ? launch_phi<__nv_bfloat16>(h, bt)
                                                  : launch_phi<float>(h, bt);
      };
      cudaError_t e = launch();  // warm-up
      if (e != cudaSuccess) return e;
      if ((e = cudaEventRecord(e0, h->stream)) != cudaSuccess) return e;
      for (int r = 0; r < reps; ++r)
        if ((e = launch()) != cudaSuccess) return e;
      if ((e = cudaEventRecord(e1, h->stream)) != cudaSuccess) return e;
      if ((e = cudaEventSynchronize(e1)) != cudaSuccess) return e;
      float ms = 0.f;
      if ((e = cudaEventElapsedTime(&ms, e0, e1)) != cudaSuccess) return e;
      if (ms < best_ms) {
        best_ms = ms;
        best = c;
      }
    }
    return cudaSuccess;
  };
  cudaError_t e = run();
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaStreamSynchronize(h->stream);
  cudaFree(scratch);
  if (e != cudaSuccess) {
    h->err = std::string("autotune: ") + cudaGetErrorString(e);
    rc = AMMSB_E_CUDA;
  }
  // the tuning draws are not an iteration: the next draw is step_count's
  const uint32_t s = (uint32_t)h->step_count;
  CK(cudaMemcpyAsync(&h->gc->next_step, &s, sizeof(s), cudaMemcpyHostToDevice, h->stream));
  h->ahead = 0;
  h->slot = 0;
  h->last = -1;
  int rc2 = apply_phi_cfg(h, best);
  CK(cudaStreamSynchronize(h->stream));
  if (rc) return rc;
  if (rc2) return rc2;
  rc = ammsb_detail::check_device_err(h);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune_cache[key] = best;
  return AMMSB_OK;
}

int ammsb_get_kernel_config(ammsb_handle* h, int32_t* out) {
  if (!h || !out) return AMMSB_E_ARG;
  out[0] = h->cfg.ring;
  out[1] = h->cfg.lpn;
  out[2] = h->cfg.vpl;
  out[3] = h->cfg.split;
  out[4] = h->cfg.ring_stages;
  return AMMSB_OK;
}

void* ammsb_stream(ammsb_handle* h) { return h ? (void*)h->stream : nullptr; }

// ---------------------------------------------------------------------------
// Sharded iteration (the distributed sampler's split of one iteration over
// ranks, mcmc_sampler_stochastic_distr.cc): every rank draws the same
// minibatch and neighbour sets (they depend only on seed, chain and step),
// updates the phi rows of the minibatch nodes it owns, all ranks exchange
// the new pi rows, each commits all of them into its own pi and sums the
// beta gradient over the edges it owns, the ranks add those sums, and each
// takes the same theta step.  These four calls are one rank's phases; the
// exchange between them is the caller's (mcmc_for_ammsb_gb300/sharded.py).
// ---------------------------------------------------------------------------
}  // extern "C"

namespace {

__global__ void k_shard_gather_nodes(Buffers from, Buffers to, const int32_t* slots, int n, int n_out) {
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < (int64_t)n * n_out;
       x += (int64_t)gridDim.x * blockDim.x) {
    const int q = (int)(x / n_out), j = (int)(x % n_out);
    const int s = slots[q];
    to.nbr[x] = from.nbr[(int64_t)s * n_out + j];
    if (j == 0) to.nodes[q] = from.nodes[s];
  }
}

__global__ void k_shard_gather_edges(Buffers from, Buffers to, const int32_t* idx, int n, int n_nodes) {
  for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x) {
    to.ea[x] = from.ea[idx[x]];
    to.eb[x] = from.eb[idx[x]];
    to.ey[x] = from.ey[idx[x]];
  }
  for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < n_nodes; x += gridDim.x * blockDim.x)
    to.nodes[x] = from.nodes[x];
}

int shard_buffers(ammsb_handle* h) {
  if (!h->d_shard_idx) {
    const size_t n = (size_t)std::max<int64_t>(h->m.max_nodes, h->m.max_edges);
    int rc = dev_alloc(h, &h->d_shard_idx, n);
    if (!rc) rc = dev_alloc(h, &h->d_shard_R, (size_t)2 * h->m.K);
    if (rc) return rc;
  }
  return AMMSB_OK;
}

DevState read_state(ammsb_handle* h, const Buffers& b, int* rc) {
  DevState st{};
  *rc = AMMSB_OK;
  if (cudaMemcpyAsync(&st, b.st, sizeof(st), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
      cudaStreamSynchronize(h->stream) != cudaSuccess) {
    h->err = "state read failed";
    *rc = AMMSB_E_CUDA;
  }
  return st;
}

}  // namespace

extern "C" {

int ammsb_shard_draw(ammsb_handle* h) {
  if (!h) return AMMSB_E_ARG;
  if (!h->state_ready) {
    h->err = "call ammsb_init_state or ammsb_set_state first";
    return AMMSB_E_STATE;
  }
  CK(cudaSetDevice(h->device));
  int rc = shard_buffers(h);
  if (rc) return rc;
  h->ahead = 0;  // nothing drawn ahead survives: the draw is for step_count
  const uint32_t s = (uint32_t)h->step_count;
  CK(cudaMemcpyAsync(&h->gc->next_step, &s, sizeof(s), cudaMemcpyHostToDevice, h->stream));
  CK(launch_sampling_phase(h, h->bufs[h->slot], h->stream));
  h->shard_drawn = h->slot;
  h->last = h->slot;
  h->shard_phase = 1;
  return check_device_err(h);
}

int ammsb_shard_update(ammsb_handle* h, int32_t n_owned, const int32_t* slots, float* rows_out) {
  if (!h || n_owned < 0 || (n_owned > 0 && (!slots || !rows_out))) return AMMSB_E_ARG;
  if (h->shard_phase != 1) {
    h->err = "ammsb_shard_update follows ammsb_shard_draw";
    return AMMSB_E_STATE;
  }
  CK(cudaSetDevice(h->device));
  const Buffers& D = h->bufs[h->shard_drawn];
  int rc = AMMSB_OK;
  DevState st = read_state(h, D, &rc);
  if (rc) return rc;
  if (n_owned > st.n_nodes) return AMMSB_E_ARG;
  for (int32_t q = 0; q < n_owned; ++q)
    if (slots[q] < 0 || slots[q] >= st.n_nodes || (q > 0 && slots[q] <= slots[q - 1])) {
      h->err = "owned slots must be ascending and inside the drawn minibatch";
      return AMMSB_E_ARG;
    }
  h->shard_phase = 2;
  if (n_owned == 0) return AMMSB_OK;
  // the owned nodes and their neighbour sets, compacted into the next
  // buffer set, then update_phi of those alone
  const Buffers& W = h->bufs[(h->shard_drawn + 1) % kRing];
  CK(cudaMemcpyAsync(h->d_shard_idx, slots, sizeof(int32_t) * n_owned, cudaMemcpyHostToDevice, h->stream));
  const int64_t work = (int64_t)n_owned * h->m.n_out;
  k_shard_gather_nodes<<<(int)std::min<int64_t>((work + 255) / 256, 152 * 8), 256, 0, h->stream>>>(
      D, W, h->d_shard_idx, n_owned, h->m.n_out);
  CK(cudaGetLastError());
  DevState ws = st;
  ws.n_nodes = n_owned;
  ws.n_edges = 0;
  CK(cudaMemcpyAsync(W.st, &ws, sizeof(ws), cudaMemcpyHostToDevice, h->stream));
  CK(h->opt.pi_dtype == AMMSB_PI_BF16 ? launch_phi<__nv_bfloat16>(h, W) : launch_phi<float>(h, W));
  CK(cudaMemcpy2DAsync(rows_out, sizeof(float) * h->m.K, h->b.stage, sizeof(float) * h->m.Kp,
                       sizeof(float) * h->m.K, n_owned, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return check_device_err(h);
}

int ammsb_shard_commit(ammsb_handle* h, const float* rows_all, int32_t n_owned_edges,
                       const int32_t* edge_idx, double* R_out) {
  if (!h || !rows_all || !R_out || n_owned_edges < 0 || (n_owned_edges > 0 && !edge_idx))
    return AMMSB_E_ARG;
  if (h->shard_phase != 2) {
    h->err = "ammsb_shard_commit follows ammsb_shard_update";
    return AMMSB_E_STATE;
  }
  CK(cudaSetDevice(h->device));
  const Buffers& D = h->bufs[h->shard_drawn];
  int rc = AMMSB_OK;
  DevState st = read_state(h, D, &rc);
  if (rc) return rc;
  for (int32_t q = 0; q < n_owned_edges; ++q)
    if (edge_idx[q] < 0 || edge_idx[q] >= st.n_edges || (q > 0 && edge_idx[q] <= edge_idx[q - 1])) {
      h->err = "owned edges must be ascending and inside the drawn minibatch";
      return AMMSB_E_ARG;
    }
  // every node's new pi row into the staging rows (slot order), the owned
  // edges into the next buffer set beside all the nodes, then the commit of
  // every row and the beta partials of the owned edges
  CK(cudaMemcpy2DAsync(h->b.stage, sizeof(float) * h->m.Kp, rows_all, sizeof(float) * h->m.K,
                       sizeof(float) * h->m.K, st.n_nodes, cudaMemcpyHostToDevice, h->stream));
  const Buffers& W = h->bufs[(h->shard_drawn + 1) % kRing];
  if (n_owned_edges > 0)
    CK(cudaMemcpyAsync(h->d_shard_idx, edge_idx, sizeof(int32_t) * n_owned_edges, cudaMemcpyHostToDevice,
                       h->stream));
  const int span = std::max(n_owned_edges, st.n_nodes);
  k_shard_gather_edges<<<std::max(1, std::min((span + 255) / 256, 152 * 8)), 256, 0, h->stream>>>(
      D, W, h->d_shard_idx, n_owned_edges, st.n_nodes);
  CK(cudaGetLastError());
  DevState ws = st;
  ws.n_edges = n_owned_edges;
  CK(cudaMemcpyAsync(W.st, &ws, sizeof(ws), cudaMemcpyHostToDevice, h->stream));
  CK(h->opt.pi_dtype == AMMSB_PI_BF16 ? launch_commit<__nv_bfloat16>(h, W) : launch_commit<float>(h, W));
  k_beta_sums<<<(h->m.K + 31) / 32, 1024, 0, h->stream>>>(h->m, W, h->d_shard_R);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(R_out, h->d_shard_R, sizeof(double) * 2 * h->m.K, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  h->shard_phase = 3;
  return check_device_err(h);
}

int ammsb_shard_theta(ammsb_handle* h, const double* R_total) {
  if (!h || !R_total) return AMMSB_E_ARG;
  if (h->shard_phase != 3) {
    h->err = "ammsb_shard_theta follows ammsb_shard_commit";
    return AMMSB_E_STATE;
  }
  CK(cudaSetDevice(h->device));
  const Buffers& D = h->bufs[h->shard_drawn];
  CK(cudaMemcpyAsync(h->d_shard_R, R_total, sizeof(double) * 2 * h->m.K, cudaMemcpyHostToDevice, h->stream));
  k_theta_given<<<(h->m.K + 31) / 32, 1024, 0, h->stream>>>(h->m, D, h->d_shard_R);
  CK(cudaGetLastError());
  h->last = h->shard_drawn;
  h->slot = (h->shard_drawn + 1) % kRing;
  h->step_count += 1;
  h->shard_phase = 0;
  h->shard_drawn = -1;
  h->ahead = 0;
  const uint32_t s = (uint32_t)h->step_count;
  CK(cudaMemcpyAsync(&h->gc->next_step, &s, sizeof(s), cudaMemcpyHostToDevice, h->stream));
  return check_device_err(h);
}

int ammsb_get_counters(ammsb_handle* h, uint64_t* edge_evals, uint64_t* iterations) {
  if (!h) return AMMSB_E_ARG;
  CK(cudaSetDevice(h->device));
  DevCounters gc;
  CK(cudaMemcpyAsync(&gc, h->gc, sizeof(gc), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (edge_evals) *edge_evals = gc.evals;
  if (iterations) *iterations = gc.iters;
  return AMMSB_OK;
}

// ---------------------------------------------------------------------------
// Checkpoint / resume.  Every draw is a function of (seed, chain, step), so
// the state below is the whole chain: restoring it continues the trajectory
// bit for bit.  Large arrays move through a bounded host staging buffer.
// ---------------------------------------------------------------------------
namespace {

constexpr char kCkMagic[8] = {'A', 'M', 'M', 'S', 'B', 'C', 'K', '1'};

struct CkHeader {
  int32_t pi_dtype, pad;
  int64_t N, K, H;
  uint32_t seed, chain;
  uint64_t step_count, average_count, n_hist, held_sum;
};

uint64_t held_checksum(ammsb_handle* h) {
  // FNV-1a over the held-out pairs (host copy of device arrays)
  std::vector<int32_t> a(h->H), b(h->H);
  std::vector<uint8_t> y(h->H);
  if (h->H > 0) {
    cudaMemcpy(a.data(), h->d_ha, sizeof(int32_t) * h->H, cudaMemcpyDeviceToHost);
    cudaMemcpy(b.data(), h->d_hb, sizeof(int32_t) * h->H, cudaMemcpyDeviceToHost);
    cudaMemcpy(y.data(), h->d_hy, h->H, cudaMemcpyDeviceToHost);
  }
  uint64_t x = 1469598103934665603ull;
  auto mix = [&](const void* p, size_t n) {
    const unsigned char* c = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) x = (x ^ c[i]) * 1099511628211ull;
  };
  mix(a.data(), a.size() * 4);
  mix(b.data(), b.size() * 4);
  mix(y.data(), y.size());
  return x;
}

// rows [0, N) of a device array with row stride Kp elements of es bytes,
// K elements per row in the file
int ck_rows(ammsb_handle* h, std::FILE* f, void* dev, size_t es, bool save) {
  const int64_t N = h->m.N, K = h->m.K, Kp = h->m.Kp;
  const int64_t rows_per = std::max<int64_t>(1, (64ll << 20) / (int64_t)(K * es));
  std::vector<unsigned char> buf((size_t)std::min<int64_t>(rows_per, N) * (size_t)(K * es));
  for (int64_t r0 = 0; r0 < N; r0 += rows_per) {
    const int64_t n = std::min<int64_t>(rows_per, N - r0);
    char* d = static_cast<char*>(dev) + (size_t)r0 * (size_t)Kp * es;
    const size_t bytes = (size_t)n * (size_t)K * es;
    if (save) {
      CK(cudaMemcpy2DAsync(buf.data(), K * es, d, Kp * es, K * es, n, cudaMemcpyDeviceToHost,
                           h->stream));
      CK(cudaStreamSynchronize(h->stream));
      if (std::fwrite(buf.data(), 1, bytes, f) != bytes) {
        h->err = "checkpoint: write failed";
        return AMMSB_E_ARG;
      }
    } else {
      if (std::fread(buf.data(), 1, bytes, f) != bytes) {
        h->err = "checkpoint: file is truncated";
        return AMMSB_E_ARG;
      }
      CK(cudaMemcpy2DAsync(d, Kp * es, buf.data(), K * es, K * es, n, cudaMemcpyHostToDevice,
                           h->stream));
      CK(cudaStreamSynchronize(h->stream));
    }
  }
  return AMMSB_OK;
}

}  // namespace

int ammsb_save_checkpoint(ammsb_handle* h, const char* path) {
  if (!h || !path) return AMMSB_E_ARG;
  if (!h->state_ready) {
    h->err = "no state to save: call ammsb_init_state or ammsb_set_state first";
    return AMMSB_E_STATE;
  }
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  std::FILE* f = std::fopen(path, "wb");
  if (!f) {
    h->err = std::string("checkpoint: cannot open ") + path;
    return AMMSB_E_ARG;
  }
  CkHeader hd{};
  hd.pi_dtype = h->opt.pi_dtype;
  hd.N = h->m.N;
  hd.K = h->m.K;
  hd.H = h->H;
  hd.seed = h->m.seed;
  hd.chain = h->m.chain;
  hd.step_count = h->step_count;
  hd.average_count = h->average_count;
  hd.n_hist = h->ppx_history.size();
  hd.held_sum = held_checksum(h);
  const int K = h->m.K;
  std::vector<double> theta(2 * (size_t)K);
  std::vector<float> beta(K), ppx(std::max<int64_t>(h->H, 1));
  int rc = AMMSB_OK;
  auto fail = [&](int code) {
    std::fclose(f);
    return code;
  };
  if (cudaMemcpy(theta.data(), h->b.theta, sizeof(double) * 2 * K, cudaMemcpyDeviceToHost) ||
      cudaMemcpy(beta.data(), h->b.beta, sizeof(float) * K, cudaMemcpyDeviceToHost) ||
      (h->H > 0 && cudaMemcpy(ppx.data(), h->d_ppx, sizeof(float) * h->H, cudaMemcpyDeviceToHost))) {
    h->err = "checkpoint: device read failed";
    return fail(AMMSB_E_CUDA);
  }
  bool ok = std::fwrite(kCkMagic, 1, 8, f) == 8 && std::fwrite(&hd, sizeof(hd), 1, f) == 1 &&
            std::fwrite(h->ppx_history.data(), sizeof(double), hd.n_hist, f) == hd.n_hist &&
            std::fwrite(theta.data(), sizeof(double), theta.size(), f) == theta.size() &&
            std::fwrite(beta.data(), sizeof(float), beta.size(), f) == beta.size() &&
            std::fwrite(ppx.data(), sizeof(float), (size_t)h->H, f) == (size_t)h->H;
  if (!ok) {
    h->err = "checkpoint: write failed";
    return fail(AMMSB_E_ARG);
  }
  if ((rc = ck_rows(h, f, h->b.phi, sizeof(float), true))) return fail(rc);
  if ((rc = ck_rows(h, f, h->b.pi, (size_t)h->pi_bytes, true))) return fail(rc);
  if (std::fclose(f) != 0) {
    h->err = "checkpoint: close failed";
    return AMMSB_E_ARG;
  }
  return AMMSB_OK;
}

int ammsb_load_checkpoint(ammsb_handle* h, const char* path) {
  if (!h || !path) return AMMSB_E_ARG;
  CK(cudaSetDevice(h->device));
  std::FILE* f = std::fopen(path, "rb");
  if (!f) {
    h->err = std::string("checkpoint: cannot open ") + path;
    return AMMSB_E_ARG;
  }
  auto fail = [&](const char* msg, int code) {
    if (msg) h->err = msg;
    std::fclose(f);
    return code;
  };
  char magic[8];
  CkHeader hd{};
  if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, kCkMagic, 8) != 0 ||
      std::fread(&hd, sizeof(hd), 1, f) != 1)
    return fail("checkpoint: not a sampler checkpoint", AMMSB_E_ARG);
  if (hd.pi_dtype != h->opt.pi_dtype || hd.N != h->m.N || hd.K != h->m.K || hd.H != h->H)
    return fail("checkpoint: pi type, N, K or held-out size differ from this sampler", AMMSB_E_ARG);
  if (hd.seed != h->m.seed || hd.chain != h->m.chain)
    return fail("checkpoint: seed or chain differ from this sampler", AMMSB_E_ARG);
  if (hd.held_sum != held_checksum(h))
    return fail("checkpoint: held-out set differs from this sampler", AMMSB_E_ARG);
  if (hd.step_count < 1 || hd.step_count > 0xffffffffull || hd.average_count < 1 ||
      hd.n_hist > (1ull << 32))
    return fail("checkpoint: corrupt counters", AMMSB_E_ARG);
  const int K = h->m.K;
  std::vector<double> hist(hd.n_hist), theta(2 * (size_t)K);
  std::vector<float> beta(h->m.Kp, 0.f), ppx(std::max<int64_t>(h->H, 1));
  if (std::fread(hist.data(), sizeof(double), hd.n_hist, f) != hd.n_hist ||
      std::fread(theta.data(), sizeof(double), theta.size(), f) != theta.size() ||
      std::fread(beta.data(), sizeof(float), K, f) != (size_t)K ||
      std::fread(ppx.data(), sizeof(float), (size_t)h->H, f) != (size_t)h->H)
    return fail("checkpoint: file is truncated", AMMSB_E_ARG);
  if (cudaMemcpyAsync(h->b.theta, theta.data(), sizeof(double) * 2 * K, cudaMemcpyHostToDevice,
                      h->stream) ||
      cudaMemcpyAsync(h->b.beta, beta.data(), sizeof(float) * h->m.Kp, cudaMemcpyHostToDevice,
                      h->stream) ||
      (h->H > 0 && cudaMemcpyAsync(h->d_ppx, ppx.data(), sizeof(float) * h->H,
                                   cudaMemcpyHostToDevice, h->stream)) ||
      cudaStreamSynchronize(h->stream))
    return fail("checkpoint: device write failed", AMMSB_E_CUDA);
  int rc = ck_rows(h, f, h->b.phi, sizeof(float), false);
  if (!rc) rc = ck_rows(h, f, h->b.pi, (size_t)h->pi_bytes, false);
  if (rc) return fail(nullptr, rc);
  std::fclose(f);
  rc = reset_counters(h);  // zeroes the running averages: restore them after
  if (rc) return rc;
  if (h->H > 0)
    CK(cudaMemcpyAsync(h->d_ppx, ppx.data(), sizeof(float) * h->H, cudaMemcpyHostToDevice,
                       h->stream));
  h->step_count = hd.step_count;
  h->average_count = hd.average_count;
  h->ppx_history = hist;
  const uint32_t s = (uint32_t)hd.step_count;
  CK(cudaMemcpyAsync(&h->gc->next_step, &s, sizeof(s), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  h->state_ready = true;
  return AMMSB_OK;
}

}  // extern "C"
