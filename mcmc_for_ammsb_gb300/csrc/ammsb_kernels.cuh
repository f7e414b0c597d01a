// ammsb_kernels.cuh -- sm_103a kernels of one SG-MCMC iteration.
//
// Phase order of MCMCSamplerStochastic::run (mcmc_sampler_stochastic.cc
// :131-174), one kernel each, all reading the per-iteration scalars from
// DevState so the sequence replays as a CUDA graph:
//   k_sample_minibatch   Network::sample_mini_batch + nodes_in_batch
//   k_sample_neighbors   sample_neighbor_nodes (h:87-108) + y lookups
//   k_update_phi         update_phi (cc:269-313), fused with the noise draw
//                        and the normalisation pi_i = phi_i / sum(phi_i)
//                        into a staging buffer (Jacobi: pi is not touched)
//   k_commit_beta        pi[nodes] = staged rows (cc:162-166) and the
//                        per-edge update_beta gradient (cc:212-240) as a
//                        segmented block reduction
//   k_theta              sum of block partials + SGRLD theta step + beta
//                        (cc:244-266), FP64
#pragma once
#include "ammsb_device.cuh"

namespace ammsb {

// Upper bound of Model::nbb, the blocks of k_commit_beta that write beta
// gradient partials (k_theta reads them back, up to 9 per warp).
#ifndef AMMSB_MAX_BETA_BLOCKS
#define AMMSB_MAX_BETA_BLOCKS 256
#endif
constexpr int kMaxBetaBlocks = AMMSB_MAX_BETA_BLOCKS;
// k_theta's 31 summing warps read up to 9 partials each in one pass
constexpr int kThetaSumWarps = 31, kThetaPerPass = 9;
static_assert(kMaxBetaBlocks <= kThetaSumWarps * kThetaPerPass, "k_theta reads the partials in one pass");

struct Model {
  int32_t K;      // communities
  int32_t Kp;     // row stride in elements (K rounded up to 16 bytes)
  int64_t N;
  float alpha, epsilon;
  float Nn;       // N / num_node_sample, as the reference (cc:300)
  float eta0, eta1;
  double a, b, c; // step-size schedule
  uint32_t seed, chain;
  int32_t n_out;  // num_node_sample + 1 neighbours per node
  int32_t max_nodes, max_edges;
  int32_t mini_batch_size;
  int32_t strategy;
  float nonlink_scale, link_scale;
  int32_t nbb;    // beta partial blocks (at most kMaxBetaBlocks)
  int32_t nbr_set_cap;  // per-warp accepted-neighbour set capacity (power of two)
  int32_t max_source;   // sampler.max-source (link stratum)
  int32_t full_set;     // random-edge: the minibatch is the whole training set
  int64_t n_entries;    // 2E: entries of the symmetric CSR
};

struct Buffers {
  void* pi;            // N x Kp, PiT
  float* phi;          // N x Kp
  float* stage;        // max_nodes x Kp: new pi rows of the minibatch nodes
  float* beta;         // K
  double* theta;       // K x 2
  int32_t* nodes;      // max_nodes
  int32_t* ea;         // max_edges: slot of first endpoint
  int32_t* eb;         // slot of second endpoint
  uint8_t* ey;         // y of each minibatch edge
  uint32_t* nbr;       // max_nodes x n_out: id | y << 31
  int32_t* cand;       // mini_batch_size: candidate scratch
  uint32_t* htab_key;  // minibatch dedup hash
  uint32_t* htab_idx;
  uint32_t hmask;
  float* beta_part;    // nbb x 2 x Kp
  const float* fed_phi_noise;    // max_nodes x K or null
  const float* fed_theta_noise;  // K x 2 or null
  DevState* st;        // this buffer set's per-iteration scalars
  DevCounters* gc;     // sampler-wide counters
};

// One chain of a multi-chain launch (blockIdx.y selects the chain): its
// model, graph and both buffer sets, plus the per-chain launch parameters
// of the single-chain kernels.
struct ChainArgs {
  Model m;
  DevGraph g;
  Buffers b[2];
  int32_t ncommit;    // k_commit_beta: blocks of the commit part
  int32_t smem_hash;  // k_sample_minibatch: the dedup hash fits shared memory
};

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Mask of the aligned group of G lanes (G a power of two <= 32) holding
// `lane`.
template <int G>
__device__ __forceinline__ uint32_t group_mask(int lane) {
  if constexpr (G >= 32) {
    return 0xffffffffu;
  } else {
    return ((1u << G) - 1u) << ((lane / G) * G);
  }
}

// Exclusive prefix sum of per-thread counts over a 1024-thread block, in
// thread order; returns the position and sets *total.  Uses s_warp[33].
__device__ __forceinline__ int block_scan_count_1024(int v, int* s_warp, int* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int n = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += n;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const int w = s_warp[lane];
    int winc = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int n = __shfl_up_sync(0xffffffffu, winc, o);
      if (lane >= o) winc += n;
    }
    s_warp[lane] = winc - w;
    if (lane == 31) s_warp[32] = winc;
  }
  __syncthreads();
  const int pos = s_warp[warp] + incl - v;
  *total = s_warp[32];
  __syncthreads();
  return pos;
}

// Exclusive prefix count of `flag` over a 1024-thread block, in thread
// order; returns the position and sets *total.  Uses s_warp[32].
__device__ __forceinline__ int block_scan_1024(bool flag, int* s_warp, int* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t bal = __ballot_sync(0xffffffffu, flag);
  const int in_warp = __popc(bal & lanemask_lt());
  if (lane == 0) s_warp[warp] = __popc(bal);
  __syncthreads();
  if (warp == 0) {
    int v = s_warp[lane];
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int n = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += n;
    }
    s_warp[lane] = incl - v;  // exclusive
    if (lane == 31) s_warp[32] = incl;
  }
  __syncthreads();
  const int pos = s_warp[warp] + in_warp;
  *total = s_warp[32];
  __syncthreads();
  return pos;
}

// Open-addressing insert of key into (hkey, hidx): keeps the smallest
// position per key.  The table is never full (callers keep it at most half
// full), so the probe ends.
__device__ __forceinline__ void hash_insert_min(uint32_t* hkey, uint32_t* hidx, uint32_t hmask,
                                                uint32_t key, uint32_t pos) {
  uint32_t slot = hash32(key) & hmask;
  for (uint32_t probe = 0; probe <= hmask; ++probe) {
    const uint32_t prev = atomicCAS(hkey + slot, 0xffffffffu, key);
    if (prev == 0xffffffffu || prev == key) {
      atomicMin(hidx + slot, pos);
      return;
    }
    slot = (slot + 1) & hmask;
  }
}

// Value stored for key (0xffffffff when absent).
__device__ __forceinline__ uint32_t hash_find(const uint32_t* hkey, const uint32_t* hidx,
                                              uint32_t hmask, uint32_t key) {
  uint32_t slot = hash32(key) & hmask;
  for (uint32_t probe = 0; probe <= hmask; ++probe) {
    const uint32_t k = hkey[slot];
    if (k == key) return hidx[slot];
    if (k == 0xffffffffu) return 0xffffffffu;
    slot = (slot + 1) & hmask;
  }
  return 0xffffffffu;
}

// Row of entry q of the CSR: the last v with row_ptr[v] <= q.
__device__ __forceinline__ int32_t csr_row_of(const int64_t* row_ptr, int64_t n, int64_t q) {
  int64_t lo = 0, hi = n;
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (__ldg(row_ptr + mid) <= q) lo = mid; else hi = mid;
  }
  return (int32_t)lo;
}

// Node numbering of a general edge list: ea/eb hold the vertex ids of
// `count` edges; the nodes are numbered by first appearance over (a0, b0,
// a1, b1, ...), written to nodes[], and ea/eb are rewritten as slots.
// Returns the node count (or -1 past max_nodes).  Block-wide; uses the
// dedup hash (reset here) and s_warp.
static __device__ int assign_node_slots(const Buffers& b, int count, int max_nodes, uint32_t* hkey,
                                 uint32_t* hidx, int* s_warp) {
  const int tid = threadIdx.x;
  for (uint32_t s = tid; s <= b.hmask; s += blockDim.x) {
    hkey[s] = 0xffffffffu;
    hidx[s] = 0xffffffffu;
  }
  __syncthreads();
  const int np = 2 * count;
  for (int p = tid; p < np; p += blockDim.x) {
    const uint32_t x = (uint32_t)((p & 1) ? b.eb[p >> 1] : b.ea[p >> 1]);
    hash_insert_min(hkey, hidx, b.hmask, x, (uint32_t)p);
  }
  __syncthreads();
  int n = 0;
  for (int base = 0; base < np; base += blockDim.x) {
    const int p = base + tid;
    bool first = false;
    uint32_t x = 0;
    if (p < np) {
      x = (uint32_t)((p & 1) ? b.eb[p >> 1] : b.ea[p >> 1]);
      first = hash_find(hkey, hidx, b.hmask, x) == (uint32_t)p;
    }
    int total;
    const int pos = block_scan_1024(first, s_warp, &total);
    if (first && n + pos < max_nodes) b.nodes[n + pos] = (int32_t)x;
    n += total;
  }
  if (n > max_nodes) return -1;
  __syncthreads();
  // the hash now maps vertex -> slot
  for (int s = tid; s < n; s += blockDim.x) {
    const uint32_t x = (uint32_t)b.nodes[s];
    uint32_t slot = hash32(x) & b.hmask;
    for (uint32_t probe = 0; probe <= b.hmask; ++probe) {
      if (hkey[slot] == x) {
        hidx[slot] = (uint32_t)s;
        break;
      }
      slot = (slot + 1) & b.hmask;
    }
  }
  __syncthreads();
  for (int e = tid; e < count; e += blockDim.x) {
    b.ea[e] = (int32_t)hash_find(hkey, hidx, b.hmask, (uint32_t)b.ea[e]);
    b.eb[e] = (int32_t)hash_find(hkey, hidx, b.hmask, (uint32_t)b.eb[e]);
  }
  __syncthreads();
  return n;
}

// ---------------------------------------------------------------------------
// k_sample_minibatch: one 1024-thread CTA.  Stratified random node
// (network.cc:410-421): flag = randint(0,1); non-link stratum
// (network.cc:274-349): source v and the first m valid new partners u in
// candidate order (u != v, (v,u) not an edge, not held-out, not test); link
// stratum (network.cc:355-407, max-source 1): all training edges of a random
// v, redrawn while empty.  Candidates are examined in rounds of
// need = m - count; within a round the first occurrence of each u wins
// (atomicMin of its index in a hash), then an ordered block scan appends
// them -- exactly the sequential scan of the oracle.
// ---------------------------------------------------------------------------
static __device__ __forceinline__ void sample_minibatch_body(const Model& m, const DevGraph& g,
                                                             const Buffers& b, int smem_hash) {
  extern __shared__ uint32_t s_htab[];  // dedup hash in shared memory when it fits
  constexpr int kRowCap = 2048;         // the source's row, staged when it fits
  __shared__ int32_t s_row[kRowCap];
  __shared__ int s_warp[33];
  __shared__ int s_flag, s_count, s_nodes;
  __shared__ uint32_t s_step;
  __shared__ int32_t s_v;
  __shared__ int s_brk, s_dup;
  const int tid = threadIdx.x;
  const Stream rs{m.seed, m.chain};
  if (tid == 0) {
    const uint32_t step = b.gc->next_step;
    b.st->step = step;
    b.gc->next_step = step + 1;
    int flag;
    if (m.strategy == 0)
      flag = (int)uniform_below(rs.draw_u64(kTagMbFlag, 0, step, 0), 2ull);
    else if (m.strategy == 3)
      flag = 2;  // random-edge
    else
      flag = (m.strategy == 1) ? 1 : 0;
    s_flag = flag;
    s_step = step;
    s_count = 0;
    s_nodes = 0;
  }
  __syncthreads();
  const uint32_t step = s_step;
  const int flag = s_flag;
  int err = 0;
  int rounds = 0;
  if (flag == 0) {
    const int mb = m.mini_batch_size;
    const int32_t v = (int32_t)uniform_below(rs.draw_u64(kTagMbNode, 0, step, 0), (uint64_t)g.n);
    uint32_t* hkey = smem_hash ? s_htab : b.htab_key;
    uint32_t* hidx = smem_hash ? s_htab + (b.hmask + 1) : b.htab_idx;
    for (uint32_t s = tid; s <= b.hmask; s += blockDim.x) {
      hkey[s] = 0xffffffffu;
      hidx[s] = 0xffffffffu;
    }
    if (mb > m.max_edges || mb + 1 > m.max_nodes) err |= kErrCapacity;
    if (tid == 0) b.nodes[0] = v;
    const int64_t vr0 = g.row_ptr[v];
    const int32_t vdeg = (int32_t)(g.row_ptr[v + 1] - vr0);
    const bool row_in_smem = vdeg <= kRowCap;
    if (row_in_smem)
      for (int q = tid; q < vdeg; q += blockDim.x) s_row[q] = g.col[vr0 + q];
    __syncthreads();
    int count = 0;
    uint64_t t = 0;
    // the spec scans candidates t = 0, 1, ... until mb are kept, giving up
    // at `cap`; a round examines R >= need of them in parallel and keeps the
    // first new valid ones, in order, up to mb.  R is what the rounds so far
    // say `need` new ones take (need at first), plus an eighth and 64, while
    // the dedup hash stays at most half full: a round's cost grows with R
    // (a first round of up to 4,096 whatever the need took the 100k-node
    // workload's non-link minibatch from 16 to 44 us), and small populations
    // with many repeats still finish in two or three rounds.
    const uint64_t cap = 64ull * (uint64_t)mb + 4096ull;
    const int half = (int)((b.hmask + 1u) / 2u);
    int64_t seen = 0, kept = 0;  // candidates examined and kept so far
    while (!err && count < mb) {
      const int need = mb - count;
      if (t >= cap) {
        err |= kErrMinibatchCap;
        break;
      }
      const int64_t est = seen == 0 ? need : (kept > 0 ? (need * seen + kept - 1) / kept : half);
      const int want = (int)min(est + est / 8 + 64, (int64_t)half);
      const int R = (int)min((uint64_t)max(need, min(half - count, want)), cap - t);
      const int count0 = count;
      // pass A: validity and first-occurrence index per value, over chunks
      // of up to G * 1,024 candidates.  Thread tid examines candidates
      // c0 + tid + 1024 j of its chunk (one each while the chunk has at most
      // 1,024); the first exclusion probes of its candidates are issued
      // together.
      constexpr int G = 4;
      const int chunk = G * (int)blockDim.x;
      for (int c0 = 0; c0 < R; c0 += chunk) {
        int32_t u[G];
        bool live[G];
        unsigned long long key[G], xs[G], xk[G];
#pragma unroll
        for (int j = 0; j < G; ++j) {
          const int c = c0 + tid + (int)blockDim.x * j;
          live[j] = c < R;
          u[j] = live[j] ? (int32_t)uniform_below(rs.draw_u64(kTagMbCand, 0, step, t + (uint64_t)c),
                                                  (uint64_t)g.n)
                         : -1;
          live[j] = live[j] && (u[j] != v);
          key[j] = pair_key(v, u[j] < 0 ? 0 : u[j]);
          xs[j] = hash64(key[j]) & g.excl_mask;
        }
#pragma unroll
        for (int j = 0; j < G; ++j) xk[j] = live[j] ? __ldg(g.excl + xs[j]) : kEmptyKey;
#pragma unroll
        for (int j = 0; j < G; ++j) {
          const int c = c0 + tid + (int)blockDim.x * j;
          if (c >= R) continue;
          const bool linked = live[j] && (row_in_smem ? row_contains(s_row, vdeg, u[j])
                                                      : has_edge(g, v, u[j]));
          const bool ok = live[j] && !linked &&
                          !probe_resolve(g.excl, g.excl_mask, key[j], xs[j], xk[j]);
          b.cand[c] = ok ? u[j] : -1;
          if (ok) {
            uint32_t slot = hash32((uint32_t)u[j]) & b.hmask;
            for (uint32_t probe = 0; probe <= b.hmask; ++probe) {
              const uint32_t prev = atomicCAS(hkey + slot, 0xffffffffu, (uint32_t)u[j]);
              if (prev == 0xffffffffu || prev == (uint32_t)u[j]) {
                atomicMin(hidx + slot, (uint32_t)(t + (uint64_t)c));
                break;
              }
              slot = (slot + 1) & b.hmask;
            }
          }
        }
      }
      __syncthreads();
      // pass B: ordered compaction of first occurrences, one block scan per
      // chunk (thread-local counts of its g consecutive candidates, g the
      // fewest per thread that cover the chunk); count is block-uniform, so
      // every thread leaves the loop together at mb
      for (int c0 = 0; c0 < R && count < mb; c0 += chunk) {
        const int n = min(R - c0, chunk);
        const int gper = (n + (int)blockDim.x - 1) / (int)blockDim.x;
        int32_t u[G];
        bool acc[G];
        int mine = 0;
#pragma unroll
        for (int j = 0; j < G; ++j) {
          const int c = c0 + gper * tid + j;
          u[j] = -1;
          acc[j] = false;
          if (j < gper && c < c0 + n) {
            u[j] = b.cand[c];
            if (u[j] >= 0) {
              uint32_t slot = hash32((uint32_t)u[j]) & b.hmask;
              for (uint32_t probe = 0; probe <= b.hmask; ++probe) {
                const uint32_t kk = hkey[slot];
                if (kk == (uint32_t)u[j]) {
                  acc[j] = (hidx[slot] == (uint32_t)(t + (uint64_t)c));
                  break;
                }
                if (kk == 0xffffffffu) break;
                slot = (slot + 1) & b.hmask;
              }
            }
          }
          mine += acc[j] ? 1 : 0;
        }
        int total;
        int pos = block_scan_count_1024(mine, s_warp, &total);
#pragma unroll
        for (int j = 0; j < G; ++j) {
          if (acc[j]) {
            const int e = count + pos;
            if (e < mb) {
              b.nodes[e + 1] = u[j];
              b.ea[e] = 0;
              b.eb[e] = e + 1;
              b.ey[e] = 0;
            }
            ++pos;
          }
        }
        count = min(count + total, mb);
      }
      t += (uint64_t)R;
      seen += R;
      kept += count - count0;
      ++rounds;
      __syncthreads();
    }
    if (tid == 0) {
      b.st->scale = m.nonlink_scale;
      s_count = count;
      s_nodes = count + 1;
    }
  } else if (flag == 2) {
    // random_edge_sampling (network.cc:237-268): m distinct training edges,
    // candidates = entries of the symmetric CSR (each edge twice, as the
    // reference's linked_edges), kept when a < b and not held-out/test; the
    // whole training set when m reaches it (network.cc:215-234)
    const int mb = m.mini_batch_size;
    uint32_t* hkey = smem_hash ? s_htab : b.htab_key;
    uint32_t* hidx = smem_hash ? s_htab + (b.hmask + 1) : b.htab_idx;
    int count = 0;
    if (m.full_set) {
      for (int64_t base = 0; base < m.n_entries && !err; base += blockDim.x) {
        const int64_t q = base + tid;
        bool acc = false;
        int32_t a = 0, c = 0;
        if (q < m.n_entries) {
          a = csr_row_of(g.row_ptr, g.n, q);
          c = g.col[q];
          acc = a < c && !is_excluded(g, a, c);
        }
        int total;
        const int pos = block_scan_1024(acc, s_warp, &total);
        if (acc && count + pos < m.max_edges) {
          b.ea[count + pos] = a;
          b.eb[count + pos] = c;
          b.ey[count + pos] = 1;
        }
        count += total;
        if (count > m.max_edges) err |= kErrCapacity;
      }
    } else {
      for (uint32_t sl = tid; sl <= b.hmask; sl += blockDim.x) {
        hkey[sl] = 0xffffffffu;
        hidx[sl] = 0xffffffffu;
      }
      if (mb > m.max_edges) err |= kErrCapacity;
      __syncthreads();
      uint64_t t = 0;
      const uint64_t cap = 64ull * (uint64_t)mb + 4096ull;
      const int half = (int)((b.hmask + 1u) / 2u);
      while (!err && count < mb) {
        const int need = mb - count;
        if (t >= cap) {
          err |= kErrMinibatchCap;
          break;
        }
        const int R = (int)min((uint64_t)max(need, min(half - count, 4096)), cap - t);
        for (int c = tid; c < R; c += blockDim.x) {
          const int64_t q = (int64_t)uniform_below(rs.draw_u64(kTagMbCand, 0, step, t + (uint64_t)c),
                                                   (uint64_t)m.n_entries);
          const int32_t a = csr_row_of(g.row_ptr, g.n, q), bb = g.col[q];
          const bool ok = a < bb && !is_excluded(g, a, bb);
          b.cand[c] = ok ? (int32_t)q : -1;
          if (ok) hash_insert_min(hkey, hidx, b.hmask, (uint32_t)q, (uint32_t)(t + (uint64_t)c));
        }
        __syncthreads();
        for (int base = 0; base < R && count < mb; base += blockDim.x) {
          const int c = base + tid;
          int32_t q = -1;
          bool acc = false;
          if (c < R) {
            q = b.cand[c];
            acc = q >= 0 && hash_find(hkey, hidx, b.hmask, (uint32_t)q) == (uint32_t)(t + (uint64_t)c);
          }
          int total;
          const int pos = block_scan_1024(acc, s_warp, &total);
          if (acc && count + pos < mb) {
            b.ea[count + pos] = csr_row_of(g.row_ptr, g.n, q);
            b.eb[count + pos] = g.col[q];
            b.ey[count + pos] = 1;
          }
          count = min(count + total, mb);
        }
        t += (uint64_t)R;
        ++rounds;
        __syncthreads();
      }
    }
    int n = 0;
    if (!err) {
      n = assign_node_slots(b, count, m.max_nodes, hkey, hidx, s_warp);
      if (n < 0) err |= kErrCapacity;
    }
    if (tid == 0) {
      b.st->scale = count > 0 ? (float)((double)(m.N - 1) * (double)m.N / 2.0 / (double)count) : 0.f;
      s_count = count;
      s_nodes = n;
    }
  } else if (m.max_source > 1) {
    // stratified_random_node_sampling_links with sampler.max-source > 1
    // (network.cc:355-407): up to S sources per attempt (draw a*S + s); from
    // the second on, one whose degree would pass m ends the attempt; each
    // source adds its training edges once (an edge to an earlier source was
    // added from it; a repeated source adds none); redrawn while empty
    const int mb = m.mini_batch_size, S = m.max_source;
    uint32_t* hkey = smem_hash ? s_htab : b.htab_key;
    uint32_t* hidx = smem_hash ? s_htab + (b.hmask + 1) : b.htab_idx;
    int32_t* s_src = s_row;  // the attempt's sources (S <= kRowCap)
    int count = 0;
    for (int attempt = 0; attempt < 4096 && count == 0 && !err; ++attempt) {
      count = 0;
      for (int sidx = 0; sidx < S && !err; ++sidx) {
        if (tid == 0) {
          const int32_t v = (int32_t)uniform_below(
              rs.draw_u64(kTagMbNode, 0, step, (uint64_t)attempt * (uint64_t)S + (uint64_t)sidx),
              (uint64_t)g.n);
          const int64_t deg = g.row_ptr[v + 1] - g.row_ptr[v];
          int dup = 0;
          for (int r = 0; r < sidx; ++r) dup |= (s_src[r] == v);
          s_brk = (sidx > 0 && (int64_t)count + deg > (int64_t)mb) ? 1 : 0;
          s_dup = dup;
          s_v = v;
          if (!s_brk) s_src[sidx] = v;
        }
        __syncthreads();
        const int32_t v = s_v;
        const int brk = s_brk, dup = s_dup;
        __syncthreads();
        if (brk) break;
        if (dup) continue;
        const int64_t r0 = g.row_ptr[v];
        const int deg = (int)(g.row_ptr[v + 1] - r0);
        for (int base = 0; base < deg; base += blockDim.x) {
          const int q = base + tid;
          int32_t u = -1;
          bool acc = false;
          if (q < deg) {
            u = g.col[r0 + q];
            acc = !is_excluded(g, v, u);
            for (int r = 0; r < sidx && acc; ++r) acc = (s_src[r] != u);
          }
          int total;
          const int pos = block_scan_1024(acc, s_warp, &total);
          if (acc && count + pos < m.max_edges) {
            b.ea[count + pos] = v;
            b.eb[count + pos] = u;
            b.ey[count + pos] = 1;
          }
          count += total;
          if (count > m.max_edges) err |= kErrCapacity;
        }
      }
      rounds = attempt + 1;
    }
    if (count == 0 && !err) err |= kErrMinibatchCap;
    int n = 0;
    if (!err) {
      n = assign_node_slots(b, count, m.max_nodes, hkey, hidx, s_warp);
      if (n < 0) err |= kErrCapacity;
    }
    if (tid == 0) {
      b.st->scale = count > 0 ? (float)(m.n_entries / 2) / (float)count : 0.f;
      s_count = count;
      s_nodes = n;
    }
  } else {
    int count = 0;
    for (int attempt = 0; attempt < 4096 && count == 0 && !err; ++attempt) {
      const int32_t v =
          (int32_t)uniform_below(rs.draw_u64(kTagMbNode, 0, step, (uint64_t)attempt), (uint64_t)g.n);
      const int64_t r0 = g.row_ptr[v], deg = g.row_ptr[v + 1] - r0;
      if (deg > m.max_edges || deg + 1 > m.max_nodes) {
        err |= kErrCapacity;
        break;
      }
      for (int64_t base = 0; base < deg; base += blockDim.x) {
        const int64_t q = base + tid;
        int32_t u = -1;
        bool acc = false;
        if (q < deg) {
          u = g.col[r0 + q];
          acc = !is_excluded(g, v, u);
        }
        int total;
        const int pos = block_scan_1024(acc, s_warp, &total);
        if (acc) {
          const int e = count + pos;
          b.nodes[e + 1] = u;
          b.ea[e] = 0;
          b.eb[e] = e + 1;
          b.ey[e] = 1;
        }
        count += total;
      }
      if (count > 0 && tid == 0) b.nodes[0] = v;
      rounds = attempt + 1;
    }
    if (count == 0 && !err) err |= kErrMinibatchCap;
    if (tid == 0) {
      b.st->scale = m.link_scale;
      s_count = count;
      s_nodes = count + 1;
    }
  }
  __syncthreads();
  if (tid == 0) {
    b.st->flag = flag;
    b.st->n_edges = err ? 0 : s_count;
    b.st->n_nodes = err ? 0 : s_nodes;
    b.st->rounds = rounds;
    if (err) atomicOr(&b.gc->err, err);
  }
}
static __global__ void __launch_bounds__(1024) k_sample_minibatch(Model m, DevGraph g, Buffers b,
                                                                  int smem_hash) {
  sample_minibatch_body(m, g, b, smem_hash);
}
// one CTA per chain (blockIdx.y), buffer set p
static __global__ void __launch_bounds__(1024) k_sample_minibatch_chains(const ChainArgs* __restrict__ c,
                                                                         int p) {
  const ChainArgs& a = c[blockIdx.y];
  sample_minibatch_body(a.m, a.g, a.b[p], a.smem_hash);
}

// ---------------------------------------------------------------------------
// k_sample_neighbors: one warp per minibatch node.  n_out distinct ids j,
// j != i, (i,j) neither held-out nor test (h:87-108); 32 candidates per
// round, the first valid new ones in candidate order are kept; y_ij is the
// graph membership the update needs (cc:279-283).
// ---------------------------------------------------------------------------
template <int WARPS>
__device__ __forceinline__ void sample_neighbors_body(const Model& m, const DevGraph& g, const Buffers& b) {
  // per warp: a set of the ids accepted so far (open addressing, capacity a
  // power of two >= 2 n_out, -1 empty) in dynamic shared memory
  extern __shared__ int32_t s_sets[];
  constexpr int kRowCap = 256;  // the node's own row, staged when it fits
  __shared__ int32_t s_rows[WARPS][kRowCap];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t smask = (uint32_t)m.nbr_set_cap - 1u;
  int32_t* set = s_sets + (size_t)warp * m.nbr_set_cap;
  int32_t* srow = s_rows[warp];
  const int n_nodes = b.st->n_nodes;
  const uint32_t step = b.st->step;
  const Stream rs{m.seed, m.chain};
  const uint64_t cap = 64ull * (uint64_t)m.n_out + 4096ull;
  // eps_t of the iteration (get_eps_t, cc:143; read by the update kernels alone): an
  // FP64 power, computed by the grid's last warp, which the launch leaves
  // without a node (the grid has a warp more than the nodes) and which no
  // other warp waits for; in the single-CTA minibatch kernel its latency
  // delayed every block barrier (2.8 us of each minibatch)
  if (blockIdx.x == gridDim.x - 1 && warp == WARPS - 1 && lane == 0)
    b.st->eps = eps_schedule(m.a, m.b, m.c, step);
  for (int slot = blockIdx.x * WARPS + warp; slot < n_nodes; slot += gridDim.x * WARPS) {
    const int32_t i = b.nodes[slot];
    const int64_t ir0 = g.row_ptr[i];
    const int32_t ideg = (int32_t)(g.row_ptr[i + 1] - ir0);
    const bool row_in_smem = ideg <= kRowCap;
    if (row_in_smem)
      for (int q = lane; q < ideg; q += 32) srow[q] = g.col[ir0 + q];
    for (uint32_t q = lane; q <= smask; q += 32) set[q] = -1;
    __syncwarp();
    int count = 0;
    uint64_t t = 0;
    while (count < m.n_out) {
      if (t >= cap) {
        if (lane == 0) atomicOr(&b.gc->err, kErrNeighborCap);
        break;
      }
      const int32_t j = (int32_t)uniform_below(rs.draw_u64(kTagNbr, (uint32_t)i, step, t + lane),
                                               (uint64_t)g.n);
      const unsigned long long key = pair_key(i, j);
      const unsigned long long xs = hash64(key) & g.excl_mask;
      const unsigned long long xk = __ldg(g.excl + xs);
      bool ok = (j != i) && !probe_resolve(g.excl, g.excl_mask, key, xs, xk);
      if (ok) {  // already accepted in an earlier round?
        uint32_t h = hash32((uint32_t)j) & smask;
        for (uint32_t probe = 0; probe <= smask; ++probe) {
          const int32_t e = set[h];
          if (e == j) {
            ok = false;
            break;
          }
          if (e < 0) break;
          h = (h + 1) & smask;
        }
      }
      const uint32_t peers = __match_any_sync(0xffffffffu, j);
      ok = ok && ((peers & lanemask_lt()) == 0);
      const uint32_t bal = __ballot_sync(0xffffffffu, ok);
      const int pos = __popc(bal & lanemask_lt());
      const int need = m.n_out - count;
      __syncwarp();  // every lane has probed the set before it grows
      if (ok && pos < need) {
        const int idx = count + pos;
        uint32_t h = hash32((uint32_t)j) & smask;
        for (uint32_t probe = 0; probe <= smask; ++probe) {
          if (atomicCAS(set + h, -1, j) == -1) break;
          h = (h + 1) & smask;
        }
        const uint32_t y = (row_in_smem ? row_contains(srow, ideg, j) : has_edge(g, i, j)) ? 1u : 0u;
        b.nbr[(int64_t)slot * m.n_out + idx] = (uint32_t)j | (y << 31);
      }
      count += min(__popc(bal), need);
      t += 32;
      __syncwarp();
    }
    __syncwarp();  // srow and set are reused by the warp's next node
  }
}
template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_sample_neighbors(Model m, DevGraph g, Buffers b) {
  sample_neighbors_body<WARPS>(m, g, b);
}
template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_sample_neighbors_chains(const ChainArgs* __restrict__ c,
                                                                      int p) {
  const ChainArgs& a = c[blockIdx.y];
  sample_neighbors_body<WARPS>(a.m, a.g, a.b[p]);
}

// ---------------------------------------------------------------------------
// k_update_phi: update_phi (cc:269-313) for NPB minibatch nodes per CTA,
// SPLIT sub-groups of LPN lanes per node, each lane holding VPL 16-byte
// vectors of a pi row.  Sub-group s takes neighbours s, s+SPLIT, ...
//
// Algebra (exact rewrite of the reference's per-k loop).  With
// pi_ik = phi_ik / S, sigma_j = +1 for y=1 else -1, e_j = y ? eps : 1-eps,
// bk = beta_k - epsilon and w_k = pi_ik * bk:
//   probs_jk = pi_ik (sigma_j bk pi_jk + e_j)
//   P_j      = sum_k probs_jk = sigma_j D_j + e_j s_i,
//              D_j = sum_k w_k pi_jk,  s_i = sum_k pi_ik
//   grad_k   = sum_j probs_jk / (P_j phi_ik) - 1/S
//            = (bk A_k + B) / S,  A_k = sum_j (sigma_j / P_j) pi_jk,
//              B = sum_j (e_j (1 - s_i) - sigma_j D_j) / P_j
// so each neighbour row costs two FMAs per element (D_j, then A_k).
// Epilogue: phi_ik <- |phi + eps/2 (alpha - phi + Nn grad) + sqrt(eps phi)
// noise|, clamped to 1e-24; the new row is normalised into the staging
// buffer (pi itself is written after all nodes, by k_commit_beta).
// ---------------------------------------------------------------------------
template <typename PiT, int LPN, int VPL, int SPLIT, int NPB>
__device__ __forceinline__ void update_phi_body(const Model& m, const Buffers& b) {
  using TR = PiTraits<PiT>;
  constexpr int EV = TR::kPerVec;
  constexpr int EPL = VPL * EV;
  constexpr int TPN = SPLIT * LPN;
  extern __shared__ float s_dyn[];
  float* s_A = s_dyn;                               // NPB x SPLIT x Kp
  float* s_B = s_A + (size_t)NPB * SPLIT * m.Kp;    // NPB x SPLIT
  float* s_red = s_B + NPB * SPLIT;                 // NPB x (TPN/32 or 1)

  const int tid = threadIdx.x;
  const int ln = tid / TPN;          // node within the CTA
  const int r = tid - ln * TPN;      // thread within the node
  const int sg = r / LPN;            // sub-group
  const int l = r - sg * LPN;        // lane within the sub-group
  const int warp_lane = tid & 31;
  const uint32_t gmask = group_mask<LPN>(warp_lane);
  const int n_nodes = b.st->n_nodes;
  const uint32_t step = b.st->step;
  const float eps_t = b.st->eps;
  const int Kp = m.Kp, K = m.K;
  const int nvec = Kp / EV;
  const PiT* __restrict__ pi = reinterpret_cast<const PiT*>(b.pi);
  const Stream rs{m.seed, m.chain};

  for (int base = blockIdx.x * NPB; base < n_nodes; base += gridDim.x * NPB) {
    const int slot = base + ln;
    const bool active = slot < n_nodes;
    float S = 0.f, s_i = 0.f, Bsum = 0.f;
    if (active) {
      const int32_t i = b.nodes[slot];
      const float* phi_i = b.phi + (int64_t)i * Kp;
      float w[EPL], A[EPL];
      // phi row -> S
#pragma unroll
      for (int v = 0; v < VPL; ++v) {
        const int vi = l + LPN * v;
#pragma unroll
        for (int e = 0; e < EV; ++e) {
          const int k = vi * EV + e;
          w[v * EV + e] = (vi < nvec) ? phi_i[k] : 0.f;
          S += w[v * EV + e];
        }
      }
#pragma unroll
      for (int o = LPN / 2; o > 0; o >>= 1) S += __shfl_xor_sync(gmask, S, o);
      // pi_i = phi_i / S, s_i = sum pi_i, w = pi_i * (beta - epsilon)
#pragma unroll
      for (int v = 0; v < VPL; ++v) {
        const int vi = l + LPN * v;
#pragma unroll
        for (int e = 0; e < EV; ++e) {
          const int k = vi * EV + e;
          const float p = __fdiv_rn(w[v * EV + e], S);
          s_i += p;
          const float bk = (vi < nvec && k < K) ? (b.beta[k] - m.epsilon) : 0.f;
          w[v * EV + e] = p * bk;
          A[v * EV + e] = 0.f;
        }
      }
#pragma unroll
      for (int o = LPN / 2; o > 0; o >>= 1) s_i += __shfl_xor_sync(gmask, s_i, o);
      const float one_m_si = 1.0f - s_i;
      const uint32_t* nb = b.nbr + (int64_t)slot * m.n_out;

      // neighbour loop, one row prefetched ahead
      uint4 cur[VPL], nxt[VPL];
      uint32_t wcur = 0, wnxt = 0;
      int q = sg;
      if (q < m.n_out) {
        wcur = nb[q];
        const PiT* row = pi + (int64_t)(wcur & 0x7fffffffu) * Kp;
#pragma unroll
        for (int v = 0; v < VPL; ++v) {
          const int vi = l + LPN * v;
          cur[v] = (vi < nvec) ? ldg_nc_v4(row + vi * EV) : make_uint4(0, 0, 0, 0);
        }
      }
      for (; q < m.n_out; q += SPLIT) {
        const int qn = q + SPLIT;
        if (qn < m.n_out) {
          wnxt = nb[qn];
          const PiT* row = pi + (int64_t)(wnxt & 0x7fffffffu) * Kp;
#pragma unroll
          for (int v = 0; v < VPL; ++v) {
            const int vi = l + LPN * v;
            nxt[v] = (vi < nvec) ? ldg_nc_v4(row + vi * EV) : make_uint4(0, 0, 0, 0);
          }
        }
        float x[EPL];
#pragma unroll
        for (int v = 0; v < VPL; ++v) TR::unpack(cur[v], x + v * EV);
        float d4[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int e = 0; e < EPL; ++e) d4[e & 3] = fmaf(w[e], x[e], d4[e & 3]);
        float D = (d4[0] + d4[1]) + (d4[2] + d4[3]);
#pragma unroll
        for (int o = LPN / 2; o > 0; o >>= 1) D += __shfl_xor_sync(gmask, D, o);
        const bool y = (wcur >> 31) != 0;
        const float sg_ = y ? 1.f : -1.f;
        const float ej = y ? m.epsilon : 1.0f - m.epsilon;
        const float P = fmaf(sg_, D, ej * s_i);
        const float invP = rcp_approx(P);
        const float cj = sg_ * invP;
        Bsum += (ej * one_m_si - sg_ * D) * invP;
#pragma unroll
        for (int e = 0; e < EPL; ++e) A[e] = fmaf(cj, x[e], A[e]);
#pragma unroll
        for (int v = 0; v < VPL; ++v) cur[v] = nxt[v];
        wcur = wnxt;
      }
      // publish A and B of this sub-group
      float* sA = s_A + ((size_t)ln * SPLIT + sg) * Kp;
#pragma unroll
      for (int v = 0; v < VPL; ++v) {
        const int vi = l + LPN * v;
        if (vi < nvec) {
#pragma unroll
          for (int e = 0; e < EV; ++e) sA[vi * EV + e] = A[v * EV + e];
        }
      }
      if (l == 0) s_B[ln * SPLIT + sg] = Bsum;
    }
    __syncthreads();
    // epilogue: TPN threads per node, element k = r + TPN * q
    // each sub-group covers the whole row: Kp <= LPN * EPL = TPN * EPL / SPLIT
    constexpr int NQ = (EPL + SPLIT - 1) / SPLIT;
    float pnew[NQ];
    float Snew = 0.f;
    int32_t i = 0;
    if (active) {
      i = b.nodes[slot];
      float Bt = 0.f;
#pragma unroll
      for (int s = 0; s < SPLIT; ++s) Bt += s_B[ln * SPLIT + s];
      float* phi_i = b.phi + (int64_t)i * Kp;
      const float invS = 1.0f / S;
      const float half_eps = eps_t / 2.0f;
#pragma unroll
      for (int qq = 0; qq < NQ; ++qq) {
        const int k = r + TPN * qq;
        float val = 0.f;
        if (k < K) {
          float Ak = 0.f;
#pragma unroll
          for (int s = 0; s < SPLIT; ++s) Ak += s_A[((size_t)ln * SPLIT + s) * Kp + k];
          const float bk = b.beta[k] - m.epsilon;
          const float grad = (bk * Ak + Bt) * invS;
          const float noise = b.fed_phi_noise
                                  ? b.fed_phi_noise[(int64_t)slot * K + k]
                                  : normal_draw(rs, kTagPhiNoise, (uint32_t)i, step, (uint64_t)k);
          const float ph = phi_i[k];
          val = fabsf((ph + half_eps * (m.alpha - ph + m.Nn * grad)) + sqrtf(eps_t * ph) * noise);
          if (val < 1.0e-24f) val = 1.0e-24f;
          phi_i[k] = val;
        }
        pnew[qq] = val;
        Snew += val;
      }
    }
    // sum of the new row over the node's TPN threads
    if constexpr (TPN <= 32) {
#pragma unroll
      for (int o = TPN / 2; o > 0; o >>= 1) Snew += __shfl_xor_sync(group_mask<TPN>(warp_lane), Snew, o);
    } else {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) Snew += __shfl_xor_sync(0xffffffffu, Snew, o);
      if (warp_lane == 0) s_red[ln * (TPN / 32) + (r >> 5)] = Snew;
      __syncthreads();
      Snew = 0.f;
#pragma unroll
      for (int w2 = 0; w2 < TPN / 32; ++w2) Snew += s_red[ln * (TPN / 32) + w2];
    }
    if (active) {
      float* st = b.stage + (int64_t)slot * Kp;
#pragma unroll
      for (int qq = 0; qq < NQ; ++qq) {
        const int k = r + TPN * qq;
        if (k < Kp) st[k] = (k < K) ? __fdiv_rn(pnew[qq], Snew) : 0.f;
      }
    }
    __syncthreads();
  }
}
template <typename PiT, int LPN, int VPL, int SPLIT, int NPB>
__global__ void __launch_bounds__(NPB * SPLIT * LPN) k_update_phi(Model m, Buffers b) {
  update_phi_body<PiT, LPN, VPL, SPLIT, NPB>(m, b);
}
template <typename PiT, int LPN, int VPL, int SPLIT, int NPB>
__global__ void __launch_bounds__(NPB * SPLIT * LPN) k_update_phi_chains(const ChainArgs* __restrict__ c,
                                                                         int p) {
  const ChainArgs& a = c[blockIdx.y];
  update_phi_body<PiT, LPN, VPL, SPLIT, NPB>(a.m, a.b[p]);
}

// ---------------------------------------------------------------------------
// k_commit_beta: blocks [0, ncommit) copy the staged rows into pi (the
// reference's update_pi loop, cc:162-166); blocks [ncommit, ncommit+nbb)
// evaluate update_beta's per-edge terms (cc:212-240) on the staged (new) pi
// and reduce them per block.  With f_k = pi_ak pi_bk, P_e = sum_k
// (y ? beta_k : 1-beta_k) f_k + (y ? eps : 1-eps)(1 - sum_k f_k) the
// gradient only needs R_yk = sum_{e: y_e = y} f_ek / P_e (k_theta applies the
// theta factors), accumulated per warp in registers, then per block.
// ---------------------------------------------------------------------------
template <typename PiT, int KQ>
__device__ __forceinline__ void commit_beta_body(const Model& m, const Buffers& b, int ncommit) {
  using TR = PiTraits<PiT>;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int Kp = m.Kp, K = m.K;
  if ((int)blockIdx.x < ncommit) {
    const int n_nodes = b.st->n_nodes;
    constexpr int EV = TR::kPerVec;
    PiT* pi = reinterpret_cast<PiT*>(b.pi);
    const int nvec = Kp / EV;
    // the staged rows come from update_phi, the launch ahead of this one,
    // which also still reads the pi rows written here
    grid_dependency_wait();
    grid_launch_dependents();
    for (int slot = blockIdx.x * 4 + warp; slot < n_nodes; slot += ncommit * 4) {
      const int32_t i = b.nodes[slot];
      const float* src = b.stage + (int64_t)slot * Kp;
      PiT* dst = pi + (int64_t)i * Kp;
      // a vector's EV floats of the staged row (16-byte aligned: Kp is a
      // multiple of EV) as float4 loads
      for (int vi = lane; vi < nvec; vi += 32) {
        float x[EV];
#pragma unroll
        for (int e = 0; e < EV; e += 4) {
          const float4 q = *reinterpret_cast<const float4*>(src + vi * EV + e);
          x[e] = q.x;
          x[e + 1] = q.y;
          x[e + 2] = q.z;
          x[e + 3] = q.w;
        }
        *reinterpret_cast<uint4*>(dst + vi * EV) = TR::pack(x);
      }
    }
    return;
  }
  __shared__ float s_part[4][2][KQ * 128];
  const int bb = blockIdx.x - ncommit;
  const int n_edges = b.st->n_edges;
  if (bb >= m.nbb || bb * 4 >= n_edges) {  // no edges for this block: k_theta skips its partial
    grid_dependency_wait();
    return;
  }
  float R0[KQ * 4], R1[KQ * 4], bt[KQ * 4];
#pragma unroll
  for (int q = 0; q < KQ; ++q)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int k = q * 128 + lane * 4 + e;
      R0[q * 4 + e] = 0.f;
      R1[q * 4 + e] = 0.f;
      bt[q * 4 + e] = (k < K) ? b.beta[k] : 0.f;
    }
  grid_dependency_wait();  // the staged rows (update_phi)
  grid_launch_dependents();
  for (int ed = bb * 4 + warp; ed < n_edges; ed += m.nbb * 4) {
    const float* pa = b.stage + (int64_t)b.ea[ed] * Kp;
    const float* pb = b.stage + (int64_t)b.eb[ed] * Kp;
    const bool y = b.ey[ed] != 0;
    float f[KQ * 4];
    float fsum = 0.f, psum = 0.f;
#pragma unroll
    for (int q = 0; q < KQ; ++q) {
      const int k0 = q * 128 + lane * 4;
      float4 xa = make_float4(0, 0, 0, 0), xb = make_float4(0, 0, 0, 0);
      if (k0 < Kp) {
        xa = *reinterpret_cast<const float4*>(pa + k0);
        xb = *reinterpret_cast<const float4*>(pb + k0);
      }
      f[q * 4 + 0] = xa.x * xb.x;
      f[q * 4 + 1] = xa.y * xb.y;
      f[q * 4 + 2] = xa.z * xb.z;
      f[q * 4 + 3] = xa.w * xb.w;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float fk = f[q * 4 + e];
        fsum += fk;
        psum += (y ? bt[q * 4 + e] : (k0 + e < K ? 1.0f - bt[q * 4 + e] : 0.f)) * fk;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      fsum += __shfl_xor_sync(0xffffffffu, fsum, o);
      psum += __shfl_xor_sync(0xffffffffu, psum, o);
    }
    const float prob0 = (y ? m.epsilon : 1.0f - m.epsilon) * (1.0f - fsum);
    const float invP = 1.0f / (psum + prob0);
    if (y) {
#pragma unroll
      for (int e = 0; e < KQ * 4; ++e) R1[e] = fmaf(f[e], invP, R1[e]);
    } else {
#pragma unroll
      for (int e = 0; e < KQ * 4; ++e) R0[e] = fmaf(f[e], invP, R0[e]);
    }
  }
#pragma unroll
  for (int q = 0; q < KQ; ++q)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      s_part[warp][0][q * 128 + lane * 4 + e] = R0[q * 4 + e];
      s_part[warp][1][q * 128 + lane * 4 + e] = R1[q * 4 + e];
    }
  __syncthreads();
  float* out = b.beta_part + (int64_t)bb * 2 * Kp;
  for (int k = threadIdx.x; k < Kp; k += 128) {
    out[k] = s_part[0][0][k] + s_part[1][0][k] + s_part[2][0][k] + s_part[3][0][k];
    out[Kp + k] = s_part[0][1][k] + s_part[1][1][k] + s_part[2][1][k] + s_part[3][1][k];
  }
}
template <typename PiT, int KQ>
__global__ void __launch_bounds__(128) k_commit_beta(Model m, Buffers b, int ncommit) {
  commit_beta_body<PiT, KQ>(m, b, ncommit);
}
template <typename PiT, int KQ>
__global__ void __launch_bounds__(128) k_commit_beta_chains(const ChainArgs* __restrict__ c, int p) {
  const ChainArgs& a = c[blockIdx.y];
  commit_beta_body<PiT, KQ>(a.m, a.b[p], a.ncommit);
}

// ---------------------------------------------------------------------------
// The parts of k's step that do not depend on the sums: 1/(theta0+theta1),
// the two gradient factors 1/theta_kc - 1/ts, and the two noise terms
// sqrt(eps theta_kc) n_kc -- three FP64 divisions and two square roots.
struct ThetaPre {
  double ts_inv, f0, f1, nz0, nz1;
};
static __device__ __forceinline__ ThetaPre theta_pre(const Model& m, const Buffers& b, int k,
                                                     uint32_t step, double eps_t, double th0,
                                                     double th1) {
  ThetaPre p;
  p.ts_inv = 1.0 / (th0 + th1);
  p.f0 = 1.0 / th0 - p.ts_inv;
  p.f1 = 1.0 / th1 - p.ts_inv;
  const Stream rs{m.seed, m.chain};
  double n0, n1;
  if (b.fed_theta_noise) {
    n0 = b.fed_theta_noise[2 * k];
    n1 = b.fed_theta_noise[2 * k + 1];
  } else {
    n0 = normal_draw(rs, kTagThetaNoise, 0, step, 2ull * k);
    n1 = normal_draw(rs, kTagThetaNoise, 0, step, 2ull * k + 1);
  }
  p.nz0 = sqrt(eps_t * th0) * n0;
  p.nz1 = sqrt(eps_t * th1) * n1;
  return p;
}

// k_theta: theta step of update_beta (cc:241-266) in FP64.  With the block
// sums R0_k, R1_k and beta_k the gradients of cc:236-239 are
//   G_k0 = beta R1 (0 - 1/ts) + (1-beta) R0 (1/theta_k0 - 1/ts)
//   G_k1 = beta R1 (1/theta_k1 - 1/ts) + (1-beta) R0 (0 - 1/ts)
// ---------------------------------------------------------------------------
// With R_given the sums are read from it (R0_k, R1_k at 2k, 2k + 1) instead
// of being formed from the partials; with R_out the sums are written there
// and no step is taken (the phases of a sharded iteration).
static __device__ __forceinline__ void theta_body(const Model& m, const Buffers& b,
                                                  const double* R_given = nullptr,
                                                  double* R_out = nullptr) {
  // 32 consecutive k per CTA (lane = k); warps 0-30 sum the partials of the
  // active beta blocks w, w+31, ... in FP32 with Kahan compensation while
  // warp 31 forms the FP64 parts of the step that do not need the sums;
  // then warp 0 adds the 31 warp sums in fixed order (deterministic) and
  // finishes the step: two FMA chains and one division after the barrier.
  constexpr int kSumWarps = kThetaSumWarps;
  __shared__ float s_r0[kSumWarps][33], s_c0[kSumWarps][33], s_r1[kSumWarps][33], s_c1[kSumWarps][33];
  __shared__ double s_pre[5][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int k = blockIdx.x * 32 + lane;
  const int Kp = m.Kp;
  const int active = min(m.nbb, (b.st->n_edges + 3) / 4);  // blocks that saw edges
  // the step's scalars and this k's theta and beta, fetched now so that their
  // latency overlaps the partial sums
  const uint32_t step = b.st->step;
  const double eps_t = (double)b.st->eps;
  const double scale = (double)b.st->scale;
  const bool kin = k < m.K;
  const double th0 = kin ? b.theta[2 * k] : 1.0, th1 = kin ? b.theta[2 * k + 1] : 1.0;
  const double bt = kin ? (double)b.beta[k] : 0.0;
  grid_dependency_wait();  // the beta partials: k_commit_beta, the launch ahead
  grid_launch_dependents();
  double R0, R1;
  ThetaPre pre;
  if (R_given) {
    if (warp != 0 || !kin) return;
    R0 = R_given[2 * k];
    R1 = R_given[2 * k + 1];
    pre = theta_pre(m, b, k, step, eps_t, th0, th1);
  } else {
    if (warp == kSumWarps) {
      if (kin && !R_out) {
        const ThetaPre q = theta_pre(m, b, k, step, eps_t, th0, th1);
        s_pre[0][lane] = q.ts_inv;
        s_pre[1][lane] = q.f0;
        s_pre[2][lane] = q.f1;
        s_pre[3][lane] = q.nz0;
        s_pre[4][lane] = q.nz1;
      }
    } else {
      // the warp's partials (blocks warp, warp + 31, ...) loaded together,
      // then added in block order
      float r0 = 0.f, c0 = 0.f, r1 = 0.f, c1 = 0.f;
      constexpr int P = kThetaPerPass;
      for (int base = warp; base < active; base += kSumWarps * P) {
        float p0v[P], p1v[P];
#pragma unroll
        for (int q = 0; q < P; ++q) {
          const int bb = base + kSumWarps * q;
          const bool on = kin && bb < active;
          const float* p0 = b.beta_part + (int64_t)bb * 2 * Kp + k;
          p0v[q] = on ? p0[0] : 0.f;
          p1v[q] = on ? p0[Kp] : 0.f;
        }
#pragma unroll
        for (int q = 0; q < P; ++q) {
          if (base + kSumWarps * q < active) {
            const float y0 = p0v[q] - c0, y1 = p1v[q] - c1;
            const float t0 = r0 + y0, t1 = r1 + y1;
            c0 = (t0 - r0) - y0;
            c1 = (t1 - r1) - y1;
            r0 = t0;
            r1 = t1;
          }
        }
      }
      s_r0[warp][lane] = r0;
      s_c0[warp][lane] = c0;
      s_r1[warp][lane] = r1;
      s_c1[warp][lane] = c1;
    }
    __syncthreads();
    if (warp != 0 || k >= m.K) return;
    float a0 = 0.f, e0 = 0.f, a1 = 0.f, e1 = 0.f;  // Kahan over the warp sums
#pragma unroll
    for (int w = 0; w < kSumWarps; ++w) {
      const float y0 = (s_r0[w][lane] - s_c0[w][lane]) - e0;
      const float y1 = (s_r1[w][lane] - s_c1[w][lane]) - e1;
      const float t0 = a0 + y0, t1 = a1 + y1;
      e0 = (t0 - a0) - y0;
      e1 = (t1 - a1) - y1;
      a0 = t0;
      a1 = t1;
    }
    R0 = (double)a0 - (double)e0;
    R1 = (double)a1 - (double)e1;
    if (R_out) {
      R_out[2 * k] = R0;
      R_out[2 * k + 1] = R1;
      return;
    }
    pre.ts_inv = s_pre[0][lane];
    pre.f0 = s_pre[1][lane];
    pre.f1 = s_pre[2][lane];
    pre.nz0 = s_pre[3][lane];
    pre.nz1 = s_pre[4][lane];
  }
  if (k == 0) {  // the iteration's edge evaluations, counted once it is applied
    b.gc->evals += (unsigned long long)b.st->n_nodes * (unsigned long long)m.n_out;
    b.gc->iters += 1ull;
  }
  const double G0 = bt * R1 * (-pre.ts_inv) + (1.0 - bt) * R0 * pre.f0;
  const double G1 = bt * R1 * pre.f1 + (1.0 - bt) * R0 * (-pre.ts_inv);
  double t0 = fabs(th0 + eps_t / 2.0 * ((double)m.eta0 - th0 + scale * G0) + pre.nz0);
  double t1 = fabs(th1 + eps_t / 2.0 * ((double)m.eta1 - th1 + scale * G1) + pre.nz1);
  if (t0 < 1.0e-24) t0 = 1.0e-24;
  if (t1 < 1.0e-24) t1 = 1.0e-24;
  b.theta[2 * k] = t0;
  b.theta[2 * k + 1] = t1;
  b.beta[k] = (float)(t1 / (t0 + t1));
}
static __global__ void __launch_bounds__(1024) k_theta(Model m, Buffers b) { theta_body(m, b); }
// the per-k sums R0, R1 of the beta partials, without the step
static __global__ void __launch_bounds__(1024) k_beta_sums(Model m, Buffers b, double* R_out) {
  theta_body(m, b, nullptr, R_out);
}
// the theta step from given sums
static __global__ void __launch_bounds__(1024) k_theta_given(Model m, Buffers b, const double* R) {
  theta_body(m, b, R, nullptr);
}
static __global__ void __launch_bounds__(1024) k_theta_chains(const ChainArgs* __restrict__ c, int p) {
  const ChainArgs& a = c[blockIdx.y];
  theta_body(a.m, a.b[p]);
}

// ---------------------------------------------------------------------------
// Held-out perplexity (learner.cc:138-183, learner.h:100-139): LPN lanes per
// held-out edge; running average per edge in FP32 as the reference; the log
// sum in FP64 with Kahan compensation, block partials, then k_ppx_final.
// ---------------------------------------------------------------------------
template <typename PiT, int LPN, int VPL>
__global__ void __launch_bounds__(256) k_perplexity(Model m, const PiT* __restrict__ pi,
                                                    const float* __restrict__ beta,
                                                    const int32_t* __restrict__ ha,
                                                    const int32_t* __restrict__ hb,
                                                    const uint8_t* __restrict__ hy, int64_t H,
                                                    float* __restrict__ ppx, float count,
                                                    double* __restrict__ part, int64_t n_rows,
                                                    unsigned int* __restrict__ bad) {
  using TR = PiTraits<PiT>;
  constexpr int EV = TR::kPerVec;
  constexpr int EPL = VPL * EV;
  constexpr int GPB = 256 / LPN;
  const int tid = threadIdx.x, grp = tid / LPN, l = tid % LPN, lane = tid & 31;
  const uint32_t gmask = group_mask<LPN>(lane);
  // rows are Kp apart; only the vectors that hold the K values are read,
  // and elements past K (row padding) take no part in either sum
  const int Kp = m.Kp, K = m.K, nvec = (K + EV - 1) / EV;
  float bt[EPL];
#pragma unroll
  for (int v = 0; v < VPL; ++v)
#pragma unroll
    for (int e = 0; e < EV; ++e) {
      const int k = (l + LPN * v) * EV + e;
      bt[v * EV + e] = (k < K) ? beta[k] : 0.f;
    }
  double sum = 0.0, comp = 0.0;
  for (int64_t ed = (int64_t)blockIdx.x * GPB + grp; ed < H; ed += (int64_t)gridDim.x * GPB) {
    const int32_t a = ha[ed], b = hb[ed];
    // a pair naming a row outside pi is skipped (no row is read) and flagged
    if ((uint64_t)(int64_t)a >= (uint64_t)n_rows || (uint64_t)(int64_t)b >= (uint64_t)n_rows) {
      if (l == 0 && bad) atomicOr(bad, 1u);
      continue;
    }
    const PiT* ra = pi + (int64_t)a * Kp;
    const PiT* rb = pi + (int64_t)b * Kp;
    const bool y = hy[ed] != 0;
    float s = 0.f, fs = 0.f;
#pragma unroll
    for (int v = 0; v < VPL; ++v) {
      const int vi = l + LPN * v;
      if (vi < nvec) {
        float xa[EV], xb[EV];
        TR::unpack(ldg_nc_v4(ra + vi * EV), xa);
        TR::unpack(ldg_nc_v4(rb + vi * EV), xb);
#pragma unroll
        for (int e = 0; e < EV; ++e) {
          if (vi * EV + e < K) {
            const float f = xa[e] * xb[e];
            fs += f;
            s += f * (y ? bt[v * EV + e] : 1.0f - bt[v * EV + e]);
          }
        }
      }
    }
#pragma unroll
    for (int o = LPN / 2; o > 0; o >>= 1) {
      s += __shfl_xor_sync(gmask, s, o);
      fs += __shfl_xor_sync(gmask, fs, o);
    }
    if (l == 0) {
      if (!y) s += (1.0f - fs) * (1.0f - m.epsilon);
      if (s < 1.0e-30f) s = 1.0e-30f;
      const float avg = (ppx[ed] * (count - 1.0f) + s) / count;
      ppx[ed] = avg;
      const double term = log((double)avg) - comp;
      const double tsum = sum + term;
      comp = (tsum - sum) - term;
      sum = tsum;
    }
  }
  // block reduction, compensated pairwise in fixed order
  __shared__ double s_sum[256], s_comp[256];
  s_sum[tid] = sum;
  s_comp[tid] = comp;
  __syncthreads();
  if (tid == 0) {
    double t = 0.0, c = 0.0;
    for (int q = 0; q < 256; q += LPN) {
      const double term = (s_sum[q] - s_comp[q]) - c;
      const double ts = t + term;
      c = (ts - t) - term;
      t = ts;
    }
    part[2 * blockIdx.x] = t;
    part[2 * blockIdx.x + 1] = c;
  }
}

// The blocks' compensated partials, summed by one block of kPpxFinalThreads:
// thread j takes partials j, j + kPpxFinalThreads, ... in order (Kahan), then
// a fixed pairwise tree adds the threads' sums (deterministic).  One thread
// walking 1,216 partials in FP64 took ~230 us on GB300.
constexpr int kPpxFinalThreads = 256;
static __global__ void __launch_bounds__(kPpxFinalThreads) k_ppx_final(const double* part, int nblk, int64_t H,
                                                                       double* out) {
  __shared__ double s[kPpxFinalThreads];
  const int tid = threadIdx.x;
  double t = 0.0, c = 0.0;
  for (int q = tid; q < nblk; q += kPpxFinalThreads) {
    const double term = (part[2 * q] - part[2 * q + 1]) - c;
    const double ts = t + term;
    c = (ts - t) - term;
    t = ts;
  }
  s[tid] = t - c;
  __syncthreads();
#pragma unroll
  for (int w = kPpxFinalThreads / 2; w > 0; w >>= 1) {
    if (tid < w) s[tid] += s[tid + w];
    __syncthreads();
  }
  if (tid == 0) out[0] = H ? -(s[0] / (double)H) : 0.0;
}

// ---------------------------------------------------------------------------
// init: phi ~ Gamma(1,1) (cc:66), row normalisation into pi (cc:75)
// ---------------------------------------------------------------------------
static __global__ void k_init_phi(Model m, float* phi, double shape, double scale, int32_t* err) {
  const Stream rs{m.seed, m.chain};
  const int64_t total = m.N * (int64_t)m.Kp;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < total;
       x += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = x / m.Kp;
    const int k = (int)(x - v * m.Kp);
    phi[x] = (k < m.K) ? (float)gamma_draw(rs, kTagPhiInit, (uint32_t)v, (uint64_t)k, shape, scale, err)
                       : 0.f;
  }
}

// np::row_normalize (np.h:63-75): one warp per row, sum in FP32.
template <typename PiT>
__global__ void k_normalize_rows(Model m, const float* phi, PiT* pi) {
  using TR = PiTraits<PiT>;
  constexpr int EV = TR::kPerVec;
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int Kp = m.Kp, nvec = Kp / EV;
  for (int64_t v = w0; v < m.N; v += nw) {
    const float* src = phi + v * Kp;
    float s = 0.f;
    for (int k = lane; k < Kp; k += 32) s += src[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    PiT* dst = pi + v * Kp;
    for (int vi = lane; vi < nvec; vi += 32) {
      float x[EV];
#pragma unroll
      for (int e = 0; e < EV; ++e) x[e] = __fdiv_rn(src[vi * EV + e], s);
      *reinterpret_cast<uint4*>(dst + vi * EV) = TR::pack(x);
    }
  }
}

}  // namespace ammsb
