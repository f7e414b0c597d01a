// ammsb_phi_tma.cuh -- update_phi for wide pi rows (>= 512 bytes), with the
// neighbour rows staged in shared memory by the Blackwell bulk-copy engine.
//
// One CTA per minibatch node, SPLIT warps.  Warp g handles neighbours
// g, g+SPLIT, ...: its lane 0 keeps STAGES row copies in flight
// (cp.async.bulk global -> shared, completion counted on one mbarrier per
// stage); every lane waits on the stage's barrier, reads its 16-byte
// vectors of the row from shared memory and does the two FMA passes of the
// factored gradient (see k_update_phi in ammsb_kernels.cuh for the algebra).
// All waits are bounded: a wait that runs out sets kErrPipeline, drains the
// copies this warp still has in flight (also bounded) and the CTA skips its
// phi write, so a stuck copy cannot hang the GPU.
#pragma once
#include "ammsb_kernels.cuh"

namespace ammsb {

enum : int32_t { kErrPipeline = 16 };

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait: gives up after 200 ms (global timer) or 2^24 polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (uint32_t it = 0; it < (1u << 16); ++it) {
    for (int r = 0; r < 256; ++r)
      if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > 200000000ull) return false;
  }
  return false;
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Packed FP32 pairs (Blackwell fma.rn.f32x2): two IEEE round-to-nearest
// FMAs per instruction, element-wise identical to two scalar fmaf.
typedef unsigned long long f32x2;

__device__ __forceinline__ f32x2 pack_f32x2(float lo, float hi) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}

__device__ __forceinline__ void unpack_f32x2(f32x2 v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}

__device__ __forceinline__ f32x2 fma_f32x2(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

__device__ __forceinline__ f32x2 add_f32x2(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

// The 16 bytes of a row vector as EV/2 float pairs.
template <typename PiT>
struct PairLoad;

template <>
struct PairLoad<float> {
  __device__ __forceinline__ static void get(const uint4& v, f32x2* out) {
    out[0] = pack_f32x2(__uint_as_float(v.x), __uint_as_float(v.y));
    out[1] = pack_f32x2(__uint_as_float(v.z), __uint_as_float(v.w));
  }
};

template <>
struct PairLoad<__nv_bfloat16> {
  __device__ __forceinline__ static f32x2 word(uint32_t w) {
    return pack_f32x2(__uint_as_float(w << 16), __uint_as_float(w & 0xffff0000u));
  }
  __device__ __forceinline__ static void get(const uint4& v, f32x2* out) {
    out[0] = word(v.x);
    out[1] = word(v.y);
    out[2] = word(v.z);
    out[3] = word(v.w);
  }
};

__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// Predicated refill (no branch): when pred, arm `bar` for `bytes` and copy
// `bytes` from global `src` into shared `dst`, completing on `bar`.  The slot
// was last touched by the warp's own shared-memory reads, ordered before the
// copy by the __syncwarp that precedes it; a proxy fence is only needed after
// generic-proxy writes (the epilogue's A vectors), which the node's first
// copies follow.
__device__ __forceinline__ void bulk_copy_g2s_if(bool pred, void* dst, const void* src, uint32_t bytes,
                                                 uint64_t* bar) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %0, 0;\n\t"
      "@p mbarrier.arrive.expect_tx.shared::cta.b64 _, [%1], %4;\n\t"
      "@p cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%2], [%3], %4, [%1];\n\t}" ::"r"(
          (int)pred),
      "r"(smem_addr(bar)), "r"(smem_addr(dst)), "l"(src), "r"(bytes)
      : "memory");
}

template <typename PiT, int VPL, int SPLIT, int STAGES>
struct PhiTmaSmem {
  // BF16 rows keep the node's phi row and normals in shared memory across
  // the rows (two more rows of floats)
  static constexpr bool kStash = sizeof(PiT) == 2;
  // the per-warp A vectors of the epilogue reuse the warp's own ring slice
  static_assert(STAGES * sizeof(PiT) >= sizeof(float), "ring slice must hold a row of floats");
  static size_t bytes(int Kp, int n_out) {
    size_t ring = (size_t)SPLIT * STAGES * Kp * sizeof(PiT);
    size_t bars = (size_t)SPLIT * STAGES * sizeof(uint64_t);
    size_t w = (size_t)(kStash ? 3 : 1) * Kp * sizeof(float);
    size_t misc = (size_t)(4 * SPLIT + 8) * sizeof(float) + (size_t)n_out * sizeof(uint32_t);
    return ring + bars + w + misc + 128;
  }
};

// One row of the ring as the lane's float pairs (FULL: every lane's vectors
// lie inside the row).
template <typename PiT, int VPL, bool FULL>
__device__ __forceinline__ void load_row_pairs(const PiT* row, int lane, int nvec, f32x2* x2) {
  constexpr int EV = PiTraits<PiT>::kPerVec;
#pragma unroll
  for (int v = 0; v < VPL; ++v) {
    const int vi = lane + 32 * v;
    const uint4 raw = (FULL || vi < nvec) ? *reinterpret_cast<const uint4*>(row + vi * EV)
                                          : make_uint4(0, 0, 0, 0);
    PairLoad<PiT>::get(raw, x2 + v * (EV / 2));
  }
}

// The four normals of elements k0 .. k0+3 of node i's phi update (one
// Philox block), or the fed values when the caller supplies them.
__device__ __forceinline__ float4 phi_normals(const Buffers& b, const Stream& rs, int slot, int32_t i,
                                              uint32_t step, int k0, int K) {
  float4 nz = make_float4(0.f, 0.f, 0.f, 0.f);
  if (b.fed_phi_noise) {
    const float* f = b.fed_phi_noise + (int64_t)slot * K + k0;
    nz.x = (k0 + 0 < K) ? f[0] : 0.f;
    nz.y = (k0 + 1 < K) ? f[1] : 0.f;
    nz.z = (k0 + 2 < K) ? f[2] : 0.f;
    nz.w = (k0 + 3 < K) ? f[3] : 0.f;
  } else {
    const U32x4 o = rs.block(kTagPhiNoise, (uint32_t)i, step, (uint64_t)k0 >> 2);
    float s0, c0, s1, c1;
    const float r0 = sqrtf(-2.0f * logf(u24_open(o.x)));
    const float r1 = sqrtf(-2.0f * logf(u24_open(o.z)));
    sincospif(2.0f * u24(o.y), &s0, &c0);
    sincospif(2.0f * u24(o.w), &s1, &c1);
    nz.x = r0 * c0;
    nz.y = r0 * s0;
    nz.z = r1 * c1;
    nz.w = r1 * s1;
  }
  return nz;
}

// Each warp walks its rows in chunks of STAGES with the ring slot of every
// row a compile-time constant (the barriers are re-armed from phase 0 at
// every node), refilling each slot, branch-free, with the row STAGES ahead
// as soon as the row in it is consumed.  The neighbour word of the row in
// each slot rides in a register beside the slot.  When FULL the row length
// is the compile-time 32 * VPL * EV, so row offsets and sizes are constants.
// A node's first STAGES copies go out from as many lanes at once.  With
// BF16 rows (STASH) the node's phi row and its normals are read and drawn in
// the prologue, where they overlap the first copies, and kept in shared
// memory for the epilogue.
template <typename PiT, int VPL, int SPLIT, int STAGES, bool FULL>
__device__ __forceinline__ void update_phi_tma_body(const Model& m, const Buffers& b) {
  using TR = PiTraits<PiT>;
  using Smem = PhiTmaSmem<PiT, VPL, SPLIT, STAGES>;
  constexpr int EV = TR::kPerVec;
  constexpr int EPL = VPL * EV;
  constexpr int NT = SPLIT * 32;
  constexpr int NP = EPL / 2;  // float pairs per lane
  constexpr bool STASH = Smem::kStash;
  // thread's elements of a row: k0 = 4 * (tid + NT * g) .. k0 + 3, g < NG
  constexpr int NG = (EPL * 32 + 4 * NT - 1) / (4 * NT);
  static_assert((SPLIT * STAGES) % 2 == 0, "s_w must start on a 16-byte boundary");
  static_assert(STAGES <= 32, "one lane per first copy");
  extern __shared__ __align__(128) unsigned char s_raw[];
  const int Kp = FULL ? 32 * EPL : m.Kp;
  const int K = m.K, n_out = m.n_out;
  PiT* ring = reinterpret_cast<PiT*>(s_raw);
  uint64_t* bars = reinterpret_cast<uint64_t*>(ring + (size_t)SPLIT * STAGES * Kp);
  float* s_w = reinterpret_cast<float*>(bars + SPLIT * STAGES);
  float* s_phi = s_w + Kp;                    // STASH: the node's phi row
  float* s_nz = s_phi + Kp;                   // STASH: its normals
  float* s_red = s_w + (STASH ? 3 : 1) * Kp;  // 4*SPLIT + 8 floats
  uint32_t* s_nb = reinterpret_cast<uint32_t*>(s_red + 4 * SPLIT + 8);
  __shared__ int s_broken;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n_nodes = b.st->n_nodes;
  const uint32_t step = b.st->step;
  const float eps_t = b.st->eps;
  const PiT* __restrict__ pi = reinterpret_cast<const PiT*>(b.pi);
  const uint32_t row_bytes = (uint32_t)(Kp * sizeof(PiT));
  const int nvec = Kp / EV;
  const Stream rs{m.seed, m.chain};

  uint64_t* my_bars = bars + warp * STAGES;
  PiT* my_ring = ring + (size_t)warp * STAGES * Kp;
  float* my_A = reinterpret_cast<float*>(my_ring);  // epilogue: this warp's A (Kp floats)
  if (tid == 0) s_broken = 0;
  bool dead = false;   // a bounded wait ran out: this warp issues and waits no more
  bool armed = false;  // this warp's barriers hold valid mbarrier objects

  for (int slot = blockIdx.x; slot < n_nodes; slot += gridDim.x) {
    const int32_t i = b.nodes[slot];
    const float* phi_i = b.phi + (int64_t)i * Kp;
    const uint32_t* nbr_g = b.nbr + (int64_t)slot * n_out;
    // rows of this warp: q = warp + SPLIT * t, t < T
    const int T = (!dead && n_out > warp) ? (n_out - warp + SPLIT - 1) / SPLIT : 0;
    // lane 0 (re)arms the barriers at phase 0, then lanes 0 .. STAGES-1 each
    // send one of the first copies, before the node prologue, which they
    // overlap; the proxy fence orders the previous node's generic accesses
    // to the ring (its A vectors) before them
    if (!dead) {
      if (lane == 0) {
        for (int s = 0; s < STAGES; ++s) {
          if (armed) mbar_inval(my_bars + s);
          mbar_init(my_bars + s, 1);
        }
        fence_mbar_init();
      }
      armed = true;
      __syncwarp();
      const int pre = T < STAGES ? T : STAGES;
      if (lane < pre) {
        const uint32_t j = nbr_g[warp + SPLIT * lane] & 0x7fffffffu;
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(my_bars + lane, row_bytes);
        bulk_copy_g2s(my_ring + (size_t)lane * Kp, pi + (int64_t)j * Kp, row_bytes, my_bars + lane);
      }
    }
    __syncwarp();
    // ---- node prologue: S = sum phi, s_i = sum pi, w = pi * (beta - eps)
    float S = 0.f;
    float4 ph[STASH ? NG : 1];
    if constexpr (STASH) {
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        const int k0 = 4 * (tid + NT * g);
        ph[g] = (k0 < Kp) ? *reinterpret_cast<const float4*>(phi_i + k0) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
      for (int q = tid; q < n_out; q += NT) s_nb[q] = nbr_g[q];
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        const int k0 = 4 * (tid + NT * g);
        if (k0 < K) *reinterpret_cast<float4*>(s_nz + k0) = phi_normals(b, rs, slot, i, step, k0, K);
      }
#pragma unroll
      for (int g = 0; g < NG; ++g) S += (ph[g].x + ph[g].y) + (ph[g].z + ph[g].w);
    } else {
      for (int k = tid; k < Kp; k += NT) S += phi_i[k];
      for (int q = tid; q < n_out; q += NT) s_nb[q] = nbr_g[q];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) S += __shfl_xor_sync(0xffffffffu, S, o);
    if (lane == 0) s_red[warp] = S;
    __syncthreads();
    S = 0.f;
#pragma unroll
    for (int w = 0; w < SPLIT; ++w) S += s_red[w];
    float si = 0.f;
    if constexpr (STASH) {
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        const int k0 = 4 * (tid + NT * g);
        if (k0 < Kp) {
          const float4 bt = *reinterpret_cast<const float4*>(b.beta + k0);
          float4 p, wv;
          p.x = __fdiv_rn(ph[g].x, S);
          p.y = __fdiv_rn(ph[g].y, S);
          p.z = __fdiv_rn(ph[g].z, S);
          p.w = __fdiv_rn(ph[g].w, S);
          si += p.x;
          si += p.y;
          si += p.z;
          si += p.w;
          wv.x = (k0 + 0 < K) ? p.x * (bt.x - m.epsilon) : 0.f;
          wv.y = (k0 + 1 < K) ? p.y * (bt.y - m.epsilon) : 0.f;
          wv.z = (k0 + 2 < K) ? p.z * (bt.z - m.epsilon) : 0.f;
          wv.w = (k0 + 3 < K) ? p.w * (bt.w - m.epsilon) : 0.f;
          *reinterpret_cast<float4*>(s_w + k0) = wv;
          *reinterpret_cast<float4*>(s_phi + k0) = ph[g];
        }
      }
    } else {
      for (int k = tid; k < Kp; k += NT) {
        const float p = __fdiv_rn(phi_i[k], S);
        si += p;
        s_w[k] = (k < K) ? p * (b.beta[k] - m.epsilon) : 0.f;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) si += __shfl_xor_sync(0xffffffffu, si, o);
    if (lane == 0) s_red[SPLIT + warp] = si;
    __syncthreads();
    si = 0.f;
#pragma unroll
    for (int w = 0; w < SPLIT; ++w) si += s_red[SPLIT + w];
    // the per-row constants of y = 1 and y = 0
    const float one_m_si = 1.0f - si;
    const float e1si = m.epsilon * si, e0si = (1.0f - m.epsilon) * si;
    const float e1o = m.epsilon * one_m_si, e0o = (1.0f - m.epsilon) * one_m_si;

    f32x2 w2[NP], A2[NP];
#pragma unroll
    for (int v = 0; v < VPL; ++v) {
      const int vi = lane + 32 * v;
#pragma unroll
      for (int e = 0; e < EV; e += 4) {
        float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
        if (FULL || vi < nvec) q = *reinterpret_cast<const float4*>(s_w + vi * EV + e);
        w2[(v * EV + e) / 2] = pack_f32x2(q.x, q.y);
        w2[(v * EV + e) / 2 + 1] = pack_f32x2(q.z, q.w);
        A2[(v * EV + e) / 2] = 0ull;
        A2[(v * EV + e) / 2 + 1] = 0ull;
      }
    }
    // neighbour word of the row in each ring slot
    uint32_t nbw[STAGES];
#pragma unroll
    for (int u = 0; u < STAGES; ++u) nbw[u] = (u < T) ? s_nb[warp + SPLIT * u] : 0u;
    float Bsum = 0.f;
    int t_fail = -1;
    for (int t0 = 0; t0 < T && t_fail < 0; t0 += STAGES) {
      const uint32_t par = (uint32_t)(t0 / STAGES) & 1u;
#pragma unroll
      for (int u = 0; u < STAGES; ++u) {
        const int t = t0 + u;
        if (t >= T) break;
        // the lanes agree on the outcome, so a wait that ran out for one
        // lane sends the whole warp down the same path
        if (!__all_sync(0xffffffffu, mbar_wait_bounded(my_bars + u, par))) {
          t_fail = t;
          break;
        }
        // neighbour word of the row that refills this slot, read early
        const int tn = t + STAGES;
        const uint32_t nxt = (tn < T) ? s_nb[warp + SPLIT * tn] : nbw[u];
        const PiT* row = my_ring + (size_t)u * Kp;
        f32x2 x2[NP];
        load_row_pairs<PiT, VPL, FULL>(row, lane, nvec, x2);
        // four independent pair accumulators break the FMA dependency chain
        f32x2 d2[4] = {0ull, 0ull, 0ull, 0ull};
#pragma unroll
        for (int e = 0; e < NP; ++e) d2[e & 3] = fma_f32x2(w2[e], x2[e], d2[e & 3]);
        float D;
        {
          float lo, hi;
          unpack_f32x2(add_f32x2(add_f32x2(d2[0], d2[1]), add_f32x2(d2[2], d2[3])), lo, hi);
          D = lo + hi;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) D += __shfl_xor_sync(0xffffffffu, D, o);
        const bool y = (nbw[u] >> 31) != 0;
        const float Ds = y ? D : -D;
        const float P = Ds + (y ? e1si : e0si);
        const float invP = __frcp_rn(P);
        const float cj = y ? invP : -invP;
        Bsum += ((y ? e1o : e0o) - Ds) * invP;
        const f32x2 c2 = pack_f32x2(cj, cj);
#pragma unroll
        for (int e = 0; e < NP; ++e) A2[e] = fma_f32x2(c2, x2[e], A2[e]);
        __syncwarp();
        // refill slot u with row t + STAGES once every lane has read row t
        nbw[u] = nxt;
        bulk_copy_g2s_if(lane == 0 && tn < T, my_ring + (size_t)u * Kp, pi + (int64_t)(nxt & 0x7fffffffu) * Kp,
                         row_bytes, my_bars + u);
      }
    }
    if (t_fail >= 0) {
      // drain the copies still in flight: rows t_fail .. min(T, t_fail + STAGES) - 1
      dead = true;
      const int last = (T < t_fail + STAGES) ? T : t_fail + STAGES;
      for (int u = t_fail; u < last; ++u)
        mbar_wait_bounded(my_bars + (u % STAGES), (uint32_t)(u / STAGES) & 1u);
      if (lane == 0) {
        atomicOr(&b.gc->err, kErrPipeline);
        s_broken = 1;
      }
    }
    __syncwarp();
    // ---- publish A (into this warp's own ring slice, now idle) and B
#pragma unroll
    for (int v = 0; v < VPL; ++v) {
      const int vi = lane + 32 * v;
      if (FULL || vi < nvec) {
#pragma unroll
        for (int e = 0; e < EV; e += 4) {
          float4 q;
          unpack_f32x2(A2[(v * EV + e) / 2], q.x, q.y);
          unpack_f32x2(A2[(v * EV + e) / 2 + 1], q.z, q.w);
          *reinterpret_cast<float4*>(my_A + vi * EV + e) = q;
        }
      }
    }
    if (lane == 0) s_red[2 * SPLIT + warp] = Bsum;
    __syncthreads();
    float Bt = 0.f;
#pragma unroll
    for (int w2i = 0; w2i < SPLIT; ++w2i) Bt += s_red[2 * SPLIT + w2i];
    const float invS = 1.0f / S;
    const float half_eps = eps_t / 2.0f;
    const bool write = (s_broken == 0);
    float* phi_w = b.phi + (int64_t)i * Kp;
    float pn[NG][4];
    float Snew = 0.f;
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      const int k0 = 4 * (tid + NT * g);
      float nz[4] = {0.f, 0.f, 0.f, 0.f};
      float Ak[4] = {0.f, 0.f, 0.f, 0.f};
      float phk[4] = {0.f, 0.f, 0.f, 0.f};
      float btk[4] = {0.f, 0.f, 0.f, 0.f};
      if (k0 < K) {
        if constexpr (STASH) {
          const float4 q = *reinterpret_cast<const float4*>(s_nz + k0);
          const float4 r = *reinterpret_cast<const float4*>(s_phi + k0);
          nz[0] = q.x, nz[1] = q.y, nz[2] = q.z, nz[3] = q.w;
          phk[0] = r.x, phk[1] = r.y, phk[2] = r.z, phk[3] = r.w;
        } else {
          const float4 q = phi_normals(b, rs, slot, i, step, k0, K);
          nz[0] = q.x, nz[1] = q.y, nz[2] = q.z, nz[3] = q.w;
#pragma unroll
          for (int e = 0; e < 4; ++e) phk[e] = (k0 + e < K) ? phi_i[k0 + e] : 0.f;
        }
        const float4 bt = *reinterpret_cast<const float4*>(b.beta + k0);
        btk[0] = bt.x, btk[1] = bt.y, btk[2] = bt.z, btk[3] = bt.w;
        // A_k: the warps' partial sums, added in warp order (Kp is a
        // multiple of 4, so the four elements lie inside the row)
#pragma unroll
        for (int s = 0; s < SPLIT; ++s) {
          const float4 a = *reinterpret_cast<const float4*>(
              reinterpret_cast<const float*>(ring + (size_t)s * STAGES * Kp) + k0);
          Ak[0] += a.x;
          Ak[1] += a.y;
          Ak[2] += a.z;
          Ak[3] += a.w;
        }
      }
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int k = k0 + e;
        float val = 0.f;
        if (k < K) {
          const float bk = btk[e] - m.epsilon;
          const float grad = (bk * Ak[e] + Bt) * invS;
          const float ph = phk[e];
          val = fabsf((ph + half_eps * (m.alpha - ph + m.Nn * grad)) + sqrtf(eps_t * ph) * nz[e]);
          if (val < 1.0e-24f) val = 1.0e-24f;
        }
        pn[g][e] = val;
        Snew += val;
      }
      if (write && k0 < K) {
        if (k0 + 3 < K) {
          *reinterpret_cast<float4*>(phi_w + k0) = make_float4(pn[g][0], pn[g][1], pn[g][2], pn[g][3]);
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (k0 + e < K) phi_w[k0 + e] = pn[g][e];
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) Snew += __shfl_xor_sync(0xffffffffu, Snew, o);
    if (lane == 0) s_red[3 * SPLIT + warp] = Snew;
    __syncthreads();
    Snew = 0.f;
#pragma unroll
    for (int w2i = 0; w2i < SPLIT; ++w2i) Snew += s_red[3 * SPLIT + w2i];
    float* st = b.stage + (int64_t)slot * Kp;
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      const int k0 = 4 * (tid + NT * g);
      if (k0 < Kp) {
        float4 o;
        o.x = (k0 + 0 < K) ? __fdiv_rn(pn[g][0], Snew) : 0.f;
        o.y = (k0 + 1 < K) ? __fdiv_rn(pn[g][1], Snew) : 0.f;
        o.z = (k0 + 2 < K) ? __fdiv_rn(pn[g][2], Snew) : 0.f;
        o.w = (k0 + 3 < K) ? __fdiv_rn(pn[g][3], Snew) : 0.f;
        *reinterpret_cast<float4*>(st + k0) = o;
      }
    }
    // smem reuse by the next node: every thread's generic accesses to the
    // ring are ordered before the async proxy's next copies into it
    fence_proxy_async_smem();
    __syncthreads();
  }
}
// The iteration's node count picks the launch that does the work: the
// kernel runs when n_lo < n_nodes <= n_hi and returns at once otherwise.
// Iterations with few nodes (the link stratum: one vertex and its edges)
// take a 16-warp variant, whose warps each hold a quarter of the rows the
// 4-warp one gives them, so a node's rows are in flight together.
template <typename PiT, int VPL, int SPLIT, int STAGES, bool FULL>
__global__ void __launch_bounds__(SPLIT * 32, (SPLIT * 32 * 128 <= 16384) ? 4 : 1)
    k_update_phi_tma(Model m, Buffers b, int n_lo, int n_hi) {
  const int n_nodes = b.st->n_nodes;
  if (n_nodes <= n_lo || n_nodes > n_hi) return;
  update_phi_tma_body<PiT, VPL, SPLIT, STAGES, FULL>(m, b);
}
template <typename PiT, int VPL, int SPLIT, int STAGES, bool FULL>
__global__ void __launch_bounds__(SPLIT * 32, (SPLIT * 32 * 128 <= 16384) ? 4 : 1)
    k_update_phi_tma_chains(const ChainArgs* __restrict__ c, int p, int n_lo, int n_hi) {
  const ChainArgs& a = c[blockIdx.y];
  const int n_nodes = a.b[p].st->n_nodes;
  if (n_nodes <= n_lo || n_nodes > n_hi) return;
  update_phi_tma_body<PiT, VPL, SPLIT, STAGES, FULL>(a.m, a.b[p]);
}

}  // namespace ammsb
