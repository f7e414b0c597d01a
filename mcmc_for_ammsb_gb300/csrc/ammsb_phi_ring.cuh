// ammsb_phi_ring.cuh -- update_phi for wide pi rows (>= 512 bytes), with the
// neighbour rows staged in shared memory through a per-warp ring.
//
// One CTA per minibatch node, SPLIT warps.  Warp g handles neighbours
// g, g+SPLIT, ...: each of its lanes keeps its own 16-byte pieces of the
// next STAGES rows in flight (cp.async global -> shared, one commit group
// per row), waits for the row's group, reads back exactly the pieces it
// copied and does the two FMA passes of the factored gradient (see
// k_update_phi in ammsb_kernels.cuh for the algebra).  A lane never reads
// another lane's pieces of a row, so the ring needs no barrier; the waits are
// on the lane's own copies, which always complete.  (A variant with one
// cp.async.bulk copy per row and an mbarrier per slot measured 5% slower:
// its per-row barrier wait, warp vote, __syncwarp and single-lane issue cost
// more than four 16-byte copies per lane.)
#pragma once
#include "ammsb_kernels.cuh"

#ifndef AMMSB_RING_WARP_PROLOGUE
#define AMMSB_RING_WARP_PROLOGUE 0
#endif

namespace ammsb {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
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

template <typename PiT, int VPL, int SPLIT, int STAGES>
struct PhiRingSmem {
  // BF16 rows keep the node's phi row and normals in shared memory across
  // the rows (two more rows of floats)
  static constexpr bool kStash = sizeof(PiT) == 2;
  // the per-warp A vectors of the epilogue reuse the warp's own ring slice
  static_assert(STAGES * sizeof(PiT) >= sizeof(float), "ring slice must hold a row of floats");
  static size_t bytes(int Kp, int n_out) {
    size_t ring = (size_t)SPLIT * STAGES * Kp * sizeof(PiT);
    size_t w = (size_t)(kStash ? 3 : 1) * Kp * sizeof(float);
    size_t misc = (size_t)(4 * SPLIT + 8) * sizeof(float) + (size_t)n_out * sizeof(uint32_t);
    return ring + w + misc + 128;
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

// The lane's 16-byte pieces of a row (vectors lane + 32 v), copied into the
// same places of a ring slot by cp.async: a lane only ever reads back the
// pieces it copied itself.
template <typename PiT, int VPL, bool FULL>
__device__ __forceinline__ void copy_row_lane(PiT* dst, const PiT* src, int lane, int nvec) {
  constexpr int EV = PiTraits<PiT>::kPerVec;
#pragma unroll
  for (int v = 0; v < VPL; ++v) {
    const int vi = lane + 32 * v;
    if (FULL || vi < nvec)
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst + vi * EV)), "l"(src + vi * EV)
                   : "memory");
  }
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Each warp walks its rows in chunks of STAGES with the ring slot of every
// row a compile-time constant, refilling each slot with the row STAGES ahead
// as soon as the row's dot product has taken it into registers; every row
// commits one group (empty past the node's last row), so
// cp.async.wait_group STAGES-1 always means "this row is in".  The neighbour
// word of the row in each slot rides in a register beside the slot.  When
// FULL the row length is the compile-time 32 * VPL * EV, so row offsets and
// sizes are constants.  A node's first STAGES rows are sent before its
// prologue, which they overlap.  With BF16 rows (STASH) the node's phi row
// and its normals are read and drawn in the prologue and kept in shared
// memory for the epilogue.
template <typename PiT, int VPL, int SPLIT, int STAGES, bool FULL>
__device__ __forceinline__ void update_phi_ring_body(const Model& m, const Buffers& b) {
  using TR = PiTraits<PiT>;
  using Smem = PhiRingSmem<PiT, VPL, SPLIT, STAGES>;
  constexpr int EV = TR::kPerVec;
  constexpr int EPL = VPL * EV;
  constexpr int NT = SPLIT * 32;
  constexpr int NP = EPL / 2;  // float pairs per lane
  constexpr bool STASH = Smem::kStash;
  // thread's elements of a row: k0 = 4 * (tid + NT * g) .. k0 + 3, g < NG
  constexpr int NG = (EPL * 32 + 4 * NT - 1) / (4 * NT);
  extern __shared__ __align__(128) unsigned char s_raw[];
  const int Kp = FULL ? 32 * EPL : m.Kp;
  const int K = m.K, n_out = m.n_out;
  PiT* ring = reinterpret_cast<PiT*>(s_raw);
  float* s_w = reinterpret_cast<float*>(ring + (size_t)SPLIT * STAGES * Kp);
  float* s_phi = s_w + Kp;                    // STASH: the node's phi row
  float* s_nz = s_phi + Kp;                   // STASH: its normals
  float* s_red = s_w + (STASH ? 3 : 1) * Kp;  // 4*SPLIT + 8 floats
  uint32_t* s_nb = reinterpret_cast<uint32_t*>(s_red + 4 * SPLIT + 8);

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n_nodes = b.st->n_nodes;
  const uint32_t step = b.st->step;
  const float eps_t = b.st->eps;
  const PiT* __restrict__ pi = reinterpret_cast<const PiT*>(b.pi);
  const int nvec = Kp / EV;
  const Stream rs{m.seed, m.chain};

  PiT* my_ring = ring + (size_t)warp * STAGES * Kp;
  float* my_A = reinterpret_cast<float*>(my_ring);  // epilogue: this warp's A (Kp floats)

  for (int slot = blockIdx.x; slot < n_nodes; slot += gridDim.x) {
    const int32_t i = b.nodes[slot];
    const float* phi_i = b.phi + (int64_t)i * Kp;
    const uint32_t* nbr_g = b.nbr + (int64_t)slot * n_out;
    // rows of this warp: q = warp + SPLIT * t, t < T
    const int T = (n_out > warp) ? (n_out - warp + SPLIT - 1) / SPLIT : 0;
    // the first STAGES rows: ids read first, then every lane sends its
    // pieces, one commit group per row (empty past T), before the node
    // prologue, which they overlap
    uint32_t j0[STAGES];
#pragma unroll
    for (int t = 0; t < STAGES; ++t) j0[t] = (t < T) ? (nbr_g[warp + SPLIT * t] & 0x7fffffffu) : 0u;
    // (BF16) the thread's phi elements, loaded before the copies are sent
    float4 ph[STASH ? NG : 1];
    if constexpr (STASH) {
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        const int k0 = 4 * (tid + NT * g);
        ph[g] = (k0 < Kp) ? *reinterpret_cast<const float4*>(phi_i + k0) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
#pragma unroll
    for (int t = 0; t < STAGES; ++t) {
      if (t < T) copy_row_lane<PiT, VPL, FULL>(my_ring + (size_t)t * Kp, pi + (int64_t)j0[t] * Kp, lane, nvec);
      cp_async_commit();
    }
    float S, si;
    f32x2 w2[NP], A2[NP];
    if constexpr (STASH && AMMSB_RING_WARP_PROLOGUE) {
      // ---- node prologue, per warp (BF16 rows): every warp reads the whole
      // phi row in its lanes' vector layout and forms S = sum phi,
      // s_i = sum pi and w = pi * (beta - eps) with shuffles alone -- the same
      // operations on the same values in every warp, so the warps agree bit
      // for bit without a CTA barrier; the thread's own epilogue elements
      // (phi and the normals) go to its private stash places
      // the neighbour words of this warp's rows (q = warp + SPLIT t), which
      // only this warp reads
      for (int t = lane; t < T; t += 32) s_nb[warp + SPLIT * t] = nbr_g[warp + SPLIT * t];
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        const int k0 = 4 * (tid + NT * g);
        if (k0 < K) *reinterpret_cast<float4*>(s_nz + k0) = phi_normals(b, rs, slot, i, step, k0, K);
        if (k0 < Kp) *reinterpret_cast<float4*>(s_phi + k0) = ph[g];
      }
      float phv[EPL];
#pragma unroll
      for (int v = 0; v < VPL; ++v) {
        const int vi = lane + 32 * v;
#pragma unroll
        for (int e = 0; e < EV; e += 4) {
          const float4 q = (FULL || vi < nvec) ? *reinterpret_cast<const float4*>(phi_i + vi * EV + e)
                                               : make_float4(0.f, 0.f, 0.f, 0.f);
          phv[v * EV + e] = q.x;
          phv[v * EV + e + 1] = q.y;
          phv[v * EV + e + 2] = q.z;
          phv[v * EV + e + 3] = q.w;
        }
      }
      S = 0.f;
#pragma unroll
      for (int e = 0; e < EPL; e += 4) S += (phv[e] + phv[e + 1]) + (phv[e + 2] + phv[e + 3]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) S += __shfl_xor_sync(0xffffffffu, S, o);
      const float rS = 1.0f / S;  // pi = phi / S as phi * (1/S): within 1 ulp
      grid_dependency_wait();  // beta: written by the theta step ahead of this launch
      grid_launch_dependents();
      si = 0.f;
#pragma unroll
      for (int v = 0; v < VPL; ++v) {
        const int vi = lane + 32 * v;
#pragma unroll
        for (int e = 0; e < EV; e += 4) {
          float4 bt = make_float4(0.f, 0.f, 0.f, 0.f);
          if (FULL || vi < nvec) bt = *reinterpret_cast<const float4*>(b.beta + vi * EV + e);
          const int kb = vi * EV + e;
          float pv[4], wv[4];
          const float btv[4] = {bt.x, bt.y, bt.z, bt.w};
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            pv[u] = phv[v * EV + e + u] * rS;
            si += pv[u];
            wv[u] = (kb + u < K) ? pv[u] * (btv[u] - m.epsilon) : 0.f;
          }
          w2[(v * EV + e) / 2] = pack_f32x2(wv[0], wv[1]);
          w2[(v * EV + e) / 2 + 1] = pack_f32x2(wv[2], wv[3]);
          A2[(v * EV + e) / 2] = 0ull;
          A2[(v * EV + e) / 2 + 1] = 0ull;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) si += __shfl_xor_sync(0xffffffffu, si, o);
      __syncwarp();  // the warp's neighbour words are in
    } else {
      // ---- node prologue: S = sum phi, s_i = sum pi, w = pi * (beta - eps)
      S = 0.f;
      if constexpr (STASH) {
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
      // beta, read from here on, is written by the theta step ahead of this
      // launch; everything read before (node ids, neighbour words and rows,
      // phi) was complete before that step started
      grid_dependency_wait();
      grid_launch_dependents();
      S = 0.f;
#pragma unroll
      for (int w = 0; w < SPLIT; ++w) S += s_red[w];
      si = 0.f;
      if constexpr (STASH) {
        const float rS = 1.0f / S;  // pi = phi / S as phi * (1/S): within 1 ulp
#pragma unroll
        for (int g = 0; g < NG; ++g) {
          const int k0 = 4 * (tid + NT * g);
          if (k0 < Kp) {
            const float4 bt = *reinterpret_cast<const float4*>(b.beta + k0);
            float4 p, wv;
            p.x = ph[g].x * rS;
            p.y = ph[g].y * rS;
            p.z = ph[g].z * rS;
            p.w = ph[g].w * rS;
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
    }
    // the per-row constants of y = 1 and y = 0
    const float one_m_si = 1.0f - si;
    const float e1si = m.epsilon * si, e0si = (1.0f - m.epsilon) * si;
    const float e1o = m.epsilon * one_m_si, e0o = (1.0f - m.epsilon) * one_m_si;
    // neighbour word of the row in each ring slot
    uint32_t nbw[STAGES];
#pragma unroll
    for (int u = 0; u < STAGES; ++u) nbw[u] = (u < T) ? s_nb[warp + SPLIT * u] : 0u;
    float Bsum = 0.f;
    for (int t0 = 0; t0 < T; t0 += STAGES) {
#pragma unroll
      for (int u = 0; u < STAGES; ++u) {
        const int t = t0 + u;
        if (t >= T) break;
        // one group per row, so the lane's pieces of row t are in once no
        // more than the STAGES - 1 later groups are pending
        cp_async_wait<STAGES - 1>();
        // neighbour word of the row that refills this slot, read early
        const int tn = t + STAGES;
        const uint32_t nxt = (tn < T) ? s_nb[warp + SPLIT * tn] : nbw[u];
        const bool y = (nbw[u] >> 31) != 0;
        const PiT* row = my_ring + (size_t)u * Kp;
        f32x2 x2[NP];
        load_row_pairs<PiT, VPL, FULL>(row, lane, nvec, x2);
        // four independent pair accumulators break the FMA dependency chain
        f32x2 d2[4] = {0ull, 0ull, 0ull, 0ull};
#pragma unroll
        for (int e = 0; e < NP; ++e) d2[e & 3] = fma_f32x2(w2[e], x2[e], d2[e & 3]);
        // refill the lane's pieces of slot u (read above, now in registers)
        // with row t + STAGES
        if (tn < T) copy_row_lane<PiT, VPL, FULL>(my_ring + (size_t)u * Kp, pi + (int64_t)(nxt & 0x7fffffffu) * Kp, lane, nvec);
        cp_async_commit();
        nbw[u] = nxt;
        float D;
        {
          float lo, hi;
          unpack_f32x2(add_f32x2(add_f32x2(d2[0], d2[1]), add_f32x2(d2[2], d2[3])), lo, hi);
          D = lo + hi;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) D += __shfl_xor_sync(0xffffffffu, D, o);
        const float Ds = y ? D : -D;
        const float P = Ds + (y ? e1si : e0si);
        const float invP = rcp_approx(P);
        const float cj = y ? invP : -invP;
        Bsum += ((y ? e1o : e0o) - Ds) * invP;
        const f32x2 c2 = pack_f32x2(cj, cj);
#pragma unroll
        for (int e = 0; e < NP; ++e) A2[e] = fma_f32x2(c2, x2[e], A2[e]);
      }
    }
    // every copy of the node is in (the groups after the last row are
    // empty); the A vectors below reuse the ring
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
      if (k0 < K) {
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
    const float rSnew = 1.0f / Snew;  // the new pi row as phi * (1/S'): within 1 ulp
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      const int k0 = 4 * (tid + NT * g);
      if (k0 < Kp) {
        float4 o;
        o.x = (k0 + 0 < K) ? pn[g][0] * rSnew : 0.f;
        o.y = (k0 + 1 < K) ? pn[g][1] * rSnew : 0.f;
        o.z = (k0 + 2 < K) ? pn[g][2] * rSnew : 0.f;
        o.w = (k0 + 3 < K) ? pn[g][3] * rSnew : 0.f;
        *reinterpret_cast<float4*>(st + k0) = o;
      }
    }
    __syncthreads();  // smem reuse by the next node
  }
}
// The iteration's node count picks the launch that does the work: the
// kernel runs when n_lo < n_nodes <= n_hi and returns at once otherwise.
// Iterations with few nodes (the link stratum: one vertex and its edges)
// take a 16-warp variant, whose warps each hold a quarter of the rows the
// 4-warp one gives them, so a node's rows are in flight together.
// Blocks per SM the register budget is sized for: 16 warps per SM.
template <int SPLIT>
constexpr int ring_min_blocks() { return SPLIT >= 16 ? 1 : 16 / SPLIT; }
template <typename PiT, int VPL, int SPLIT, int STAGES, bool FULL>
__global__ void __launch_bounds__(SPLIT * 32, ring_min_blocks<SPLIT>())
    k_update_phi_ring(Model m, Buffers b, int n_lo, int n_hi) {
  // CTAs with no work wait for the kernel ahead before they exit, so that
  // this launch completes after it
  const int n_nodes = b.st->n_nodes;
  if (n_nodes <= n_lo || n_nodes > n_hi) {
    grid_dependency_wait();
    return;
  }
  update_phi_ring_body<PiT, VPL, SPLIT, STAGES, FULL>(m, b);
}
template <typename PiT, int VPL, int SPLIT, int STAGES, bool FULL>
__global__ void __launch_bounds__(SPLIT * 32, ring_min_blocks<SPLIT>())
    k_update_phi_ring_chains(const ChainArgs* __restrict__ c, int p, int n_lo, int n_hi) {
  const ChainArgs& a = c[blockIdx.y];
  const int n_nodes = a.b[p].st->n_nodes;
  if (n_nodes <= n_lo || n_nodes > n_hi) return;
  update_phi_ring_body<PiT, VPL, SPLIT, STAGES, FULL>(a.m, a.b[p]);
}

}  // namespace ammsb
