// ammsb_rng.h -- counter-based random streams of the sampler, host + device.
//
// The reference draws every random number from one sequential xorshift128+
// generator per thread (random.cc:136-176), so its draws depend on the order
// in which nodes and hash-set entries are visited.  A GPU sampler needs draws
// that any thread can compute independently; this header defines them as
// Philox4x32-10 blocks (Salmon et al., SC'11) addressed by
//   counter = {block index, entity, step, tag | (block index >> 32) << 8}
//   key     = {seed, chain}
// and the derived draws used by the hot path:
//   * draw_u64(t): 64 bits from half t%2 of block t/2; uniform integers in
//     [0, range) are uniform_below(draw, range) = floor(draw * range / 2^64)
//     (the reference's randint() reduces rand() % range, random.cc:174-176);
//   * normal(idx): Box-Muller on 24-bit uniforms, 4 normals per block.
// The same code compiles for the host (graph generator, theta init) and the
// device (sampling kernels), so integer draws agree bit for bit.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define AMMSB_HD __host__ __device__ __forceinline__
#else
#define AMMSB_HD inline
#endif
#ifdef __CUDA_ARCH__
#define AMMSB_UNROLL _Pragma("unroll")
#else
#define AMMSB_UNROLL
#endif

namespace ammsb {

enum StreamTag : uint32_t {
  kTagMbFlag = 1,      // stratum choice, network.cc:414
  kTagMbNode = 2,      // source node of a stratum, network.cc:278/364
  kTagMbCand = 3,      // non-link partner candidates, network.cc:297
  kTagNbr = 4,         // neighbour candidates, mcmc_sampler_stochastic.h:101
  kTagPhiNoise = 5,    // update_phi noise, cc:299
  kTagThetaNoise = 6,  // update_beta noise, cc:245
  kTagPhiInit = 7,     // phi ~ Gamma(1,1), cc:66
  kTagThetaInit = 8,   // theta ~ Gamma(eta0, eta1), cc:54
  kTagGraph = 9,       // synthetic graph generator
  kTagHeldOut = 10     // held-out / test construction
};

struct U32x4 {
  uint32_t x, y, z, w;
};

AMMSB_HD uint32_t mulhi32(uint32_t a, uint32_t b, uint32_t* lo) {
#if defined(__CUDA_ARCH__)
  *lo = a * b;
  return __umulhi(a, b);
#else
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *lo = (uint32_t)p;
  return (uint32_t)(p >> 32);
#endif
}

AMMSB_HD U32x4 philox4x32_10(U32x4 c, uint32_t k0, uint32_t k1) {
  AMMSB_UNROLL
  for (int r = 0; r < 10; ++r) {
    uint32_t lo0, lo1;
    uint32_t hi0 = mulhi32(0xD2511F53u, c.x, &lo0);
    uint32_t hi1 = mulhi32(0xCD9E8D57u, c.z, &lo1);
    U32x4 n;
    n.x = hi1 ^ c.y ^ k0;
    n.y = lo1;
    n.z = hi0 ^ c.w ^ k1;
    n.w = lo0;
    c = n;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

struct Stream {
  uint32_t seed, chain;
  AMMSB_HD U32x4 block(uint32_t tag, uint32_t entity, uint32_t step,
                       uint64_t blk) const {
    U32x4 c;
    c.x = (uint32_t)blk;
    c.y = entity;
    c.z = step;
    c.w = (tag & 0xffu) | ((uint32_t)(blk >> 32) << 8);
    return philox4x32_10(c, seed, chain);
  }
  AMMSB_HD uint64_t draw_u64(uint32_t tag, uint32_t entity, uint32_t step,
                             uint64_t t) const {
    U32x4 o = block(tag, entity, step, t >> 1);
    return (t & 1) ? ((uint64_t)o.z | ((uint64_t)o.w << 32))
                   : ((uint64_t)o.x | ((uint64_t)o.y << 32));
  }
};

// Uniform integer in [0, n): floor(x * n / 2^64), the multiply-high map of a
// 64-bit draw (bias at most n / 2^64).  A 64-bit remainder would run through
// the slow FP64 path of the GPU.
AMMSB_HD uint64_t uniform_below(uint64_t x, uint64_t n) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(x, n);
#else
  return (uint64_t)(((unsigned __int128)x * (unsigned __int128)n) >> 64);
#endif
}

// 24-bit uniforms are exact in float everywhere.
AMMSB_HD float u24_open(uint32_t x) {  // (0, 1)
  return ((float)(x >> 8) + 0.5f) * 5.9604644775390625e-08f;
}
AMMSB_HD float u24(uint32_t x) {  // [0, 1)
  return (float)(x >> 8) * 5.9604644775390625e-08f;
}

}  // namespace ammsb
