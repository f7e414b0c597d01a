// ammsb_device.cuh -- device-side building blocks shared by the sampler
// kernels: state structs, graph membership queries, pi row loads and the
// random draws of ammsb_rng.h specialised for the GPU.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "ammsb_rng.h"

namespace ammsb {

// 1/x by the hardware approximation (rcp.approx.ftz.f32: at most 1 ulp from
// the rounded reciprocal for normal x), one instruction instead of the
// correctly rounded reciprocal's refinement and its slow path.
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Programmatic dependent launch (PTX griddepcontrol, sm_90 and later): a
// kernel launched with the programmatic stream serialization attribute may
// start before the kernel ahead of it in the stream has finished, once every
// CTA of that kernel has called grid_launch_dependents() or exited; it must
// call grid_dependency_wait() before it reads what that kernel writes, and
// the wait returns once that kernel has completed and its writes are
// visible.  Both are no-ops in a kernel launched without the attribute.
// The iteration's kernels keep three rules, under which each early start is
// safe by looking at the kernel's own reads: (1) no CTA triggers before its
// own wait (a CTA that exits without waiting counts as triggered); (2) in
// every launch at least one CTA waits before it exits (every CTA, where the
// launch has no work); (3) before its wait a kernel reads only what kernels
// at least two launches ahead in the stream wrote (or draws joined before
// the launch ahead).  By (1) and (2) a launch completes after the kernel
// ahead of it, and starts only once the kernel two ahead has completed.
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Error bits of DevState::err (returned to the host as AMMSB_E_*).
enum : int32_t {
  kErrMinibatchCap = 1,  // minibatch rejection loop hit its cap
  kErrNeighborCap = 2,   // neighbour rejection loop hit its cap
  kErrCapacity = 4,      // minibatch larger than its buffers
  kErrInitCap = 8        // gamma rejection loop hit its cap
};

// Per-iteration scalars of one minibatch buffer set, resident in device
// memory so that a captured CUDA graph can replay the iteration without host
// involvement.  The sampler keeps a ring of buffer sets: the draws of
// iterations t+2 and t+3 are made while iterations t and t+1 update the
// state.
struct DevState {
  uint32_t step;   // step_count of the iteration these draws belong to
  float eps;       // eps_t of that iteration
  float scale;     // minibatch scale (network.cc:263, 341, 386-390)
  int32_t flag;    // 0 non-link stratum, 1 link stratum, 2 random-edge
  int32_t n_edges;
  int32_t n_nodes;
  int32_t rounds;
  int32_t pad;
};

// Sampler-wide counters shared by all buffer sets.
struct DevCounters {
  uint32_t next_step;        // step_count the next sampling pass draws for
  int32_t err;               // error bits
  unsigned long long evals;  // running sum of n_nodes * n_out (edge evaluations)
  unsigned long long iters;  // running count of updated iterations
};

// Graph in device memory: symmetric CSR with sorted rows, plus an
// open-addressing hash (linear probing, power-of-two capacity, load <= 1/2)
// of the held-out and test pairs.
struct DevGraph {
  int64_t n;
  const int64_t* row_ptr;
  const int32_t* col;
  const unsigned long long* excl;  // keys min<<32|max, empty = ~0ull
  uint32_t excl_mask;
};

// Membership of b in a sorted row held in shared memory.
__device__ __forceinline__ bool row_contains(const int32_t* row, int32_t deg, int32_t b) {
  int32_t lo = 0, hi = deg;
  while (lo < hi) {
    const int32_t mid = (lo + hi) >> 1;
    if (row[mid] < b)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo < deg && row[lo] == b;
}

constexpr unsigned long long kEmptyKey = ~0ull;

__host__ __device__ __forceinline__ unsigned long long pair_key(int32_t a, int32_t b) {
  uint32_t lo = (uint32_t)(a < b ? a : b), hi = (uint32_t)(a < b ? b : a);
  return ((unsigned long long)lo << 32) | hi;
}

__host__ __device__ __forceinline__ uint64_t hash64_full(unsigned long long k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}

__host__ __device__ __forceinline__ uint32_t hash64(unsigned long long k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return (uint32_t)k;
}

__host__ __device__ __forceinline__ uint32_t hash32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// Edge::in(held_out_map) || Edge::in(test_map)
__device__ __forceinline__ bool is_excluded(const DevGraph& g, int32_t a, int32_t b) {
  const unsigned long long key = pair_key(a, b);
  uint32_t slot = hash64(key) & g.excl_mask;
  for (uint32_t probe = 0; probe <= g.excl_mask; ++probe) {
    unsigned long long k = __ldg(g.excl + slot);
    if (k == key) return true;
    if (k == kEmptyKey) return false;
    slot = (slot + 1) & g.excl_mask;
  }
  return false;
}

// Finishes a linear-probing lookup whose first slot `slot` was already
// loaded as `first` (so callers can issue several first loads at once).
__device__ __forceinline__ bool probe_resolve(const unsigned long long* tab,
                                              unsigned long long mask,
                                              unsigned long long key,
                                              unsigned long long slot,
                                              unsigned long long first) {
  if (first == key) return true;
  if (first == kEmptyKey) return false;
  for (unsigned long long probe = 1; probe <= mask; ++probe) {
    slot = (slot + 1) & mask;
    const unsigned long long k = __ldg(tab + slot);
    if (k == key) return true;
    if (k == kEmptyKey) return false;
  }
  return false;
}

// Edge::in(NetworkGraph) by binary search in the sorted row of a.
__device__ __forceinline__ bool has_edge(const DevGraph& g, int32_t a, int32_t b) {
  int64_t lo = __ldg(g.row_ptr + a), hi = __ldg(g.row_ptr + a + 1);
  const int64_t end = hi;
  while (lo < hi) {
    int64_t mid = lo + ((hi - lo) >> 1);
    if (__ldg(g.col + mid) < b)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo < end && __ldg(g.col + lo) == b;
}

// ---- pi storage types -------------------------------------------------------
template <typename T>
struct PiTraits;

template <>
struct PiTraits<float> {
  static constexpr int kPerVec = 4;  // elements per 16-byte vector
  __device__ __forceinline__ static void unpack(const uint4& v, float* out) {
    out[0] = __uint_as_float(v.x);
    out[1] = __uint_as_float(v.y);
    out[2] = __uint_as_float(v.z);
    out[3] = __uint_as_float(v.w);
  }
  __device__ __forceinline__ static uint4 pack(const float* in) {
    return make_uint4(__float_as_uint(in[0]), __float_as_uint(in[1]),
                      __float_as_uint(in[2]), __float_as_uint(in[3]));
  }
};

template <>
struct PiTraits<__nv_bfloat16> {
  static constexpr int kPerVec = 8;
  __device__ __forceinline__ static void unpack(const uint4& v, float* out) {
    out[0] = __uint_as_float(v.x << 16);
    out[1] = __uint_as_float(v.x & 0xffff0000u);
    out[2] = __uint_as_float(v.y << 16);
    out[3] = __uint_as_float(v.y & 0xffff0000u);
    out[4] = __uint_as_float(v.z << 16);
    out[5] = __uint_as_float(v.z & 0xffff0000u);
    out[6] = __uint_as_float(v.w << 16);
    out[7] = __uint_as_float(v.w & 0xffff0000u);
  }
  __device__ __forceinline__ static uint32_t pack2(float lo, float hi) {
    __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&h);
  }
  __device__ __forceinline__ static uint4 pack(const float* in) {
    return make_uint4(pack2(in[0], in[1]), pack2(in[2], in[3]),
                      pack2(in[4], in[5]), pack2(in[6], in[7]));
  }
};

__device__ __forceinline__ uint4 ldg_nc_v4(const void* p) {
  uint4 r;
  asm volatile("ld.global.nc.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "l"(p));
  return r;
}

// ---- random draws -------------------------------------------------------------
// Standard normal #idx of stream (tag, entity, step): Box-Muller on the
// 24-bit uniforms of words 2p, 2p+1 of block idx/4, p = (idx/2)%2; even idx
// takes the cosine branch, odd idx the sine branch.
__device__ __forceinline__ float normal_draw(const Stream& s, uint32_t tag,
                                             uint32_t entity, uint32_t step,
                                             uint64_t idx) {
  U32x4 o = s.block(tag, entity, step, idx >> 2);
  const bool second = (idx >> 1) & 1;
  const uint32_t x0 = second ? o.z : o.x;
  const uint32_t x1 = second ? o.w : o.y;
  const float u1 = u24_open(x0);
  const float u2 = u24(x1);
  const float r = sqrtf(-2.0f * logf(u1));
  float sn, cs;
  sincospif(2.0f * u2, &sn, &cs);
  return r * ((idx & 1) ? sn : cs);
}

// Marsaglia & Tsang (ACM TOMS 26(3), 2000) gamma(shape, scale), double
// precision; attempt a uses block (entity, step = a) at index idx; shape < 1
// through Gamma(a) = Gamma(a + 1) * U^(1/a) with U from step 0xffffffff.
__device__ __forceinline__ double gamma_draw(const Stream& s, uint32_t tag,
                                             uint32_t entity, uint64_t idx,
                                             double shape, double scale,
                                             int32_t* err) {
  double a = shape, boost = 1.0;
  if (a < 1.0) {
    U32x4 o = s.block(tag, entity, 0xffffffffu, idx);
    double u = ((double)o.w + 0.5) * 2.3283064365386963e-10;
    boost = pow(u, 1.0 / a);
    a += 1.0;
  }
  const double d = a - 1.0 / 3.0;
  const double c = 1.0 / sqrt(9.0 * d);
  for (uint32_t attempt = 0; attempt < 64; ++attempt) {
    U32x4 o = s.block(tag, entity, attempt, idx);
    double u1 = ((double)o.x + 0.5) * 2.3283064365386963e-10;
    double u2 = (double)o.y * 2.3283064365386963e-10;
    double x = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
    double v = 1.0 + c * x;
    if (v <= 0.0) continue;
    v = v * v * v;
    double u = ((double)o.z + 0.5) * 2.3283064365386963e-10;
    if (u < 1.0 - 0.0331 * x * x * x * x) return d * v * boost * scale;
    if (log(u) < 0.5 * x * x + d * (1.0 - v + log(v))) return d * v * boost * scale;
  }
  atomicOr(err, kErrInitCap);
  return d * boost * scale;
}

__device__ __forceinline__ float eps_schedule(double a, double b, double c, uint32_t step) {
  return (float)(a * pow(1.0 + (double)step / b, -c));
}

}  // namespace ammsb
