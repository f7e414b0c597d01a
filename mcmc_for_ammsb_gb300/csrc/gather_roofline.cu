// gather_roofline.cu -- the memory system's rate for the access pattern of
// update_phi: whole rows of a large table gathered at random row ids into a
// per-warp shared-memory ring (16-byte cp.async per lane, one commit group
// per row, the same pipeline as k_update_phi_ring) and read back, with no
// arithmetic.  Its GB/s is the ceiling a row-gather kernel of this shape can
// reach; bench.py --gather-roofline runs it.
//
// Usage: gather_roofline [table GiB (default 8)] [CTAs per SM (default 4)]
// Prints one JSON line per row size (1, 2, 4 KiB).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#define CK(x)                                                                   \
  do {                                                                          \
    cudaError_t e_ = (x);                                                       \
    if (e_ != cudaSuccess) {                                                    \
      std::fprintf(stderr, "CUDA %s at line %d\n", cudaGetErrorString(e_), __LINE__); \
      return 1;                                                                 \
    }                                                                           \
  } while (0)

namespace {

constexpr int kWarps = 4;    // per CTA, as k_update_phi_ring
constexpr int kStages = 4;   // ring depth
constexpr int kRowsPerWarp = 128;

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Grid covers exactly nrows_gathered = gridDim.x * kWarps * kRowsPerWarp ids.
template <int RB>
__global__ void __launch_bounds__(kWarps * 32) gather(const uint8_t* __restrict__ table,
                                                      const uint32_t* __restrict__ ids, uint32_t* __restrict__ out) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint32_t s_ids[kWarps * kRowsPerWarp];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint8_t* ring = smem + (size_t)warp * kStages * RB;
  for (int q = threadIdx.x; q < kWarps * kRowsPerWarp; q += kWarps * 32)
    s_ids[q] = ids[(size_t)blockIdx.x * kWarps * kRowsPerWarp + q];
  __syncthreads();
  const uint32_t* my = s_ids + warp * kRowsPerWarp;
  auto copy_row = [&](int slot, uint32_t id) {
    const uint8_t* src = table + (size_t)id * RB;
#pragma unroll
    for (int v = lane; v < RB / 16; v += 32)
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(saddr(ring + slot * RB + v * 16)),
                   "l"(src + v * 16)
                   : "memory");
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
#pragma unroll
  for (int t = 0; t < kStages; ++t) copy_row(t, my[t]);
  uint32_t acc = 0;
  for (int t0 = 0; t0 < kRowsPerWarp; t0 += kStages) {
#pragma unroll
    for (int u = 0; u < kStages; ++u) {
      const int t = t0 + u;
      asm volatile("cp.async.wait_group %0;" ::"n"(kStages - 1) : "memory");
#pragma unroll
      for (int v = lane; v < RB / 16; v += 32) {
        const uint4 x = *reinterpret_cast<const uint4*>(ring + u * RB + v * 16);
        acc ^= x.x ^ x.y ^ x.z ^ x.w;
      }
      if (t + kStages < kRowsPerWarp) {
        copy_row(u, my[t + kStages]);
      } else {
        asm volatile("cp.async.commit_group;" ::: "memory");
      }
    }
  }
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

template <int RB>
int run(const uint8_t* table, size_t table_bytes, int ctas_per_sm, int nsm) {
  const long nrows = (long)(table_bytes / RB);
  const int grid = 2048;
  const long ngather = (long)grid * kWarps * kRowsPerWarp;
  std::vector<uint32_t> ids(ngather);
  std::mt19937_64 rng(12345);
  for (auto& x : ids) x = (uint32_t)(rng() % (uint64_t)nrows);
  uint32_t* d_ids = nullptr;
  uint32_t* d_out = nullptr;
  CK(cudaMalloc(&d_ids, ngather * sizeof(uint32_t)));
  CK(cudaMalloc(&d_out, (size_t)grid * kWarps * 32 * sizeof(uint32_t)));
  CK(cudaMemcpy(d_ids, ids.data(), ngather * sizeof(uint32_t), cudaMemcpyHostToDevice));
  // dynamic shared memory: the rings, padded so that ctas_per_sm CTAs fit
  const size_t need = (size_t)kWarps * kStages * RB;
  const size_t cap = (size_t)228 * 1024 / ctas_per_sm - 1024 - kWarps * kRowsPerWarp * 4 - 256;
  const size_t smem = need > cap ? need : cap;
  CK(cudaFuncSetAttribute(gather<RB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int occ = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gather<RB>, kWarps * 32, smem));
  uint8_t* flush = nullptr;
  const size_t flush_bytes = (size_t)512 << 20;  // larger than L2
  CK(cudaMalloc(&flush, flush_bytes));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 6; ++rep) {
    CK(cudaMemset(flush, rep, flush_bytes));
    CK(cudaEventRecord(e0));
    gather<RB><<<grid, kWarps * 32, smem>>>(table, d_ids, d_out);
    CK(cudaEventRecord(e1));
    CK(cudaEventSynchronize(e1));
    CK(cudaGetLastError());
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    if (rep > 0 && ms < best) best = ms;  // the first launch warms up
  }
  std::printf("{\"row_bytes\": %d, \"rows\": %ld, \"table_gb\": %.2f, \"ctas_per_sm\": %d, \"warps_per_sm\": %d, "
              "\"ms\": %.4f, \"GBps\": %.1f}\n",
              RB, ngather, table_bytes / 1e9, occ, occ * kWarps, best, (double)ngather * RB / (best * 1e-3) / 1e9);
  CK(cudaFree(flush));
  CK(cudaFree(d_ids));
  CK(cudaFree(d_out));
  CK(cudaEventDestroy(e0));
  CK(cudaEventDestroy(e1));
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  const double gib = argc > 1 ? std::atof(argv[1]) : 8.0;
  const int ctas = argc > 2 ? std::atoi(argv[2]) : 4;
  if (!(gib >= 0.5 && gib <= 64.0) || ctas < 1 || ctas > 8) {
    std::fprintf(stderr, "usage: gather_roofline [table GiB in 0.5..64] [CTAs per SM in 1..8]\n");
    return 2;
  }
  int nsm = 0;
  CK(cudaSetDevice(0));
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, 0));
  const size_t table_bytes = (size_t)(gib * (1 << 30)) & ~(size_t)4095;
  uint8_t* table = nullptr;
  CK(cudaMalloc(&table, table_bytes));
  CK(cudaMemset(table, 1, table_bytes));
  if (run<1024>(table, table_bytes, ctas, nsm) || run<2048>(table, table_bytes, ctas, nsm) ||
      run<4096>(table, table_bytes, ctas, nsm))
    return 1;
  CK(cudaFree(table));
  return 0;
}
