// ammsb_noalloc.cu -- held-out perplexity for callers that must not
// allocate GPU memory.
//
// Some host programs cannot call cudaMalloc at all: a process embedding the
// sampler in a runtime that owns every device allocation (a memory pool or
// arena handed out by a framework, a sandbox that forbids driver
// allocations, a real-time loop that must not allocate after start-up).
// They hold pi, beta and the held-out arrays in memory they obtained their
// own way and need the perplexity of that state.  ammsb_perplexity_noalloc
// computes it with the same kernels as ammsb_perplexity, keeping the
// kernels' scratch (per-block compensated partial sums, the result and an
// index-error flag) in a fixed file-scope __device__ array instead of
// handle-owned memory.
//
// The array has room for kMaxBlocks partials and the kernel runs one block
// per 256 held-out edges, so one call accepts at most kMaxBlocks * 256 =
// 4,194,304 held-out edges and rejects more with AMMSB_E_CAPACITY (the
// message goes to stderr, as do those of the other rejected arguments).
// The array lives in every GPU that loads the library, until the process
// exits.  All calls on a device share it and it keeps the last call's
// contents: every call writes the partials it reads and clears the flag
// before its kernels run, but calls whose kernels overlap on the GPU race
// on it.  The first call on a device looks up the array's device address
// (cudaGetSymbolAddress) with that device current.  Every call ends by
// copying the result into pageable host memory and synchronising its
// stream, so it cannot be called on a stream that is being captured.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/ammsb_gpu.h"
#include "ammsb_kernels.cuh"

using namespace ammsb;

namespace {

constexpr int kMaxBlocks = 16384;
constexpr int kEdgesPerBlock = 256;
constexpr int kMaxDevices = 64;

// partial (sum, compensation) per block, then the result (2 doubles), then
// the index-error flag (one double's room)
static __device__ __align__(256) double g_ppx_scratch[2 * kMaxBlocks + 3];
constexpr int kResult = 2 * kMaxBlocks;
constexpr int kFlag = 2 * kMaxBlocks + 2;

std::mutex g_mu;
double* g_scratch_ptr[kMaxDevices] = {nullptr};

int next_pow2i(int v) {
  int p = 1;
  while (p < v) p <<= 1;
  return p;
}

template <typename PiT, int LPN, int VPL>
cudaError_t launch(const Model& m, const void* pi, const float* beta, const int32_t* ha,
                   const int32_t* hb, const uint8_t* hy, int64_t H, float* ppx, float count,
                   double* scratch, int nblk, int64_t n_rows, cudaStream_t s) {
  k_perplexity<PiT, LPN, VPL><<<nblk, 256, 0, s>>>(
      m, reinterpret_cast<const PiT*>(pi), beta, ha, hb, hy, H, ppx, count, scratch, n_rows,
      reinterpret_cast<unsigned int*>(scratch + kFlag));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_ppx_final<<<1, kPpxFinalThreads, 0, s>>>(scratch, nblk, H, scratch + kResult);
  return cudaGetLastError();
}

template <typename PiT>
cudaError_t dispatch(int lpn, int vpl, const Model& m, const void* pi, const float* beta,
                     const int32_t* ha, const int32_t* hb, const uint8_t* hy, int64_t H, float* ppx,
                     float count, double* scratch, int nblk, int64_t n_rows, cudaStream_t s) {
#define CASE(L, V) \
  if (lpn == L && vpl == V)  \
    return launch<PiT, L, V>(m, pi, beta, ha, hb, hy, H, ppx, count, scratch, nblk, n_rows, s);
  CASE(1, 1) CASE(2, 1) CASE(4, 1) CASE(8, 1) CASE(16, 1) CASE(32, 1) CASE(32, 2) CASE(32, 4) CASE(32, 8)
#undef CASE
  return cudaErrorInvalidConfiguration;
}

}  // namespace

extern "C" {

int ammsb_perplexity_noalloc(const void* pi, int32_t pi_dtype, int64_t K, int64_t row_stride,
                             int64_t n_rows, const float* beta, double epsilon, const int32_t* held_a,
                             const int32_t* held_b, const uint8_t* held_y, int64_t held_count,
                             float* ppx, uint64_t average_count, void* stream, double* out) {
  auto fail = [](const std::string& msg, int code) {
    std::fprintf(stderr, "ammsb_perplexity_noalloc: %s\n", msg.c_str());
    return code;
  };
  if (!out || (held_count > 0 && (!pi || !beta || !held_a || !held_b || !held_y || !ppx)))
    return fail("null argument", AMMSB_E_ARG);
  if (pi_dtype != AMMSB_PI_F32 && pi_dtype != AMMSB_PI_BF16)
    return fail("pi_dtype must be AMMSB_PI_F32 or AMMSB_PI_BF16", AMMSB_E_ARG);
  const int ev = (pi_dtype == AMMSB_PI_BF16) ? 8 : 4;
  const int64_t es = (pi_dtype == AMMSB_PI_BF16) ? 2 : 4;
  if (K < 1 || K > 1024 || row_stride < K || (row_stride * es) % 16 != 0)
    return fail("need 1 <= K <= 1024 and a row stride >= K that is a multiple of 16 bytes",
                AMMSB_E_ARG);
  if ((reinterpret_cast<uintptr_t>(pi) & 15) != 0)
    return fail("pi must be 16-byte aligned", AMMSB_E_ARG);
  if (n_rows < 1 || n_rows > (int64_t)INT32_MAX + 1)
    return fail("n_rows must be in [1, 2^31]", AMMSB_E_ARG);
  if (held_count < 0 || held_count > (int64_t)kMaxBlocks * kEdgesPerBlock)
    return fail("held_count exceeds the static scratch: at most 4,194,304 held-out edges",
                AMMSB_E_CAPACITY);
  if (average_count < 1) return fail("average_count starts at 1", AMMSB_E_ARG);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail("no current CUDA device", AMMSB_E_CUDA);
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {  // once per device, with that device current
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_ppx_scratch);
      if (e != cudaSuccess)
        return fail(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e), AMMSB_E_CUDA);
      g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    scratch = g_scratch_ptr[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (held_count == 0) {
    *out = 0.0;
    return AMMSB_OK;
  }
  Model m{};
  m.K = (int32_t)K;
  m.Kp = (int32_t)row_stride;  // addressing only: the kernel reads the K values of a row
  m.epsilon = (float)epsilon;
  const int nvec = (int)((K + ev - 1) / ev);
  int lpn, vpl;
  if (nvec <= 32) {
    lpn = next_pow2i(nvec);
    vpl = 1;
  } else {
    lpn = 32;
    vpl = next_pow2i((nvec + 31) / 32);
  }
  if (vpl > 8) return fail("row too wide", AMMSB_E_ARG);  // K <= 1024 keeps vpl <= 8
  const int nblk = (int)((held_count + kEdgesPerBlock - 1) / kEdgesPerBlock);
  const float count = (float)average_count;
  cudaError_t e = cudaMemsetAsync(scratch + kFlag, 0, sizeof(double), s);
  if (e != cudaSuccess) return fail(std::string("flag clear: ") + cudaGetErrorString(e), AMMSB_E_CUDA);
  e = (pi_dtype == AMMSB_PI_BF16)
          ? dispatch<__nv_bfloat16>(lpn, vpl, m, pi, beta, held_a, held_b, held_y, held_count, ppx,
                                    count, scratch, nblk, n_rows, s)
          : dispatch<float>(lpn, vpl, m, pi, beta, held_a, held_b, held_y, held_count, ppx, count,
                            scratch, nblk, n_rows, s);
  if (e != cudaSuccess) return fail(std::string("launch: ") + cudaGetErrorString(e), AMMSB_E_CUDA);
  double res[3];  // result (2 doubles: value, compensation) and the flag
  e = cudaMemcpyAsync(res, scratch + kResult, sizeof(res), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(std::string("result copy: ") + cudaGetErrorString(e), AMMSB_E_CUDA);
  unsigned int flag = 0;
  std::memcpy(&flag, &res[2], sizeof(flag));
  if (flag != 0)
    return fail("a held-out pair names a row outside [0, n_rows): those pairs were skipped",
                AMMSB_E_ARG);
  *out = res[0];
  return AMMSB_OK;
}

}  // extern "C"
