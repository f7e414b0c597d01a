// ammsb_adjoint.cu -- the minibatch edge log-likelihood and its hand-written
// adjoint: the SGRLD drift of phi and theta.
//
// The reference never forms this function; it differentiates it by hand:
//   L(phi, theta) = sum over pairs q = (a, b, y) of log p_q,
//   p_q = sum_k pi_ak pi_bk (f_qk - e_q) + e_q,          pi_a = phi_a / S_a,
//   f_qk = y ? beta_k : 1 - beta_k,  e_q = y ? eps : 1 - eps,
//   beta_k = theta_k1 / (theta_k0 + theta_k1),
// p_q is the normaliser prob_sum of update_beta (mcmc_sampler_stochastic.cc
// :212-240) and, as sum_k pi_ak = 1, of update_phi (cc:279-290).
// cal_edge_likelihood (learner.h:100-139) equals it for a non-link and leaves
// out the term eps * (1 - sum_k pi_ak pi_bk) for a link.
// Its gradients are the reference's hand-derived terms:
//   dL/dphi_ak = sum_q (probs_qk / (p_q phi_ak) - 1/S_a)  -- update_phi
//                (mcmc_sampler_stochastic.cc:274-296, pi_b held fixed)
//   dL/dtheta  = the update_beta gradient (cc:212-240).
// With sigma_q = +-1 for y = 1/0, f - e = sigma (beta - eps), so
//   p_q = sigma_q D_q + e_q,  D_q = sum_k w_ak pi_bk,  w_ak = pi_ak (beta_k - eps),
//   dL/dphi_ak  = ((beta_k - eps) A_ak - B_a) / S_a,
//       A_ak = sum_{q of a} sigma_q pi_bk / p_q,  B_a = sum_{q of a} (p_q - e_q) / p_q,
//   dL/dbeta_k  = sum_a pi_ak A_ak,
//   dL/dpi_bk   = (beta_k - eps) sum_{q of b} sigma_q pi_ak / p_q,
// and beta's chain rule: dbeta/dtheta_k0 = -beta_k / T_k,
// dbeta/dtheta_k1 = (1 - beta_k) / T_k, T_k = theta_k0 + theta_k1.
//
// The forward keeps one scalar per pair (p_q) and per source (S_a); the
// backward recomputes every per-pair K-vector from the rows.  All sums are in
// a fixed order (one warp per source row for dphi and the theta partials, one
// warp per neighbour row for dpi, one thread per k for dtheta), so repeated
// calls give identical bits.  One warp owns a row: lane l holds elements
// l, l + 32, ..., so K <= 32 * VPL with VPL in {1, 2, 4, 8, 16, 32}.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/ammsb_gpu.h"

namespace {

constexpr int kWarpsPerBlock = 8;
constexpr int kErrIndex = 1;   // a pair or CSR index out of range
constexpr int kErrNonPos = 2;  // a row sum S_a or a probability p_q <= 0

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// workspace: [err word | S (n_src) | ll (n_src) | p (n_pairs) | t (n_src x K)]
struct Workspace {
  int32_t* err;
  size_t off_S, off_ll, off_p, off_t, bytes;
};

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

Workspace layout(size_t es, int64_t K, int64_t n_src, int64_t n_pairs) {
  Workspace w{};
  w.off_S = 256;
  w.off_ll = w.off_S + align256(es * (size_t)n_src);
  w.off_p = w.off_ll + align256(es * (size_t)n_src);
  w.off_t = w.off_p + align256(es * (size_t)n_pairs);
  w.bytes = w.off_t + align256(es * (size_t)n_src * (size_t)K);
  return w;
}

struct Args {
  int32_t K;
  const void* phi;   // n_src x ld_phi
  int64_t ld_phi;
  const void* pin;   // n_nbr x ld_pi
  int64_t ld_pi;
  int64_t n_nbr;
  const void* theta; // K x 2
  double eps;
  const int64_t* src_ptr;  // n_src + 1: pairs of source a are [src_ptr[a], src_ptr[a+1])
  int64_t n_src;
  const int32_t* pair_nbr; // n_pairs: row of pin
  const uint8_t* pair_y;
  int64_t n_pairs;
  // backward only
  const int32_t* pair_src; // n_pairs: source row of each pair
  const int64_t* nbr_ptr;  // n_nbr + 1 over nbr_pairs
  const int32_t* nbr_pairs;
  const void* gout;        // device scalar dL
  void* gphi;              // n_src x ld_phi
  void* gpin;              // n_nbr x ld_pi (or null)
  void* gtheta;            // K x 2
  char* ws;
  Workspace w;
};

template <typename T>
__device__ __forceinline__ T beta_of(const T* theta, int k) {
  const T t0 = theta[2 * k], t1 = theta[2 * k + 1];
  return t1 / (t0 + t1);
}

template <typename T, int VPL>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_ll_forward(Args g) {
  const int lane = threadIdx.x & 31;
  const int64_t a = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  if (a >= g.n_src) return;
  const T* phi = static_cast<const T*>(g.phi) + a * g.ld_phi;
  const T* pin = static_cast<const T*>(g.pin);
  const T* theta = static_cast<const T*>(g.theta);
  const T eps = (T)g.eps;
  T* S_out = reinterpret_cast<T*>(g.ws + g.w.off_S);
  T* ll_out = reinterpret_cast<T*>(g.ws + g.w.off_ll);
  T* p_out = reinterpret_cast<T*>(g.ws + g.w.off_p);
  int32_t* err = g.w.err;

  T x[VPL], w[VPL];
  T S = 0;
#pragma unroll
  for (int v = 0; v < VPL; ++v) {
    const int k = lane + 32 * v;
    x[v] = (k < g.K) ? phi[k] : T(0);
    S += x[v];
  }
  S = warp_sum(S);
  if (!(S > T(0)) && lane == 0) atomicOr(err, kErrNonPos);
#pragma unroll
  for (int v = 0; v < VPL; ++v) {
    const int k = lane + 32 * v;
    w[v] = (k < g.K) ? x[v] / S * (beta_of(theta, k) - eps) : T(0);
  }
  const int64_t q0 = g.src_ptr[a], q1 = g.src_ptr[a + 1];
  T ll = 0;
  if (q0 < 0 || q1 < q0 || q1 > g.n_pairs) {
    if (lane == 0) atomicOr(err, kErrIndex);
  } else {
    for (int64_t q = q0; q < q1; ++q) {
      const int32_t b = g.pair_nbr[q];
      if (b < 0 || b >= g.n_nbr) {
        if (lane == 0) { atomicOr(err, kErrIndex); p_out[q] = T(1); }
        continue;
      }
      const T* row = pin + (int64_t)b * g.ld_pi;
      T D = 0;
#pragma unroll
      for (int v = 0; v < VPL; ++v) {
        const int k = lane + 32 * v;
        if (k < g.K) D += w[v] * row[k];
      }
      D = warp_sum(D);
      const bool y = g.pair_y[q] != 0;
      const T p = (y ? D : -D) + (y ? eps : T(1) - eps);
      if (lane == 0) {
        p_out[q] = p;
        if (!(p > T(0))) atomicOr(err, kErrNonPos);
      }
      ll += log(p);
    }
  }
  if (lane == 0) {
    S_out[a] = S;
    ll_out[a] = ll;
  }
}

// loss = sum_a ll[a], one block, fixed order
template <typename T>
__global__ void __launch_bounds__(256) k_ll_sum(Args g, T* loss) {
  __shared__ T part[256];
  const T* ll = reinterpret_cast<const T*>(g.ws + g.w.off_ll);
  T s = 0;
  for (int64_t a = threadIdx.x; a < g.n_src; a += 256) s += ll[a];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h) part[threadIdx.x] += part[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = part[0];
}

// dL/dphi rows and the per-source theta partials t[a][k] = pi_ak A_ak
template <typename T, int VPL>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_ll_backward_src(Args g) {
  const int lane = threadIdx.x & 31;
  const int64_t a = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  if (a >= g.n_src) return;
  const T* phi = static_cast<const T*>(g.phi) + a * g.ld_phi;
  const T* pin = static_cast<const T*>(g.pin);
  const T* theta = static_cast<const T*>(g.theta);
  const T eps = (T)g.eps;
  const T gout = *static_cast<const T*>(g.gout);
  const T* p_in = reinterpret_cast<const T*>(g.ws + g.w.off_p);
  const T S = reinterpret_cast<const T*>(g.ws + g.w.off_S)[a];
  T* t_out = reinterpret_cast<T*>(g.ws + g.w.off_t) + a * g.K;

  T A[VPL];
#pragma unroll
  for (int v = 0; v < VPL; ++v) A[v] = T(0);
  T B = 0;
  const int64_t q0 = g.src_ptr[a], q1 = g.src_ptr[a + 1];
  if (q0 >= 0 && q1 >= q0 && q1 <= g.n_pairs) {
    for (int64_t q = q0; q < q1; ++q) {
      const int32_t b = g.pair_nbr[q];
      if (b < 0 || b >= g.n_nbr) continue;  // flagged by the forward
      const bool y = g.pair_y[q] != 0;
      const T p = p_in[q];
      const T c = (y ? T(1) : T(-1)) / p;
      B += (p - (y ? eps : T(1) - eps)) / p;
      const T* row = pin + (int64_t)b * g.ld_pi;
#pragma unroll
      for (int v = 0; v < VPL; ++v) {
        const int k = lane + 32 * v;
        if (k < g.K) A[v] += c * row[k];
      }
    }
  }
  T* gphi = static_cast<T*>(g.gphi) + a * g.ld_phi;
#pragma unroll
  for (int v = 0; v < VPL; ++v) {
    const int k = lane + 32 * v;
    if (k < g.K) {
      const T bk = beta_of(theta, k);
      gphi[k] = gout * ((bk - eps) * A[v] - B) / S;
      t_out[k] = phi[k] / S * A[v];
    }
  }
}

// dL/dtheta: thread per k, sources summed in order
template <typename T>
__global__ void __launch_bounds__(256) k_ll_backward_theta(Args g) {
  const int k = blockIdx.x * 256 + threadIdx.x;
  if (k >= g.K) return;
  const T* t = reinterpret_cast<const T*>(g.ws + g.w.off_t);
  const T* theta = static_cast<const T*>(g.theta);
  const T gout = *static_cast<const T*>(g.gout);
  T U = 0;
  for (int64_t a = 0; a < g.n_src; ++a) U += t[a * g.K + k];
  const T t0 = theta[2 * k], t1 = theta[2 * k + 1];
  const T Tk = t0 + t1;
  const T bk = t1 / Tk;
  T* gt = static_cast<T*>(g.gtheta);
  gt[2 * k] = gout * U * (-bk / Tk);
  gt[2 * k + 1] = gout * U * ((T(1) - bk) / Tk);
}

// dL/dpi_nbr rows: warp per neighbour row over its pairs (nbr CSR)
template <typename T, int VPL>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_ll_backward_nbr(Args g) {
  const int lane = threadIdx.x & 31;
  const int64_t b = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  if (b >= g.n_nbr) return;
  const T* phi = static_cast<const T*>(g.phi);
  const T* theta = static_cast<const T*>(g.theta);
  const T eps = (T)g.eps;
  const T gout = *static_cast<const T*>(g.gout);
  const T* p_in = reinterpret_cast<const T*>(g.ws + g.w.off_p);
  const T* S_in = reinterpret_cast<const T*>(g.ws + g.w.off_S);

  T acc[VPL];
#pragma unroll
  for (int v = 0; v < VPL; ++v) acc[v] = T(0);
  const int64_t r0 = g.nbr_ptr[b], r1 = g.nbr_ptr[b + 1];
  if (r0 < 0 || r1 < r0 || r1 > g.n_pairs) {
    if (lane == 0) atomicOr(g.w.err, kErrIndex);
  } else {
    for (int64_t r = r0; r < r1; ++r) {
      const int32_t q = g.nbr_pairs[r];
      if (q < 0 || q >= g.n_pairs) {
        if (lane == 0) atomicOr(g.w.err, kErrIndex);
        continue;
      }
      const int32_t a = g.pair_src[q];
      if (a < 0 || a >= g.n_src || g.pair_nbr[q] != b) {
        if (lane == 0) atomicOr(g.w.err, kErrIndex);
        continue;
      }
      const bool y = g.pair_y[q] != 0;
      const T c = (y ? T(1) : T(-1)) / (p_in[q] * S_in[a]);
      const T* row = phi + (int64_t)a * g.ld_phi;
#pragma unroll
      for (int v = 0; v < VPL; ++v) {
        const int k = lane + 32 * v;
        if (k < g.K) acc[v] += c * row[k];
      }
    }
  }
  T* gp = static_cast<T*>(g.gpin) + b * g.ld_pi;
#pragma unroll
  for (int v = 0; v < VPL; ++v) {
    const int k = lane + 32 * v;
    if (k < g.K) gp[k] = gout * (beta_of(theta, k) - eps) * acc[v];
  }
}

int vpl_of(int64_t K) {
  int v = 1;
  while (32 * v < K) v <<= 1;
  return v;
}

template <typename T, int VPL>
cudaError_t launch_forward(const Args& g, cudaStream_t s) {
  const unsigned grid = (unsigned)((g.n_src + kWarpsPerBlock - 1) / kWarpsPerBlock);
  if (grid) k_ll_forward<T, VPL><<<grid, kWarpsPerBlock * 32, 0, s>>>(g);
  return cudaGetLastError();
}

template <typename T, int VPL>
cudaError_t launch_backward(const Args& g, cudaStream_t s) {
  const unsigned grid = (unsigned)((g.n_src + kWarpsPerBlock - 1) / kWarpsPerBlock);
  if (grid) k_ll_backward_src<T, VPL><<<grid, kWarpsPerBlock * 32, 0, s>>>(g);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_ll_backward_theta<T><<<(g.K + 255) / 256, 256, 0, s>>>(g);
  e = cudaGetLastError();
  if (e != cudaSuccess || !g.gpin) return e;
  const unsigned gridn = (unsigned)((g.n_nbr + kWarpsPerBlock - 1) / kWarpsPerBlock);
  if (gridn) k_ll_backward_nbr<T, VPL><<<gridn, kWarpsPerBlock * 32, 0, s>>>(g);
  return cudaGetLastError();
}

template <typename T>
cudaError_t dispatch(bool fwd, int vpl, const Args& g, cudaStream_t s) {
#define CASE(V)                                                                  \
  if (vpl == V) return fwd ? launch_forward<T, V>(g, s) : launch_backward<T, V>(g, s);
  CASE(1) CASE(2) CASE(4) CASE(8) CASE(16) CASE(32)
#undef CASE
  return cudaErrorInvalidConfiguration;
}

int fail(const char* fn, const std::string& msg, int code) {
  std::fprintf(stderr, "%s: %s\n", fn, msg.c_str());
  return code;
}

int check_common(const char* fn, int32_t dtype, int64_t K, const void* phi, int64_t ld_phi,
                 const void* pin, int64_t ld_pi, int64_t n_nbr, const void* theta,
                 const int64_t* src_ptr, int64_t n_src, const int32_t* pair_nbr,
                 const uint8_t* pair_y, int64_t n_pairs, const void* ws) {
  if (dtype != AMMSB_REAL_F32 && dtype != AMMSB_REAL_F64)
    return fail(fn, "dtype must be AMMSB_REAL_F32 or AMMSB_REAL_F64", AMMSB_E_ARG);
  if (K < 1 || K > 1024) return fail(fn, "need 1 <= K <= 1024", AMMSB_E_ARG);
  if (ld_phi < K || ld_pi < K) return fail(fn, "row strides must be >= K", AMMSB_E_ARG);
  if (n_src < 0 || n_nbr < 0 || n_pairs < 0 || n_pairs > INT32_MAX)
    return fail(fn, "negative size, or more than 2^31 - 1 pairs", AMMSB_E_ARG);
  if (!theta || !src_ptr || !ws || (n_src > 0 && !phi) || (n_nbr > 0 && !pin) ||
      (n_pairs > 0 && (!pair_nbr || !pair_y)))
    return fail(fn, "null argument", AMMSB_E_ARG);
  return AMMSB_OK;
}

}  // namespace

extern "C" {

size_t ammsb_edge_loglik_workspace_size(int32_t dtype, int64_t K, int64_t n_src,
                                        int64_t n_pairs) {
  if (K < 1 || n_src < 0 || n_pairs < 0) return 0;
  const size_t es = (dtype == AMMSB_REAL_F64) ? 8 : 4;
  return layout(es, K, n_src, n_pairs).bytes;
}

int ammsb_edge_loglik_forward(int32_t dtype, int64_t K, const void* phi_src, int64_t ld_phi,
                              const void* pi_nbr, int64_t ld_pi, int64_t n_nbr,
                              const void* theta, double epsilon, const int64_t* src_ptr,
                              int64_t n_src, const int32_t* pair_nbr, const uint8_t* pair_y,
                              int64_t n_pairs, void* loss, void* workspace, void* stream) {
  const char* fn = "ammsb_edge_loglik_forward";
  int rc = check_common(fn, dtype, K, phi_src, ld_phi, pi_nbr, ld_pi, n_nbr, theta, src_ptr,
                        n_src, pair_nbr, pair_y, n_pairs, workspace);
  if (rc) return rc;
  if (!loss) return fail(fn, "null loss", AMMSB_E_ARG);
  const size_t es = (dtype == AMMSB_REAL_F64) ? 8 : 4;
  Args g{};
  g.K = (int32_t)K;
  g.phi = phi_src; g.ld_phi = ld_phi;
  g.pin = pi_nbr; g.ld_pi = ld_pi; g.n_nbr = n_nbr;
  g.theta = theta; g.eps = epsilon;
  g.src_ptr = src_ptr; g.n_src = n_src;
  g.pair_nbr = pair_nbr; g.pair_y = pair_y; g.n_pairs = n_pairs;
  g.ws = static_cast<char*>(workspace);
  g.w = layout(es, K, n_src, n_pairs);
  g.w.err = reinterpret_cast<int32_t*>(g.ws);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(g.w.err, 0, sizeof(int32_t), s);
  if (e == cudaSuccess)
    e = (dtype == AMMSB_REAL_F64) ? dispatch<double>(true, vpl_of(K), g, s)
                                  : dispatch<float>(true, vpl_of(K), g, s);
  if (e == cudaSuccess) {
    if (dtype == AMMSB_REAL_F64) k_ll_sum<double><<<1, 256, 0, s>>>(g, static_cast<double*>(loss));
    else k_ll_sum<float><<<1, 256, 0, s>>>(g, static_cast<float*>(loss));
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return fail(fn, cudaGetErrorString(e), AMMSB_E_CUDA);
  return AMMSB_OK;
}

int ammsb_edge_loglik_backward(int32_t dtype, int64_t K, const void* phi_src, int64_t ld_phi,
                               const void* pi_nbr, int64_t ld_pi, int64_t n_nbr,
                               const void* theta, double epsilon, const int64_t* src_ptr,
                               int64_t n_src, const int32_t* pair_nbr, const uint8_t* pair_y,
                               int64_t n_pairs, const int32_t* pair_src, const int64_t* nbr_ptr,
                               const int32_t* nbr_pairs, const void* grad_loss,
                               void* grad_phi_src, void* grad_pi_nbr, void* grad_theta,
                               void* workspace, void* stream) {
  const char* fn = "ammsb_edge_loglik_backward";
  int rc = check_common(fn, dtype, K, phi_src, ld_phi, pi_nbr, ld_pi, n_nbr, theta, src_ptr,
                        n_src, pair_nbr, pair_y, n_pairs, workspace);
  if (rc) return rc;
  if (!grad_loss || !grad_theta || (n_src > 0 && !grad_phi_src))
    return fail(fn, "null gradient argument", AMMSB_E_ARG);
  if (grad_pi_nbr && (!nbr_ptr || (n_pairs > 0 && (!pair_src || !nbr_pairs))))
    return fail(fn, "grad_pi_nbr needs pair_src, nbr_ptr and nbr_pairs", AMMSB_E_ARG);
  const size_t es = (dtype == AMMSB_REAL_F64) ? 8 : 4;
  Args g{};
  g.K = (int32_t)K;
  g.phi = phi_src; g.ld_phi = ld_phi;
  g.pin = pi_nbr; g.ld_pi = ld_pi; g.n_nbr = n_nbr;
  g.theta = theta; g.eps = epsilon;
  g.src_ptr = src_ptr; g.n_src = n_src;
  g.pair_nbr = pair_nbr; g.pair_y = pair_y; g.n_pairs = n_pairs;
  g.pair_src = pair_src; g.nbr_ptr = nbr_ptr; g.nbr_pairs = nbr_pairs;
  g.gout = grad_loss; g.gphi = grad_phi_src; g.gpin = grad_pi_nbr; g.gtheta = grad_theta;
  g.ws = static_cast<char*>(workspace);
  g.w = layout(es, K, n_src, n_pairs);
  g.w.err = reinterpret_cast<int32_t*>(g.ws);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = (dtype == AMMSB_REAL_F64) ? dispatch<double>(false, vpl_of(K), g, s)
                                            : dispatch<float>(false, vpl_of(K), g, s);
  if (e != cudaSuccess) return fail(fn, cudaGetErrorString(e), AMMSB_E_CUDA);
  return AMMSB_OK;
}

int ammsb_edge_loglik_status(const void* workspace, void* stream, int32_t* flags) {
  if (!workspace || !flags) return AMMSB_E_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemcpyAsync(flags, workspace, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail("ammsb_edge_loglik_status", cudaGetErrorString(e), AMMSB_E_CUDA);
  return AMMSB_OK;
}

}  // extern "C"
