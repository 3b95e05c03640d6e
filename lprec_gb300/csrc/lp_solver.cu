// Fused vector kernels of the iterative solvers (lpmethods: cg, cg_exact, em).
//
// The reference's solvers (src/lprec/lpmethods.py:62-128) run every vector
// update and inner product as separate CuPy elementwise ops and float32
// reductions over the whole batch: several full passes over HBM per update
// and a float32 sum.  Here one kernel does an update and the inner product it
// needs in a single pass, accumulating in float64; scalars (step lengths,
// inner products) stay on the device, so an iteration needs no host round trip.
//
// Reductions are deterministic: a fixed grid writes one partial sum per block
// into caller-provided work memory, and one block adds the partials in a fixed
// order.  Nothing here allocates device memory.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/lprec_gb300.h"

int lp_internal_set_err(int code, const char* msg);  // lp_handle.cu

namespace {

constexpr int kThreads = 256;
constexpr int kPartsTotal = 2048;  // partial sums per reduction (all slices together)

// partial sums per slice for S slices
__host__ __device__ inline int parts_per_slice(int S) {
  const int p = (kPartsTotal + S - 1) / S;
  return p < 8 ? 8 : p;
}

// sum of v over the block, valid in thread 0
__device__ double block_sum(double v) {
  __shared__ double ws[kThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) ws[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < kThreads / 32; ++i) s += ws[i];
  return s;
}

// Partial inner products: slice s = blockIdx.y, part blockIdx.x of P parts per slice.
__global__ void __launch_bounds__(kThreads) k_dot_parts(const float* __restrict__ a, const float* __restrict__ b,
                                                       int64_t m, int P, double* __restrict__ part) {
  const int s = blockIdx.y;
  const float* as = a + (size_t)s * m;
  const float* bs = b + (size_t)s * m;
  const int64_t stride = (int64_t)P * kThreads;
  double acc = 0.0;
  const bool vec = ((((uintptr_t)as) | ((uintptr_t)bs)) & 15) == 0;
  if (vec) {
    const int64_t m4 = m / 4;
    const float4* a4 = reinterpret_cast<const float4*>(as);
    const float4* b4 = reinterpret_cast<const float4*>(bs);
    for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < m4; i += stride) {
      const float4 x = __ldg(a4 + i), y = __ldg(b4 + i);
      acc += (double)x.x * y.x + (double)x.y * y.y + (double)x.z * y.z + (double)x.w * y.w;
    }
    for (int64_t i = 4 * m4 + (int64_t)blockIdx.x * kThreads + threadIdx.x; i < m; i += stride)
      acc += (double)__ldg(as + i) * __ldg(bs + i);
  } else {
    for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < m; i += stride)
      acc += (double)__ldg(as + i) * __ldg(bs + i);
  }
  const double v = block_sum(acc);
  if (threadIdx.x == 0) part[(size_t)s * P + blockIdx.x] = v;
}

// out[s] = sum of the P partials of slice s (one block per slice, fixed order)
__global__ void __launch_bounds__(kThreads) k_sum_parts(const double* __restrict__ part, int P,
                                                       double* __restrict__ out) {
  const int s = blockIdx.x;
  double acc = 0.0;
  for (int i = threadIdx.x; i < P; i += kThreads) acc += part[(size_t)s * P + i];
  const double v = block_sum(acc);
  if (threadIdx.x == 0) out[s] = v;
}

// x += alpha p; r -= alpha q; partial sums of r.r; alpha = num / den (rounded to float32)
__global__ void __launch_bounds__(kThreads) k_cg_step(float* __restrict__ x, float* __restrict__ r,
                                                     const float* __restrict__ p, const float* __restrict__ q,
                                                     int64_t n, const double* __restrict__ num,
                                                     const double* __restrict__ den, double* __restrict__ part) {
  const float alpha = (float)(*num / *den);
  const int64_t stride = (int64_t)gridDim.x * kThreads;
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += stride) {
    x[i] = x[i] + alpha * p[i];
    const float ri = r[i] - alpha * q[i];
    r[i] = ri;
    acc += (double)ri * ri;
  }
  const double v = block_sum(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = v;
}

// p = r + beta p; beta = num / den (rounded to float32)
__global__ void __launch_bounds__(kThreads) k_cg_dir(float* __restrict__ p, const float* __restrict__ r, int64_t n,
                                                    const double* __restrict__ num, const double* __restrict__ den) {
  const float beta = (float)(*num / *den);
  const int64_t stride = (int64_t)gridDim.x * kThreads;
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += stride) p[i] = r[i] + beta * p[i];
}

// g = tomo / (g + eps)  (the EM data ratio, in place)
__global__ void __launch_bounds__(kThreads) k_em_ratio(float* __restrict__ g, const float* __restrict__ tomo,
                                                      float eps, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * kThreads;
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += stride) g[i] = tomo[i] / (g[i] + eps);
}

// x *= upd / xi
__global__ void __launch_bounds__(kThreads) k_em_step(float* __restrict__ x, const float* __restrict__ upd,
                                                     const float* __restrict__ xi, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * kThreads;
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += stride) x[i] = x[i] * (upd[i] / xi[i]);
}

int launch_err(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) return LP_OK;
  char buf[256];
  snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
  return lp_internal_set_err(LP_ERR_CUDA, buf);
}

}  // namespace

extern "C" {

int64_t lp_vec_work_doubles(int S) { return S < 1 ? 0 : (int64_t)S * parts_per_slice(S); }

int lp_vec_dot(const float* a, const float* b, int64_t m, int S, double* work, double* out, void* stream) {
  if (!a || !b || !work || !out) return lp_internal_set_err(LP_ERR_ARG, "lp_vec_dot: null pointer");
  if (m < 0 || S < 1 || S > 65535) return lp_internal_set_err(LP_ERR_ARG, "lp_vec_dot: bad sizes");
  cudaStream_t st = (cudaStream_t)stream;
  const int P = parts_per_slice(S);
  k_dot_parts<<<dim3(P, S), kThreads, 0, st>>>(a, b, m, P, work);
  k_sum_parts<<<S, kThreads, 0, st>>>(work, P, out);
  return launch_err("lp_vec_dot");
}

int lp_cg_step(float* x, float* r, const float* p, const float* q, int64_t n, const double* num, const double* den,
               double* work, double* rr, void* stream) {
  if (!x || !r || !p || !q || !num || !den || !work || !rr)
    return lp_internal_set_err(LP_ERR_ARG, "lp_cg_step: null pointer");
  if (n < 0) return lp_internal_set_err(LP_ERR_ARG, "lp_cg_step: bad size");
  cudaStream_t st = (cudaStream_t)stream;
  const int P = parts_per_slice(1);
  k_cg_step<<<P, kThreads, 0, st>>>(x, r, p, q, n, num, den, work);
  k_sum_parts<<<1, kThreads, 0, st>>>(work, P, rr);
  return launch_err("lp_cg_step");
}

int lp_cg_dir(float* p, const float* r, int64_t n, const double* num, const double* den, void* stream) {
  if (!p || !r || !num || !den) return lp_internal_set_err(LP_ERR_ARG, "lp_cg_dir: null pointer");
  if (n < 0) return lp_internal_set_err(LP_ERR_ARG, "lp_cg_dir: bad size");
  k_cg_dir<<<parts_per_slice(1), kThreads, 0, (cudaStream_t)stream>>>(p, r, n, num, den);
  return launch_err("lp_cg_dir");
}

int lp_em_ratio(float* g, const float* tomo, float eps, int64_t n, void* stream) {
  if (!g || !tomo) return lp_internal_set_err(LP_ERR_ARG, "lp_em_ratio: null pointer");
  if (n < 0) return lp_internal_set_err(LP_ERR_ARG, "lp_em_ratio: bad size");
  k_em_ratio<<<parts_per_slice(1), kThreads, 0, (cudaStream_t)stream>>>(g, tomo, eps, n);
  return launch_err("lp_em_ratio");
}

int lp_em_step(float* x, const float* upd, const float* xi, int64_t n, void* stream) {
  if (!x || !upd || !xi) return lp_internal_set_err(LP_ERR_ARG, "lp_em_step: null pointer");
  if (n < 0) return lp_internal_set_err(LP_ERR_ARG, "lp_em_step: bad size");
  k_em_step<<<parts_per_slice(1), kThreads, 0, (cudaStream_t)stream>>>(x, upd, xi, n);
  return launch_err("lp_em_step");
}

}  // extern "C"
