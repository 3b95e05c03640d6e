// Fused vector kernels of the iterative solvers (lpmethods: cg, cg_exact, em,
// and the total-variation family tv, tve, tvl1).
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

// ---- total-variation family (tv, tve, tvl1: lpmethods.py:131-288) -------------
// Each kernel does one group of the reference's CuPy statements in one pass, in
// the statements' float32 operation order with rounded intrinsics (no fused
// multiply-adds), so a result equals the elementwise sequence's bit for bit.

// Rows of S*ny rows of nx: blocks stride over rows, threads over x.
constexpr int kRowBlocks = 152 * 8;

// prox0x[:, :, :-1] += c*(recon[:, :, 1:] - recon[:, :, :-1])
// prox0y[:, :-1, :] += c*(recon[:, 1:, :] - recon[:, :-1, :])
// nprox = maximum(1, sqrt(prox0x*prox0x + prox0y*prox0y)/lam); prox0x /= nprox; prox0y /= nprox
// One element: a, b the old prox0x/prox0y, ri recon here, rx/ry its x/y neighbours
// (used when hx/hy).
__device__ __forceinline__ void tv_prox0_elem(float& a, float& b, float ri, float rx, float ry, bool hx, bool hy,
                                              float c, float lam) {
  if (hx) a = __fadd_rn(a, __fmul_rn(c, __fsub_rn(rx, ri)));
  if (hy) b = __fadd_rn(b, __fmul_rn(c, __fsub_rn(ry, ri)));
  float n = __fdiv_rn(__fsqrt_rn(__fadd_rn(__fmul_rn(a, a), __fmul_rn(b, b))), lam);
  n = n < 1.f ? 1.f : n;  // NaN stays NaN, as maximum(1, NaN)
  a = __fdiv_rn(a, n);
  b = __fdiv_rn(b, n);
}

// VEC: four consecutive x per thread with 16-byte accesses (nx % 4 == 0, aligned rows)
template <bool VEC>
__global__ void __launch_bounds__(kThreads) k_tv_prox0(float* __restrict__ px, float* __restrict__ py,
                                                      const float* __restrict__ r, int64_t rows, int ny, int nx,
                                                      float c, float lam) {
  for (int64_t row = blockIdx.x; row < rows; row += gridDim.x) {
    const int y = (int)(row % ny);
    const bool hy = y < ny - 1;
    const int64_t base = row * nx;
    if constexpr (VEC) {
      for (int x = 4 * threadIdx.x; x < nx; x += 4 * kThreads) {
        const int64_t i = base + x;
        const float4 r4 = __ldg(reinterpret_cast<const float4*>(r + i));
        const float4 y4 = hy ? __ldg(reinterpret_cast<const float4*>(r + i + nx)) : r4;
        const float rn = x + 4 < nx ? __ldg(r + i + 4) : 0.f;
        float4 a = *reinterpret_cast<const float4*>(px + i);
        float4 b = *reinterpret_cast<const float4*>(py + i);
        tv_prox0_elem(a.x, b.x, r4.x, r4.y, y4.x, true, hy, c, lam);
        tv_prox0_elem(a.y, b.y, r4.y, r4.z, y4.y, true, hy, c, lam);
        tv_prox0_elem(a.z, b.z, r4.z, r4.w, y4.z, true, hy, c, lam);
        tv_prox0_elem(a.w, b.w, r4.w, rn, y4.w, x + 4 < nx, hy, c, lam);
        *reinterpret_cast<float4*>(px + i) = a;
        *reinterpret_cast<float4*>(py + i) = b;
      }
    } else {
      for (int x = threadIdx.x; x < nx; x += kThreads) {
        const int64_t i = base + x;
        const bool hx = x < nx - 1;
        const float ri = __ldg(r + i);
        float a = px[i], b = py[i];
        tv_prox0_elem(a, b, ri, hx ? __ldg(r + i + 1) : 0.f, hy ? __ldg(r + i + nx) : 0.f, hx, hy, c, lam);
        px[i] = a;
        py[i] = b;
      }
    }
  }
}

// prox1 update of the data term, per element (q = prox1, t = tomo)
//   tv:   (prox1 + c*g - c*tomo)/(1 + c)
//   tve:  u = prox1 + c*g; tmp = 0.5*(u - 1 + sqrt((u - 1)**2 + 4*c*tomo)); tmp[tmp<0] = 0; u - tmp
//   tvl1: tmp = prox1 + c*g - c*tomo; tmp2 = |tmp| - 1; tmp2[tmp2<0] = 0; tmp - tmp2*sign(tmp)
template <int MODE>
__device__ __forceinline__ float tv_prox1_elem(float q, float g, float t, float c, float c1, float c4) {
  const float u = __fadd_rn(q, __fmul_rn(c, g));
  if constexpr (MODE == LP_TV_L2) {
    return __fdiv_rn(__fsub_rn(u, __fmul_rn(c, t)), c1);
  } else if constexpr (MODE == LP_TV_ENTROPY) {
    const float v = __fsub_rn(u, 1.f);
    float tmp = __fmul_rn(0.5f, __fadd_rn(v, __fsqrt_rn(__fadd_rn(__fmul_rn(v, v), __fmul_rn(c4, t)))));
    tmp = tmp < 0.f ? 0.f : tmp;
    return __fsub_rn(u, tmp);
  } else {
    const float tmp = __fsub_rn(u, __fmul_rn(c, t));
    float tmp2 = __fsub_rn(fabsf(tmp), 1.f);
    tmp2 = tmp2 < 0.f ? 0.f : tmp2;
    const float sg = tmp > 0.f ? 1.f : (tmp < 0.f ? -1.f : tmp);  // sign, zeros and NaN kept
    return __fsub_rn(tmp, __fmul_rn(tmp2, sg));
  }
}

// VEC: n4 float4 groups with 16-byte accesses, then the n % 4 tail
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_tv_prox1(float* __restrict__ q, const float* __restrict__ g,
                                                      const float* __restrict__ tomo, int64_t n, int64_t n4, float c,
                                                      float c1, float c4) {
  const int64_t stride = (int64_t)gridDim.x * kThreads;
  const int64_t i0 = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  for (int64_t i = i0; i < n4; i += stride) {
    float4 a = reinterpret_cast<float4*>(q)[i];
    const float4 b = __ldg(reinterpret_cast<const float4*>(g) + i);
    const float4 t = __ldg(reinterpret_cast<const float4*>(tomo) + i);
    a.x = tv_prox1_elem<MODE>(a.x, b.x, t.x, c, c1, c4);
    a.y = tv_prox1_elem<MODE>(a.y, b.y, t.y, c, c1, c4);
    a.z = tv_prox1_elem<MODE>(a.z, b.z, t.z, c, c1, c4);
    a.w = tv_prox1_elem<MODE>(a.w, b.w, t.w, c, c1, c4);
    reinterpret_cast<float4*>(q)[i] = a;
  }
  for (int64_t i = 4 * n4 + i0; i < n; i += stride) q[i] = tv_prox1_elem<MODE>(q[i], __ldg(g + i), __ldg(tomo + i), c, c1, c4);
}

// div0 = d/dx prox0x + d/dy prox0y (backward differences, first row/column taken as is);
// recon0_new = recon0 - c*p + c*div0; recon = 2*recon0_new - recon0
__global__ void __launch_bounds__(kThreads) k_tv_recon(float* __restrict__ r0, float* __restrict__ r,
                                                      const float* __restrict__ p, const float* __restrict__ px,
                                                      const float* __restrict__ py, int64_t rows, int ny, int nx,
                                                      float c) {
  for (int64_t row = blockIdx.x; row < rows; row += gridDim.x) {
    const int y = (int)(row % ny);
    const int64_t base = row * nx;
    for (int x = threadIdx.x; x < nx; x += kThreads) {
      const int64_t i = base + x;
      const float a = __ldg(px + i), b = __ldg(py + i);
      const float dx = x > 0 ? __fsub_rn(a, __ldg(px + i - 1)) : a;
      const float dy = y > 0 ? __fsub_rn(b, __ldg(py + i - nx)) : b;
      const float d = __fadd_rn(dx, dy);
      const float old = r0[i];
      const float nw = __fadd_rn(__fsub_rn(old, __fmul_rn(c, __ldg(p + i))), __fmul_rn(c, d));
      r0[i] = nw;
      r[i] = __fsub_rn(__fmul_rn(2.f, nw), old);
    }
  }
}

int row_grid(int64_t rows) { return (int)(rows < kRowBlocks ? rows : kRowBlocks); }

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

int lp_tv_prox0(float* prox0x, float* prox0y, const float* recon, int S, int ny, int nx, double c, double lam,
                void* stream) {
  if (!prox0x || !prox0y || !recon) return lp_internal_set_err(LP_ERR_ARG, "lp_tv_prox0: null pointer");
  if (S < 1 || ny < 1 || nx < 1) return lp_internal_set_err(LP_ERR_ARG, "lp_tv_prox0: bad sizes");
  const int64_t rows = (int64_t)S * ny;
  const bool vec = nx % 4 == 0 && ((((uintptr_t)prox0x) | ((uintptr_t)prox0y) | ((uintptr_t)recon)) & 15) == 0;
  cudaStream_t st = (cudaStream_t)stream;
  if (vec)
    k_tv_prox0<true><<<row_grid(rows), kThreads, 0, st>>>(prox0x, prox0y, recon, rows, ny, nx, (float)c, (float)lam);
  else
    k_tv_prox0<false><<<row_grid(rows), kThreads, 0, st>>>(prox0x, prox0y, recon, rows, ny, nx, (float)c, (float)lam);
  return launch_err("lp_tv_prox0");
}

int lp_tv_prox1(float* prox1, const float* g, const float* tomo, int64_t n, double c, int mode, void* stream) {
  if (!prox1 || !g || !tomo) return lp_internal_set_err(LP_ERR_ARG, "lp_tv_prox1: null pointer");
  if (n < 0) return lp_internal_set_err(LP_ERR_ARG, "lp_tv_prox1: bad size");
  if (mode != LP_TV_L2 && mode != LP_TV_ENTROPY && mode != LP_TV_L1)
    return lp_internal_set_err(LP_ERR_ARG, "lp_tv_prox1: mode must be LP_TV_L2, LP_TV_ENTROPY or LP_TV_L1");
  // c, 1 + c and 4*c each rounded once from double, as the reference's Python
  // scalars reach its float32 arrays
  const float c1 = (float)(1.0 + c), c4 = (float)(4.0 * c);
  const bool vec = ((((uintptr_t)prox1) | ((uintptr_t)g) | ((uintptr_t)tomo)) & 15) == 0;
  const int64_t n4 = vec ? n / 4 : 0;
  cudaStream_t st = (cudaStream_t)stream;
  const int grid = parts_per_slice(1);
  if (mode == LP_TV_L2)
    k_tv_prox1<LP_TV_L2><<<grid, kThreads, 0, st>>>(prox1, g, tomo, n, n4, (float)c, c1, c4);
  else if (mode == LP_TV_ENTROPY)
    k_tv_prox1<LP_TV_ENTROPY><<<grid, kThreads, 0, st>>>(prox1, g, tomo, n, n4, (float)c, c1, c4);
  else
    k_tv_prox1<LP_TV_L1><<<grid, kThreads, 0, st>>>(prox1, g, tomo, n, n4, (float)c, c1, c4);
  return launch_err("lp_tv_prox1");
}

int lp_tv_recon(float* recon0, float* recon, const float* p, const float* prox0x, const float* prox0y, int S, int ny,
                int nx, double c, void* stream) {
  if (!recon0 || !recon || !p || !prox0x || !prox0y) return lp_internal_set_err(LP_ERR_ARG, "lp_tv_recon: null pointer");
  if (S < 1 || ny < 1 || nx < 1) return lp_internal_set_err(LP_ERR_ARG, "lp_tv_recon: bad sizes");
  const int64_t rows = (int64_t)S * ny;
  k_tv_recon<<<row_grid(rows), kThreads, 0, (cudaStream_t)stream>>>(recon0, recon, p, prox0x, prox0y, rows, ny, nx,
                                                                     (float)c);
  return launch_err("lp_tv_recon");
}

}  // extern "C"
