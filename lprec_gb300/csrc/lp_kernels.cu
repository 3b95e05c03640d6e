// Hot-path kernels of the log-polar Radon transform (fwd) and back-projection (adj).
//
// Reference pipeline (src/cuda/lpRgpu.cu:243-330): per angular span, gather the
// input onto a 2N x N log-polar grid through texture fetches, 2-D R2C FFT,
// multiply by fZ, C2R, gather back.  Here the grid is processed column-wise
// (a column = one log-polar angle theta, 2N samples along rho):
//
//   * gather + real FFT along rho are fused (two columns per complex FFT);
//   * the FFT along theta, the kernel multiply and the inverse theta FFT are
//     one kernel per rho frequency;
//   * the inverse FFT along rho is fused with the gather that reads the grid:
//     every polar angle row samples a single theta position, so its four
//     theta taps are combined in the frequency domain and one inverse FFT
//     yields the whole row's rho profile.
//
// Texture fetches are replaced by explicit interpolation with wrap addressing
// at index position (x, y), which is what sampling the reference's textures
// at (x+0.5, y+0.5) means (src/include/main_kernels.cuh:21-84).
#include "lp_kernels.cuh"

namespace lpgb {

// cubic B-spline pole and gain (src/include/main_kernels.cuh:2, :124)
#define LP_POLE (-0.2679491924311228f)
#define LP_LAMBDA (6.0f)
#define LP_WARM 16  // warm-up length of the chunked recursions: |pole|^16 < 1e-9

__device__ __forceinline__ int wrapi(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

// cubic B-spline weights for taps i-1, i, i+1, i+2 at fraction f
__device__ __forceinline__ void bspline_w(float f, float* w) {
  const float one = 1.0f - f;
  const float f2 = f * f;
  const float o2 = one * one;
  w[0] = (1.0f / 6.0f) * o2 * one;
  w[1] = (2.0f / 3.0f) - 0.5f * f2 * (2.0f - f);
  w[2] = (2.0f / 3.0f) - 0.5f * o2 * (2.0f - one);
  w[3] = (1.0f / 6.0f) * f2 * f;
}

// 2-D interpolation of a row-major image (W columns, H rows) at index position
// (x, y) with wrap addressing.
__device__ __forceinline__ float interp2d(const float* __restrict__ img, int W, int H, float x, float y,
                                          int cubic) {
  const float fx = floorf(x), fy = floorf(y);
  const int ix = (int)fx, iy = (int)fy;
  const float ax = x - fx, ay = y - fy;
  if (cubic) {
    float wx[4], wy[4];
    bspline_w(ax, wx);
    bspline_w(ay, wy);
    int cx[4];
    if (ix >= 1 && ix + 2 < W) {
#pragma unroll
      for (int i = 0; i < 4; ++i) cx[i] = ix - 1 + i;
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i) cx[i] = wrapi(ix - 1 + i, W);
    }
    float acc = 0.f;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float* row = img + (size_t)wrapi(iy - 1 + j, H) * W;
      const float r = wx[0] * __ldg(row + cx[0]) + wx[1] * __ldg(row + cx[1]) + wx[2] * __ldg(row + cx[2]) +
                      wx[3] * __ldg(row + cx[3]);
      acc += wy[j] * r;
    }
    return acc;
  }
  const int x0 = wrapi(ix, W), x1 = wrapi(ix + 1, W);
  const float* r0 = img + (size_t)wrapi(iy, H) * W;
  const float* r1 = img + (size_t)wrapi(iy + 1, H) * W;
  return (1.f - ay) * ((1.f - ax) * __ldg(r0 + x0) + ax * __ldg(r0 + x1)) +
         ay * ((1.f - ax) * __ldg(r1 + x0) + ax * __ldg(r1 + x1));
}

// 1-D interpolation along a shared-memory line of length L (wrap).
template <typename Get>
__device__ __forceinline__ float interp1d(Get get, int L, float x, int cubic) {
  const float fx = floorf(x);
  const int ix = (int)fx;
  const float ax = x - fx;
  if (cubic) {
    float w[4];
    bspline_w(ax, w);
    float acc = 0.f;
    if (ix >= 1 && ix + 2 < L) {
#pragma unroll
      for (int i = 0; i < 4; ++i) acc += w[i] * get(ix - 1 + i);
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i) acc += w[i] * get(wrapi(ix - 1 + i, L));
    }
    return acc;
  }
  return (1.f - ax) * get(wrapi(ix, L)) + ax * get(wrapi(ix + 1, L));
}

// Interpolation weights along one axis at coordinate t: taps start at *first.
__device__ __forceinline__ int axis_weights(float t, int cubic, float* w) {
  const float ft = floorf(t);
  const int it = (int)ft;
  if (cubic) {
    bspline_w(t - ft, w);
    return it - 1;
  }
  w[0] = 1.f - (t - ft);
  w[1] = t - ft;
  w[2] = 0.f;
  w[3] = 0.f;
  return it;
}

// ---------------------------------------------------------------------------
// Cubic B-spline prefilter of one line held in shared memory
// (ConvertToInterpolationCoefficients, src/include/main_kernels.cuh:97-142).
// The block splits the line into chunks; every chunk starts its causal and
// anticausal recursions LP_WARM samples early from a zero state, which is
// exact to |pole|^16 ~ 7e-10; the first and last chunk use the reference's
// boundary initialisations.  `cp` is scratch of L floats.
// ---------------------------------------------------------------------------
__device__ void prefilter_line(float* line, float* cp, int L, int tid, int nth) {
  const float z = LP_POLE;
  const int C = (L + nth - 1) / nth;
  const int b = tid * C;
  const int e = min(b + C, L);
  if (b < L) {
    float prev;
    const int n0 = b - LP_WARM;
    int n = 0;
    if (n0 <= 0) {
      const int hor = min(12, L);
      float sum = line[0];
      float zn = z;
      for (int i = 0; i < hor; ++i) {
        sum += zn * line[i];
        zn *= z;
      }
      prev = LP_LAMBDA * sum;
      if (b == 0) cp[0] = prev;
      n = 1;
    } else {
      prev = LP_LAMBDA * line[n0];
      n = n0 + 1;
    }
    for (; n < e; ++n) {
      prev = LP_LAMBDA * line[n] + z * prev;
      if (n >= b) cp[n] = prev;
    }
  }
  __syncthreads();
  if (b < L) {
    const int n1 = e - 1 + LP_WARM;
    float c;
    int n;
    if (n1 >= L - 1) {
      c = (z / (z - 1.0f)) * cp[L - 1];
      if (L - 1 < e) line[L - 1] = c;
      n = L - 2;
    } else {
      c = -z * cp[n1];
      n = n1 - 1;
    }
    for (; n >= b; --n) {
      c = z * (c - cp[n]);
      if (n < e) line[n] = c;
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// forward: centre the image in the padded grid and prefilter along x
// (copy3Dshifted lpRgpu.cu:189 + first half of prefilter2D lpRgpu.cu:219-229)
// ---------------------------------------------------------------------------
__global__ void k_fwd_ingest(FwdIngestArgs a) {
  extern __shared__ float smf[];
  float* line = smf;
  float* cp = smf + a.N;
  const int s = blockIdx.x;
  const int y = blockIdx.y;
  const int Y = y - a.off;
  const float* src = a.fin + ((size_t)s * a.N0 + (size_t)max(Y, 0)) * a.N0;
  for (int x = threadIdx.x; x < a.N; x += blockDim.x) {
    const int X = x - a.off;
    line[x] = (Y >= 0 && Y < a.N0 && X >= 0 && X < a.N0) ? __ldg(src + X) : 0.f;
  }
  __syncthreads();
  if (a.cubic) prefilter_line(line, cp, a.N, threadIdx.x, blockDim.x);
  float* dst = a.fbuf + ((size_t)s * a.N + y) * a.N;
  for (int x = threadIdx.x; x < a.N; x += blockDim.x) dst[x] = line[x];
}

// ---------------------------------------------------------------------------
// prefilter along the slow axis, in place: block = 32 columns x nch chunks.
// Each chunk reads its warm-up samples before anyone overwrites them, writes
// its causal coefficients in place, then reads the next chunk's first
// LP_WARM causal coefficients before the anticausal pass overwrites them.
// ---------------------------------------------------------------------------
__global__ void k_col_prefilter(ColPrefilterArgs a) {
  const int x = blockIdx.x * 32 + threadIdx.x;
  const int s = blockIdx.y;
  const int nch = blockDim.y;
  const int H = a.H, W = a.W;
  const int C = (H + nch - 1) / nch;
  const int b = threadIdx.y * C;
  const int e = min(b + C, H);
  const bool active = (x < W) && (b < H);
  float* col = a.img + (size_t)s * H * W + x;
  const float z = LP_POLE;
  float wu[LP_WARM];
  // phase 0: warm-up samples (or the exact causal initialisation)
  float prev = 0.f;
  if (active) {
    if (b == 0) {
      const int hor = min(12, H);
      float sum = col[0];
      float zn = z;
      for (int i = 0; i < hor; ++i) {
        sum += zn * col[(size_t)i * W];
        zn *= z;
      }
      prev = sum;  // marker: exact start handled below
    } else {
#pragma unroll
      for (int i = 0; i < LP_WARM; ++i) {
        const int n = b - LP_WARM + i;
        wu[i] = n >= 0 ? col[(size_t)n * W] : 0.f;
      }
    }
  }
  __syncthreads();
  if (active) {
    int n;
    if (b == 0) {
      prev = LP_LAMBDA * prev;
      col[0] = prev;
      n = 1;
    } else {
      prev = 0.f;
#pragma unroll
      for (int i = 0; i < LP_WARM; ++i) prev = LP_LAMBDA * wu[i] + z * prev;
      n = b;
    }
    for (; n < e; ++n) {
      prev = LP_LAMBDA * col[(size_t)n * W] + z * prev;
      col[(size_t)n * W] = prev;
    }
  }
  __syncthreads();
  int nw = 0;
  if (active) {
    nw = min(LP_WARM, H - e);
#pragma unroll
    for (int i = 0; i < LP_WARM; ++i)
      if (i < nw) wu[i] = col[(size_t)(e + i) * W];
  }
  __syncthreads();
  if (active) {
    float c;
    int n;
    if (e + nw >= H) {
      // exact anticausal initialisation at H-1
      float last = (nw > 0) ? wu[nw - 1] : col[(size_t)(H - 1) * W];
      c = (z / (z - 1.0f)) * last;
      if (nw == 0) {
        col[(size_t)(H - 1) * W] = c;
        n = H - 2;
      } else {
        for (int i = nw - 2; i >= 0; --i) c = z * (c - wu[i]);
        n = e - 1;
      }
    } else {
      c = -z * wu[LP_WARM - 1];
      for (int i = LP_WARM - 2; i >= 0; --i) c = z * (c - wu[i]);
      n = e - 1;
    }
    for (; n >= b; --n) {
      c = z * (c - col[(size_t)n * W]);
      col[(size_t)n * W] = c;
    }
  }
}

// ---------------------------------------------------------------------------
// forward, per span: gather Cartesian -> log-polar for two theta columns,
// multiply by e^rho, FFT along rho (two real columns in one complex FFT).
// Reference: interp mode 3 (lpRgpu.cu:263), mulexp (:267), R2C (:270).
// ---------------------------------------------------------------------------
__global__ void k_fwd_c2lp(FwdC2LPArgs a) {
  extern __shared__ float2 sm2[];
  float2* A = sm2;
  float2* B = sm2 + a.Nrho;
  const int s = blockIdx.x;
  const int th = 2 * blockIdx.y;
  const int thb = th + 1 < a.Nth ? th + 1 : -1;
  const float* img = a.fbuf + (size_t)s * a.N * a.N;
  const float2* ca = a.c2lp + (size_t)th * a.Nrho;
  const float2* cb = a.c2lp + (size_t)max(thb, 0) * a.Nrho;
  for (int r = threadIdx.x; r < a.Nrho; r += blockDim.x) {
    const float e = __ldg(a.erho + r);
    const float2 pa = __ldg(ca + r);
    float va = 0.f, vb = 0.f;
    if (!isnan(pa.x)) va = e * interp2d(img, a.N, a.N, pa.x, pa.y, a.cubic);
    if (thb >= 0) {
      const float2 pb = __ldg(cb + r);
      if (!isnan(pb.x)) vb = e * interp2d(img, a.N, a.N, pb.x, pb.y, a.cubic);
    }
    A[r] = make_float2(va, vb);
  }
  __syncthreads();
  const float2* Z = fft_block<-1>(A, B, a.plan, 1, a.Nrho);
  float2* out = a.spec + (size_t)s * a.Nk * a.Nth;
  for (int k = threadIdx.x; k < a.Nk; k += blockDim.x) {
    const float2 z1 = Z[k];
    const float2 z2 = Z[k == 0 ? 0 : a.Nrho - k];
    out[(size_t)k * a.Nth + th] = make_float2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
    if (thb >= 0) out[(size_t)k * a.Nth + thb] = make_float2(0.5f * (z1.y + z2.y), 0.5f * (z2.x - z1.x));
  }
}

// ---------------------------------------------------------------------------
// per rho frequency: FFT along theta, multiply by fZ/(Nrho*Ntheta), inverse.
// Reference: the theta half of cuFFT's 2-D R2C/C2R and `mul`
// (lpRgpu.cu:270-277, simple_kernels.cuh:2-12).
// ---------------------------------------------------------------------------
__global__ void k_theta_conv(ThetaConvArgs a) {
  extern __shared__ float2 sm2[];
  float2* A = sm2;
  float2* B = sm2 + a.Nth;
  const int s = blockIdx.x;
  const int k = blockIdx.y;
  float2* row = a.spec + ((size_t)s * a.Nk + k) * a.Nth;
  for (int t = threadIdx.x; t < a.Nth; t += blockDim.x)
    A[t] = (t >= a.in_lo && t <= a.in_hi) ? row[t] : make_float2(0.f, 0.f);
  __syncthreads();
  float2* X = fft_block<-1>(A, B, a.plan, 1, a.Nth);
  const float2* fz = a.fz + (size_t)k * a.Nth;
  for (int t = threadIdx.x; t < a.Nth; t += blockDim.x) {
    float2 w = __ldg(fz + t);
    if (a.conj_fz) w.y = -w.y;
    X[t] = cscale(cmul(X[t], w), a.scale);
  }
  __syncthreads();
  float2* Y = fft_block<1>(X, X == A ? B : A, a.plan, 1, a.Nth);
  for (int t = a.out_lo + threadIdx.x; t <= a.out_hi; t += blockDim.x) row[t] = Y[t];
}

// Build the complex signal whose inverse FFT gives two real rho profiles
// from their half spectra V0, V1 (kr = 0..Nrho/2); C2R semantics: the
// imaginary parts at kr = 0 and kr = Nrho/2 are ignored.
__device__ __forceinline__ void put_pair(float2* Z, int k, int Nrho, float2 v0, float2 v1) {
  const int half = Nrho / 2;
  if (k == 0 || k == half) {
    Z[k] = make_float2(v0.x, v1.x);
  } else {
    Z[k] = make_float2(v0.x - v1.y, v0.y + v1.x);
    Z[Nrho - k] = make_float2(v0.x + v1.y, v1.x - v0.y);
  }
}

// ---------------------------------------------------------------------------
// forward, per span: two polar angle rows per block.  Each row's theta taps
// are combined in the frequency domain, one inverse FFT along rho gives both
// rows' rho profiles, then the rho interpolation at every s.  Writes straight
// into the caller's sinogram (stepangles + cor window, lpRgpu.cu:191-192).
// Reference: C2R (:277), interp mode 5 (:284).
// ---------------------------------------------------------------------------
__global__ void k_fwd_lp2polar(FwdLP2PolarArgs a) {
  extern __shared__ float2 sm2[];
  float2* A = sm2;
  float2* B = sm2 + a.Nrho;
  const int s = blockIdx.x;
  const int i0 = 2 * blockIdx.y;
  const int r0 = a.rows[i0];
  const int r1 = (i0 + 1 < a.nrows) ? a.rows[i0 + 1] : -1;
  float w0[4], w1[4];
  const int c0 = axis_weights(__ldg(a.thc + r0), a.cubic, w0);
  int c1 = 0;
  if (r1 >= 0) {
    c1 = axis_weights(__ldg(a.thc + r1), a.cubic, w1);
  } else {
    w1[0] = w1[1] = w1[2] = w1[3] = 0.f;
  }
  int t0[4], t1[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    t0[j] = wrapi(c0 + j, a.Nth);
    t1[j] = wrapi(c1 + j, a.Nth);
  }
  const int ntap = a.cubic ? 4 : 2;
  const float2* sp = a.spec + (size_t)s * a.Nk * a.Nth;
  for (int k = threadIdx.x; k < a.Nk; k += blockDim.x) {
    const float2* row = sp + (size_t)k * a.Nth;
    float2 v0 = make_float2(0.f, 0.f), v1 = make_float2(0.f, 0.f);
    for (int j = 0; j < ntap; ++j) {
      const float2 q0 = row[t0[j]];
      v0.x += w0[j] * q0.x;
      v0.y += w0[j] * q0.y;
      const float2 q1 = row[t1[j]];
      v1.x += w1[j] * q1.x;
      v1.y += w1[j] * q1.y;
    }
    put_pair(A, k, a.Nrho, v0, v1);
  }
  __syncthreads();
  const float2* zr = fft_block<1>(A, B, a.plan, 1, a.Nrho);
  const int Nrho = a.Nrho;
  for (int x = threadIdx.x; x < a.N; x += blockDim.x) {
    const int xo = x - a.cor_off;
    if (xo < 0 || xo >= a.N0) continue;
    if (r0 % a.os == 0) {
      const float t = __ldg(a.rhoc + (size_t)r0 * a.N + x);
      const float v = interp1d([&](int i) { return zr[i].x; }, Nrho, t, a.cubic);
      a.Rout[((size_t)s * a.Nproj0 + r0 / a.os) * a.N0 + xo] = v;
    }
    if (r1 >= 0 && r1 % a.os == 0) {
      const float t = __ldg(a.rhoc + (size_t)r1 * a.N + x);
      const float v = interp1d([&](int i) { return zr[i].y; }, Nrho, t, a.cubic);
      a.Rout[((size_t)s * a.Nproj0 + r1 / a.os) * a.N0 + xo] = v;
    }
  }
}

// ---------------------------------------------------------------------------
// adjoint ingest, two input rows per block: cor shift + angle step + edge
// padding (lpRgpu.cu:199-203, :211-216, padker), the FBP filter (applyFilter
// lpRgpu.cu:333-382) as one complex FFT of length 4N for both rows, and the
// row (s direction) prefilter.  Rows between angle steps are written as 0.
// ---------------------------------------------------------------------------
__global__ void k_adj_ingest(AdjIngestArgs a) {
  extern __shared__ float2 sm2[];
  const int N = a.N;
  const int M = 4 * N;
  const bool filt = a.H != nullptr;
  float2* F0 = sm2;
  float2* F1 = sm2 + (filt ? M : 0);
  float* lines = reinterpret_cast<float*>(sm2 + (filt ? 2 * M : 0));  // 2 rows
  float* cp = lines + 2 * N;                                          // 2 rows scratch
  const int s = blockIdx.x;
  const int q0 = 2 * blockIdx.y;
  const int q1 = q0 + 1 < a.Nproj0 ? q0 + 1 : -1;
  const float* in0 = a.Rin + ((size_t)s * a.Nproj0 + q0) * a.N0;
  const float* in1 = a.Rin + ((size_t)s * a.Nproj0 + max(q1, 0)) * a.N0;
  for (int x = threadIdx.x; x < N; x += blockDim.x) {
    const int xi = min(max(x - a.cor_off, 0), a.N0 - 1);
    lines[x] = __ldg(in0 + xi);
    lines[N + x] = q1 >= 0 ? __ldg(in1 + xi) : 0.f;
  }
  __syncthreads();
  if (filt) {
    for (int x = threadIdx.x; x < M; x += blockDim.x)
      F0[x] = x < N ? make_float2(lines[x], lines[N + x]) : make_float2(0.f, 0.f);
    __syncthreads();
    float2* X = fft_block<-1>(F0, F1, a.plan, 1, M);
    const float sc = 1.0f / (float)M;
    for (int k = threadIdx.x; k < M; k += blockDim.x) X[k] = cscale(X[k], __ldg(a.H + k) * sc);
    __syncthreads();
    float2* Y = fft_block<1>(X, X == F0 ? F1 : F0, a.plan, 1, M);
    for (int x = threadIdx.x; x < N; x += blockDim.x) {
      lines[x] = Y[x].x;
      lines[N + x] = Y[x].y;
    }
    __syncthreads();
  }
  if (a.cubic) {
    // two lines at once: half of the block each
    const int half = blockDim.x / 2;
    const int which = threadIdx.x >= half;
    const int tid = threadIdx.x - which * half;
    // prefilter_line synchronises the whole block; both halves call it together
    prefilter_line(lines + which * N, cp + which * N, N, tid, half);
  }
  for (int rr = 0; rr < 2; ++rr) {
    const int q = rr == 0 ? q0 : q1;
    if (q < 0) break;
    for (int j = 0; j < a.os; ++j) {
      float* dst = a.rbuf + ((size_t)s * a.Nproj + (size_t)q * a.os + j) * N;
      for (int x = threadIdx.x; x < N; x += blockDim.x) dst[x] = j == 0 ? lines[rr * N + x] : 0.f;
    }
  }
}

// ---------------------------------------------------------------------------
// adjoint, per span: two log-polar theta columns per block.  Every column
// samples the sinogram at one angle position: its four angle taps are
// combined into one s profile, interpolated along s for every rho; wrap
// points add a direct 2-D sample.  Then FFT along rho.
// Reference: interp mode 4 for lpids and wids (lpRgpu.cu:307, :311), R2C (:314).
// ---------------------------------------------------------------------------
__global__ void k_adj_polar2lp(AdjPolar2LPArgs a) {
  extern __shared__ float2 sm2[];
  float2* A = sm2;
  float2* B = sm2 + a.Nrho;
  float* prof = reinterpret_cast<float*>(sm2 + 2 * a.Nrho);  // 2 x N
  const int s = blockIdx.x;
  const int th0 = a.clo + 2 * blockIdx.y;
  const int th1 = th0 + 1 <= a.chi ? th0 + 1 : -1;
  const float* img = a.rbuf + (size_t)s * a.Nproj * a.N;
  const float ta0 = __ldg(a.ta + th0);
  const float ta1 = th1 >= 0 ? __ldg(a.ta + th1) : __int_as_float(0x7fc00000);
  float w0[4], w1[4];
  int rw0[4], rw1[4];
  const bool has0 = !isnan(ta0), has1 = !isnan(ta1);
  const int ntap = a.cubic ? 4 : 2;
  {
    const int c0 = has0 ? axis_weights(ta0, a.cubic, w0) : 0;
    const int c1 = has1 ? axis_weights(ta1, a.cubic, w1) : 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      rw0[j] = wrapi(c0 + j, a.Nproj);
      rw1[j] = wrapi(c1 + j, a.Nproj);
    }
  }
  for (int x = threadIdx.x; x < a.N; x += blockDim.x) {
    float p0 = 0.f, p1 = 0.f;
    for (int j = 0; j < ntap; ++j) {
      if (has0) p0 += w0[j] * __ldg(img + (size_t)rw0[j] * a.N + x);
      if (has1) p1 += w1[j] * __ldg(img + (size_t)rw1[j] * a.N + x);
    }
    prof[x] = p0;
    prof[a.N + x] = p1;
  }
  __syncthreads();
  const float* sx0 = a.sx + (size_t)th0 * a.Nrho;
  const float* sx1 = a.sx + (size_t)max(th1, 0) * a.Nrho;
  for (int r = threadIdx.x; r < a.Nrho; r += blockDim.x) {
    float v0 = 0.f, v1 = 0.f;
    const float x0 = __ldg(sx0 + r);
    if (!isnan(x0)) v0 = interp1d([&](int i) { return prof[i]; }, a.N, x0, a.cubic);
    if (th1 >= 0) {
      const float x1 = __ldg(sx1 + r);
      if (!isnan(x1)) v1 = interp1d([&](int i) { return prof[a.N + i]; }, a.N, x1, a.cubic);
    }
    A[r] = make_float2(v0, v1);
  }
  __syncthreads();
  // wrap points (distinct rho within a column)
  for (int c = 0; c < 2; ++c) {
    const int th = c == 0 ? th0 : th1;
    if (th < 0) break;
    const int w_begin = __ldg(a.woff + th), w_end = __ldg(a.woff + th + 1);
    for (int w = w_begin + threadIdx.x; w < w_end; w += blockDim.x) {
      const float4 p = __ldg(a.wpt + w);
      const int r = (int)p.x;
      const float v = interp2d(img, a.N, a.Nproj, p.y, p.z, a.cubic);
      if (c == 0) A[r].x += v;
      else A[r].y += v;
    }
    __syncthreads();
  }
  const float2* Z = fft_block<-1>(A, B, a.plan, 1, a.Nrho);
  float2* out = a.spec + (size_t)s * a.Nk * a.Nth;
  for (int k = threadIdx.x; k < a.Nk; k += blockDim.x) {
    const float2 z1 = Z[k];
    const float2 z2 = Z[k == 0 ? 0 : a.Nrho - k];
    out[(size_t)k * a.Nth + th0] = make_float2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
    if (th1 >= 0) out[(size_t)k * a.Nth + th1] = make_float2(0.5f * (z1.y + z2.y), 0.5f * (z2.x - z1.x));
  }
}

// ---------------------------------------------------------------------------
// adjoint, per span: inverse FFT along rho for two theta columns, store the
// real log-polar columns [theta][rho] for the Cartesian gather (C2R :321).
// ---------------------------------------------------------------------------
__global__ void k_adj_lpcols(AdjLPColsArgs a) {
  extern __shared__ float2 sm2[];
  float2* A = sm2;
  float2* B = sm2 + a.Nrho;
  const int s = blockIdx.x;
  const int th0 = a.lo2 + 2 * blockIdx.y;
  const int th1 = th0 + 1 <= a.hi2 ? th0 + 1 : -1;
  const float2* sp = a.spec + (size_t)s * a.Nk * a.Nth;
  for (int k = threadIdx.x; k < a.Nk; k += blockDim.x) {
    const float2 v0 = sp[(size_t)k * a.Nth + th0];
    const float2 v1 = th1 >= 0 ? sp[(size_t)k * a.Nth + th1] : make_float2(0.f, 0.f);
    put_pair(A, k, a.Nrho, v0, v1);
  }
  __syncthreads();
  const float2* z = fft_block<1>(A, B, a.plan, 1, a.Nrho);
  float* g0 = a.G + ((size_t)s * a.W2 + (th0 - a.lo2)) * a.Nrho;
  for (int r = threadIdx.x; r < a.Nrho; r += blockDim.x) {
    g0[r] = z[r].x;
    if (th1 >= 0) g0[a.Nrho + r] = z[r].y;
  }
}

// ---------------------------------------------------------------------------
// adjoint: log-polar -> Cartesian gather summed over the three spans, written
// straight into the caller's N0 x N0 window (interp mode 5, lpRgpu.cu:328,
// copy3Dshifted :206).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float interp_cols(const float* __restrict__ G, int Nrho, int Nth, int lo2, int W2,
                                             float2 t, int cubic) {
  float wt[4], wr[4];
  const int ct = axis_weights(t.x, cubic, wt);
  const int cr = axis_weights(t.y, cubic, wr);
  const int nt = cubic ? 4 : 2;
  int rr[4];
  const bool inner = (cr >= 0 && cr + 3 < Nrho);
#pragma unroll
  for (int i = 0; i < 4; ++i) rr[i] = inner ? cr + i : wrapi(cr + i, Nrho);
  float acc = 0.f;
  for (int j = 0; j < nt; ++j) {
    const int col = wrapi(ct + j, Nth) - lo2;
    if (col < 0 || col >= W2) continue;  // outside the stored band: zero weight by construction
    const float* g = G + (size_t)col * Nrho;
    float v = 0.f;
#pragma unroll
    for (int i = 0; i < 4; ++i)
      if (i < nt) v += wr[i] * __ldg(g + rr[i]);
    acc += wt[j] * v;
  }
  return acc;
}

__global__ void k_adj_lp2cart(AdjLP2CartArgs a) {
  const int s = blockIdx.x;
  const int p = blockIdx.y * blockDim.x + threadIdx.x;
  if (p >= a.npix) return;
  const size_t gs = (size_t)s * a.W2 * a.Nrho;
  float acc = 0.f;
  const float2 t0 = __ldg(a.c2lp0 + p);
  if (!isnan(t0.x)) {
    acc += interp_cols(a.G0 + gs, a.Nrho, a.Nth, a.lo2, a.W2, t0, a.cubic);
    acc += interp_cols(a.G1 + gs, a.Nrho, a.Nth, a.lo2, a.W2, __ldg(a.c2lp1 + p), a.cubic);
    acc += interp_cols(a.G2 + gs, a.Nrho, a.Nth, a.lo2, a.W2, __ldg(a.c2lp2 + p), a.cubic);
  }
  a.fout[(size_t)s * a.npix + p] = acc;
}

// ---------------------------------------------------------------------------
// launches
// ---------------------------------------------------------------------------
static const int kFFTThreads = 256;

static size_t smem_c2lp(int Nrho) { return 2 * (size_t)Nrho * sizeof(float2); }
static size_t smem_theta(int Nth) { return 2 * (size_t)Nth * sizeof(float2); }
static size_t smem_adj_ingest(int N, bool filt) {
  return (filt ? 2 * (size_t)4 * N * sizeof(float2) : 0) + 4 * (size_t)N * sizeof(float);
}
static size_t smem_polar2lp(int Nrho, int N) { return 2 * (size_t)Nrho * sizeof(float2) + 2 * (size_t)N * sizeof(float); }

static int g_smem_optin = 48 * 1024;

// Allow every kernel the device's opt-in shared memory; launches check their
// own need against it.
cudaError_t configure_kernels(int N) {
  (void)N;
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  g_smem_optin = optin;
  const void* ks[] = {(const void*)k_fwd_ingest, (const void*)k_fwd_c2lp, (const void*)k_theta_conv,
                      (const void*)k_fwd_lp2polar, (const void*)k_adj_ingest, (const void*)k_adj_polar2lp,
                      (const void*)k_adj_lpcols};
  for (const void* k : ks) {
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

static cudaError_t smem_ok(size_t need) {
  return need <= (size_t)g_smem_optin ? cudaSuccess : cudaErrorInvalidConfiguration;
}

cudaError_t launch_fwd_ingest(const FwdIngestArgs& a, int S, cudaStream_t st) {
  if (smem_ok(2 * (size_t)a.N * sizeof(float)) != cudaSuccess) return cudaErrorInvalidConfiguration;
  dim3 grid(S, a.N);
  k_fwd_ingest<<<grid, 128, 2 * (size_t)a.N * sizeof(float), st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_col_prefilter(const ColPrefilterArgs& a, int S, cudaStream_t st) {
  int nch = a.H / LP_WARM;
  if (nch > 32) nch = 32;
  if (nch < 1) nch = 1;
  dim3 block(32, nch);
  dim3 grid((a.W + 31) / 32, S);
  k_col_prefilter<<<grid, block, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_fwd_c2lp(const FwdC2LPArgs& a, int S, cudaStream_t st) {
  if (smem_ok(smem_c2lp(a.Nrho)) != cudaSuccess) return cudaErrorInvalidConfiguration;
  dim3 grid(S, (a.Nth + 1) / 2);
  k_fwd_c2lp<<<grid, kFFTThreads, smem_c2lp(a.Nrho), st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_theta_conv(const ThetaConvArgs& a, int S, cudaStream_t st) {
  if (smem_ok(smem_theta(a.Nth)) != cudaSuccess) return cudaErrorInvalidConfiguration;
  dim3 grid(S, a.Nk);
  k_theta_conv<<<grid, kFFTThreads, smem_theta(a.Nth), st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_fwd_lp2polar(const FwdLP2PolarArgs& a, int S, cudaStream_t st) {
  if (a.nrows <= 0) return cudaSuccess;
  if (smem_ok(smem_c2lp(a.Nrho)) != cudaSuccess) return cudaErrorInvalidConfiguration;
  dim3 grid(S, (a.nrows + 1) / 2);
  k_fwd_lp2polar<<<grid, kFFTThreads, smem_c2lp(a.Nrho), st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_adj_ingest(const AdjIngestArgs& a, int S, cudaStream_t st) {
  if (smem_ok(smem_adj_ingest(a.N, a.H != nullptr)) != cudaSuccess) return cudaErrorInvalidConfiguration;
  dim3 grid(S, (a.Nproj0 + 1) / 2);
  k_adj_ingest<<<grid, kFFTThreads, smem_adj_ingest(a.N, a.H != nullptr), st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_adj_polar2lp(const AdjPolar2LPArgs& a, int S, cudaStream_t st) {
  if (a.chi < a.clo) return cudaSuccess;
  if (smem_ok(smem_polar2lp(a.Nrho, a.N)) != cudaSuccess) return cudaErrorInvalidConfiguration;
  dim3 grid(S, (a.chi - a.clo + 2) / 2);
  k_adj_polar2lp<<<grid, kFFTThreads, smem_polar2lp(a.Nrho, a.N), st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_adj_lpcols(const AdjLPColsArgs& a, int S, cudaStream_t st) {
  if (smem_ok(smem_c2lp(a.Nrho)) != cudaSuccess) return cudaErrorInvalidConfiguration;
  dim3 grid(S, (a.hi2 - a.lo2 + 2) / 2);
  k_adj_lpcols<<<grid, kFFTThreads, smem_c2lp(a.Nrho), st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_adj_lp2cart(const AdjLP2CartArgs& a, int S, cudaStream_t st) {
  dim3 grid(S, (a.npix + 255) / 256);
  k_adj_lp2cart<<<grid, 256, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace lpgb
