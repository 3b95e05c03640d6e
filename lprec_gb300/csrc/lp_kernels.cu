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
#include <algorithm>

#include "lp_p2.cuh"

namespace lpgb {

// ---------------------------------------------------------------------------
// forward: centre the image in the padded grid and prefilter along x
// (copy3Dshifted lpRgpu.cu:189 + first half of prefilter2D lpRgpu.cu:219-229)
// ---------------------------------------------------------------------------
__global__ void k_fwd_ingest(FwdIngestArgs a) {
  extern __shared__ float smf[];
  const int C = line_chunk(a.N, blockDim.x);
  float* line = smf;
  float* cp = smf + line_floats(a.N, blockDim.x);
  const int s = blockIdx.x;
  const int y = blockIdx.y;
  const int Y = y - a.off;
  const float* src = a.fin + ((size_t)s * a.N0 + (size_t)max(Y, 0)) * a.N0;
  float* dst = a.fbuf + ((size_t)s * a.N + y) * a.N;
  // 16-byte path: with off, N0 and N multiples of 4 every group of 4 samples lies
  // wholly inside or outside the image, and rows start 16-byte aligned
  const bool vec = ((a.off | a.N0 | a.N) & 3) == 0 && ((((uintptr_t)a.fin) | ((uintptr_t)a.fbuf)) & 15) == 0;
  const bool rowin = Y >= 0 && Y < a.N0;
  if (vec) {
#pragma unroll 4
    for (int x = 4 * threadIdx.x; x < a.N; x += 4 * blockDim.x) {
      const int X = x - a.off;
      const float4 v = (rowin && X >= 0 && X < a.N0) ? __ldg(reinterpret_cast<const float4*>(src + X))
                                                      : make_float4(0.f, 0.f, 0.f, 0.f);
      *reinterpret_cast<float4*>(line + x) = v;
    }
  } else {
    for (int x = threadIdx.x; x < a.N; x += blockDim.x) {
      const int X = x - a.off;
      line[lpos(x, C)] = (rowin && X >= 0 && X < a.N0) ? __ldg(src + X) : 0.f;
    }
  }
  __syncthreads();
  if (a.cubic) prefilter_line(line, cp, a.N, threadIdx.x, blockDim.x);
  if (vec) {
#pragma unroll 4
    for (int x = 4 * threadIdx.x; x < a.N; x += 4 * blockDim.x)
      *reinterpret_cast<float4*>(dst + x) = *reinterpret_cast<const float4*>(line + x);
  } else {
    for (int x = threadIdx.x; x < a.N; x += blockDim.x) dst[x] = line[lpos(x, C)];
  }
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
    // groups of 8: the loads of a group are issued before its recursion steps
    for (; n + 8 <= e; n += 8) {
      float xv[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) xv[i] = col[(size_t)(n + i) * W];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        prev = LP_LAMBDA * xv[i] + z * prev;
        col[(size_t)(n + i) * W] = prev;
      }
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
    const cudaSurfaceObject_t so = a.surf ? a.surf[s] : 0;
    if (e + nw >= H) {
      // exact anticausal initialisation at H-1 (static indices only, so wu stays in registers)
      float last = 0.f;
#pragma unroll
      for (int i = 0; i < LP_WARM; ++i)
        if (i == nw - 1) last = wu[i];
      if (nw == 0) last = col[(size_t)(H - 1) * W];
      c = (z / (z - 1.0f)) * last;
      if (nw == 0) {
        if (a.surf) surf2Dwrite(c, so, x * (int)sizeof(float), H - 1);
        else col[(size_t)(H - 1) * W] = c;
        n = H - 2;
      } else {
#pragma unroll
        for (int i = LP_WARM - 2; i >= 0; --i)
          if (i <= nw - 2) c = z * (c - wu[i]);
        n = e - 1;
      }
    } else {
      c = -z * wu[LP_WARM - 1];
      for (int i = LP_WARM - 2; i >= 0; --i) c = z * (c - wu[i]);
      n = e - 1;
    }
    for (; n - 8 >= b - 1; n -= 8) {
      float xv[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) xv[i] = col[(size_t)(n - i) * W];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        c = z * (c - xv[i]);
        if (a.surf) surf2Dwrite(c, so, x * (int)sizeof(float), n - i);
        else col[(size_t)(n - i) * W] = c;
      }
    }
    for (; n >= b; --n) {
      c = z * (c - col[(size_t)n * W]);
      if (a.surf) surf2Dwrite(c, so, x * (int)sizeof(float), n);
      else col[(size_t)n * W] = c;
    }
  }
}

// ---------------------------------------------------------------------------
// prefilter along the slow axis, out of place (final coefficients to the
// per-slice surfaces or to a separate array): one warp per 32 columns x kColC rows.  The warp copies
// its rows plus LP_WARM rows on either side into shared memory with
// asynchronous copies (all of them in flight at once), runs both recursions
// there -- the same zero-state warm-ups and boundary initialisations as
// k_col_prefilter -- and writes each coefficient once.  The input is only
// read, so warps need no ordering between them.
// ---------------------------------------------------------------------------
constexpr int kColC = 64;                          // output rows per warp
constexpr int kColRows = kColC + 2 * LP_WARM;      // rows staged per warp
constexpr int kColWarps = 4;                       // 4 x 96 x 32 floats = 48 KB per block


__global__ void __launch_bounds__(32 * kColWarps) k_col_prefilter_staged(ColPrefilterArgs a) {
  __shared__ float tile[kColWarps][kColRows][32];
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int H = a.H, W = a.W;
  const int b = (blockIdx.y * kColWarps + wp) * kColC;
  if (b >= H) return;  // warps are independent: no block-wide barrier below
  const int e = min(b + kColC, H);
  const int r0 = max(0, b - LP_WARM), r1 = min(H, e + LP_WARM);
  const int x = blockIdx.x * 32 + lane;
  const int s = blockIdx.z;
  const bool inx = x < W;
  float(*t)[32] = tile[wp];
  const float* col = a.img + (size_t)s * H * W + x;
  for (int r = r0; r < r1; ++r) {
    if (inx) cp_async4(&t[r - r0][lane], col + (size_t)r * W);
    else t[r - r0][lane] = 0.f;
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncwarp();
  const float z = LP_POLE;
  // causal: exact initialisation at row 0, else LP_WARM warm-up rows from a zero state
  float prev = 0.f;
  int n;
  if (b == 0) {
    const int hor = min(12, H);
    float sum = t[0][lane];
    float zn = z;
    for (int i = 0; i < hor; ++i) {
      sum += zn * t[i][lane];
      zn *= z;
    }
    prev = LP_LAMBDA * sum;
    t[0][lane] = prev;
    n = 1;
  } else {
#pragma unroll
    for (int i = 0; i < LP_WARM; ++i) prev = LP_LAMBDA * t[i][lane] + z * prev;
    n = b;
  }
  for (; n < r1; ++n) {
    prev = LP_LAMBDA * t[n - r0][lane] + z * prev;
    t[n - r0][lane] = prev;
  }
  // anticausal: exact initialisation at row H-1 when it is within reach, else a
  // zero state LP_WARM rows past the chunk
  const cudaSurfaceObject_t so = a.surf ? a.surf[s] : 0;
  float* dst = a.out + (size_t)s * H * W + x;
  auto put = [&](int row, float v) {
    if (a.surf) surf2Dwrite(v, so, x * (int)sizeof(float), row);
    else dst[(size_t)row * W] = v;
  };
  float c;
  if (r1 == H && H - e <= LP_WARM) {
    c = (z / (z - 1.0f)) * t[H - 1 - r0][lane];
    if (e == H && inx) put(H - 1, c);
    n = H - 2;
  } else {
    c = -z * t[r1 - 1 - r0][lane];
    n = r1 - 2;
  }
  for (; n >= b; --n) {
    c = z * (c - t[n - r0][lane]);
    if (n < e && inx) put(n, c);
  }
}

// ---------------------------------------------------------------------------
// forward, per span: gather Cartesian -> log-polar for two theta columns,
// multiply by e^rho, FFT along rho (two real columns in one complex FFT).
// Reference: interp mode 3 (lpRgpu.cu:263), mulexp (:267), R2C (:270).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256, 4) k_fwd_c2lp(FwdC2LPArgs a) {
  extern __shared__ float smf[];
  CBuf A, B;
  carve(smf, a.Nrho, 1, A, B);
  const int s = blockIdx.x;
  const int th = 2 * blockIdx.y;
  const int thb = th + 1 < a.Nth ? th + 1 : -1;
  const float* img = a.fbuf + (size_t)s * a.N * a.N;
  const int2* ca = a.c2lp + (size_t)th * a.Nrho;
  const int2* cb = a.c2lp + (size_t)max(thb, 0) * a.Nrho;
  const bool use_tex = a.tex != nullptr;
  const cudaTextureObject_t tx = use_tex ? a.tex[s] : 0;
  const float invN = 1.0f / (float)a.N;
  for (int r = threadIdx.x; r < a.Nrho; r += blockDim.x) {
    const float e = __ldg(a.erho + r);
    const int2 pa = __ldg(ca + r);
    float va = 0.f, vb = 0.f;
    if (pa.x != LP_FX_NONE)
      va = e * (use_tex ? interp_tex_cubic_fx(tx, invN, invN, pa.x, pa.y, a.F, a.fsc)
                        : interp2d_fx(img, a.N, a.N, pa.x, pa.y, a.F, a.fsc, a.cubic));
    if (thb >= 0) {
      const int2 pb = __ldg(cb + r);
      if (pb.x != LP_FX_NONE)
        vb = e * (use_tex ? interp_tex_cubic_fx(tx, invN, invN, pb.x, pb.y, a.F, a.fsc)
                          : interp2d_fx(img, a.N, a.N, pb.x, pb.y, a.F, a.fsc, a.cubic));
    }
    A.set(r, make_float2(va, vb));
  }
  __syncthreads();
  const CBuf Z = fft_block<-1>(A, B, a.plan, 1, 0);
  float2* out = a.spec + (size_t)s * spec_slice(a.Nk, a.Nth);
  for (int k = threadIdx.x; k < a.Nk; k += blockDim.x) {
    const float2 z1 = Z.get(k);
    const float2 z2 = Z.get(k == 0 ? 0 : a.Nrho - k);
    out[sidx(k, th, a.Nth)] = make_float2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
    if (thb >= 0) out[sidx(k, thb, a.Nth)] = make_float2(0.5f * (z1.y + z2.y), 0.5f * (z2.x - z1.x));
  }
}

// ---------------------------------------------------------------------------
// per rho frequency: FFT along theta, multiply by fZ/(Nrho*Ntheta), inverse.
// Reference: the theta half of cuFFT's 2-D R2C/C2R and `mul`
// (lpRgpu.cu:270-277, simple_kernels.cuh:2-12).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256, 4) k_theta_conv(ThetaConvArgs a) {
  extern __shared__ float smf[];
  CBuf A, B;
  carve(smf, a.Nth, 2, A, B);
  const int s = blockIdx.x;
  const int k0 = 2 * blockIdx.y;
  const int nrow = (k0 + 1 < a.Nk) ? 2 : 1;
  float2* sp = a.spec + (size_t)s * spec_slice(a.Nk, a.Nth);
  const int ps = fft_plane_floats(a.Nth);  // plane stride between the two rows
  // rows k0, k0 + 1 (k0 even) are adjacent in the tiled layout: neighbouring threads
  // take the two rows of one column, so global accesses cover 16 of every 32 bytes
  for (int i = threadIdx.x; i < 2 * a.Nth; i += blockDim.x) {
    const int r = i & 1, t = i >> 1;
    const bool in = r < nrow && t >= a.in_lo && t <= a.in_hi;
    A.offset(r * ps).set(t, in ? sp[sidx(k0 + r, t, a.Nth)] : make_float2(0.f, 0.f));
  }
  __syncthreads();
  const CBuf X = fft_block<-1>(A, B, a.plan, 2, ps);
  for (int i = threadIdx.x; i < 2 * a.Nth; i += blockDim.x) {
    const int r = i & 1, t = i >> 1;
    if (r >= nrow) continue;
    float2 w = __ldg(a.fz + sidx(k0 + r, t, a.Nth));
    if (a.conj_fz) w.y = -w.y;
    const CBuf Xr = X.offset(r * ps);
    Xr.set(t, cmul(Xr.get(t), w));
  }
  __syncthreads();
  const CBuf Y = fft_block<1>(X, X.re == A.re ? B : A, a.plan, 2, ps);
  const int w = a.out_hi - a.out_lo + 1;
  for (int i = threadIdx.x; i < 2 * w; i += blockDim.x) {
    const int r = i & 1, t = a.out_lo + (i >> 1);
    if (r < nrow) sp[sidx(k0 + r, t, a.Nth)] = Y.offset(r * ps).get(t);
  }
}

// ---------------------------------------------------------------------------
// forward, per span: two polar angle rows per block.  Each row's theta taps
// are combined in the frequency domain, one inverse FFT along rho gives both
// rows' rho profiles, then the rho interpolation at every s.  Writes straight
// into the caller's sinogram (stepangles + cor window, lpRgpu.cu:191-192).
// Reference: C2R (:277), interp mode 5 (:284).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256, 4) k_fwd_lp2polar(FwdLP2PolarArgs a) {
  extern __shared__ float smf[];
  CBuf A, B;
  carve(smf, a.Nrho, 1, A, B);
  const int s = blockIdx.x;
  const int i0 = 2 * blockIdx.y;
  const int r0 = a.rows[i0];
  const int r1 = (i0 + 1 < a.nrows) ? a.rows[i0 + 1] : -1;
  float w0[4], w1[4];
  const int c0 = axis_weights_fx(__ldg(a.thc + r0), a.F, a.fsc, a.cubic, w0);
  int c1 = 0;
  if (r1 >= 0) {
    c1 = axis_weights_fx(__ldg(a.thc + r1), a.F, a.fsc, a.cubic, w1);
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
  const float2* sp = a.spec + (size_t)s * spec_slice(a.Nk, a.Nth);
  for (int k = threadIdx.x; k < a.Nk; k += blockDim.x) {
    float2 v0 = make_float2(0.f, 0.f), v1 = make_float2(0.f, 0.f);
    for (int j = 0; j < ntap; ++j) {
      const float2 q0 = sp[sidx(k, t0[j], a.Nth)];
      v0.x += w0[j] * q0.x;
      v0.y += w0[j] * q0.y;
      if (r1 >= 0) {
        const float2 q1 = sp[sidx(k, t1[j], a.Nth)];
        v1.x += w1[j] * q1.x;
        v1.y += w1[j] * q1.y;
      }
    }
    put_pair(A, k, a.Nrho, v0, v1);
  }
  __syncthreads();
  const CBuf zr = fft_block<1>(A, B, a.plan, 1, 0);
  const int Nrho = a.Nrho;
  for (int x = threadIdx.x; x < a.N; x += blockDim.x) {
    const int xo = x - a.cor_off;
    if (xo < 0 || xo >= a.N0) continue;
    if (r0 % a.os == 0) {
      const int t = __ldg(a.rhoc + (size_t)r0 * a.N + x);
      const float v = interp1d_fx([&](int i) { return zr.re[fpad(i)]; }, Nrho, t, a.F, a.fsc, a.cubic);
      a.Rout[((size_t)s * a.Nproj0 + r0 / a.os) * a.N0 + xo] = v;
    }
    if (r1 >= 0 && r1 % a.os == 0) {
      const int t = __ldg(a.rhoc + (size_t)r1 * a.N + x);
      const float v = interp1d_fx([&](int i) { return zr.im[fpad(i)]; }, Nrho, t, a.F, a.fsc, a.cubic);
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
__global__ void __launch_bounds__(256, 4) k_adj_ingest(AdjIngestArgs a) {
  extern __shared__ float smf[];
  const int N = a.N;
  const int M = 2 * N;  // the filter couples samples less than N apart: a 2N circular convolution is exact
  const bool filt = a.H != nullptr;
  CBuf F0, F1;
  float* lines = filt ? carve(smf, M, 1, F0, F1) : smf;  // 2 rows, chunked layout
  const int half = blockDim.x / 2;
  const int C = line_chunk(N, half);
  const int LF = line_floats(N, half);
  float* cp = lines + 2 * LF;                            // 2 rows of scratch
  const int s = blockIdx.x;
  const int q0 = 2 * blockIdx.y;
  const int q1 = q0 + 1 < a.Nproj0 ? q0 + 1 : -1;
  const float* in0 = a.Rin + ((size_t)s * a.Nproj0 + q0) * a.N0;
  const float* in1 = a.Rin + ((size_t)s * a.Nproj0 + max(q1, 0)) * a.N0;
  for (int x = threadIdx.x; x < N; x += blockDim.x) {
    const int xi = min(max(x - a.cor_off, 0), a.N0 - 1);
    lines[lpos(x, C)] = __ldg(in0 + xi);
    lines[LF + lpos(x, C)] = q1 >= 0 ? __ldg(in1 + xi) : 0.f;
  }
  __syncthreads();
  if (filt) {
    for (int x = threadIdx.x; x < M; x += blockDim.x)
      F0.set(x, x < N ? make_float2(lines[lpos(x, C)], lines[LF + lpos(x, C)]) : make_float2(0.f, 0.f));
    __syncthreads();
    const CBuf X = fft_block<-1>(F0, F1, a.plan, 1, 0);
    for (int k = threadIdx.x; k < M; k += blockDim.x) X.set(k, cscale(X.get(k), __ldg(a.H + k)));
    __syncthreads();
    const CBuf Y = fft_block<1>(X, X.re == F0.re ? F1 : F0, a.plan, 1, 0);
    for (int x = threadIdx.x; x < N; x += blockDim.x) {
      const float2 y = Y.get(x);
      lines[lpos(x, C)] = y.x;
      lines[LF + lpos(x, C)] = y.y;
    }
    __syncthreads();
  }
  if (a.cubic) {
    // two lines at once: half of the block each
    const int which = threadIdx.x >= half;
    const int tid = threadIdx.x - which * half;
    // prefilter_line synchronises the whole block; both halves call it together
    prefilter_line(lines + which * LF, cp + which * LF, N, tid, half);
  }
  for (int rr = 0; rr < 2; ++rr) {
    const int q = rr == 0 ? q0 : q1;
    if (q < 0) break;
    for (int j = 0; j < a.os; ++j) {
      float* dst = a.rbuf + ((size_t)s * a.Nproj + (size_t)q * a.os + j) * N;
      for (int x = threadIdx.x; x < N; x += blockDim.x) dst[x] = j == 0 ? lines[rr * LF + lpos(x, C)] : 0.f;
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
__global__ void __launch_bounds__(256, 4) k_adj_polar2lp(AdjPolar2LPArgs a) {
  extern __shared__ float smf[];
  CBuf A, B;
  float* prof = carve(smf, a.Nrho, 1, A, B);  // 2 x N
  const int s = blockIdx.x;
  const int th0 = a.clo + 2 * blockIdx.y;
  const int th1 = th0 + 1 <= a.chi ? th0 + 1 : -1;
  const float* img = a.rbuf + (size_t)s * a.Nproj * a.N;
  const int ta0 = __ldg(a.ta + th0);
  const int ta1 = th1 >= 0 ? __ldg(a.ta + th1) : LP_FX_NONE;
  float w0[4], w1[4];
  int rw0[4], rw1[4];
  const bool has0 = ta0 != LP_FX_NONE, has1 = ta1 != LP_FX_NONE;
  const int ntap = a.cubic ? 4 : 2;
  {
    const int c0 = has0 ? axis_weights_fx(ta0, a.F, a.fsc, a.cubic, w0) : 0;
    const int c1 = has1 ? axis_weights_fx(ta1, a.F, a.fsc, a.cubic, w1) : 0;
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
  const int* sx0 = a.sx + (size_t)th0 * a.Nrho;
  const int* sx1 = a.sx + (size_t)max(th1, 0) * a.Nrho;
  for (int r = threadIdx.x; r < a.Nrho; r += blockDim.x) {
    float v0 = 0.f, v1 = 0.f;
    const int x0 = __ldg(sx0 + r);
    if (x0 != LP_FX_NONE) v0 = interp1d_fx([&](int i) { return prof[i]; }, a.N, x0, a.F, a.fsc, a.cubic);
    if (th1 >= 0) {
      const int x1 = __ldg(sx1 + r);
      if (x1 != LP_FX_NONE) v1 = interp1d_fx([&](int i) { return prof[a.N + i]; }, a.N, x1, a.F, a.fsc, a.cubic);
    }
    A.set(r, make_float2(v0, v1));
  }
  __syncthreads();
  // wrap points (distinct rho within a column)
  for (int c = 0; c < 2; ++c) {
    const int th = c == 0 ? th0 : th1;
    if (th < 0) break;
    const int w_begin = __ldg(a.woff + th), w_end = __ldg(a.woff + th + 1);
    for (int w = w_begin + threadIdx.x; w < w_end; w += blockDim.x) {
      const int4 p = __ldg(a.wpt + w);
      const int r = p.x;
      const float v = interp2d_fx(img, a.N, a.Nproj, p.y, p.z, a.F, a.fsc, a.cubic);
      if (c == 0) A.re[fpad(r)] += v;
      else A.im[fpad(r)] += v;
    }
    __syncthreads();
  }
  const CBuf Z = fft_block<-1>(A, B, a.plan, 1, 0);
  float2* out = a.spec + (size_t)s * spec_slice(a.Nk, a.Nth);
  for (int k = threadIdx.x; k < a.Nk; k += blockDim.x) {
    const float2 z1 = Z.get(k);
    const float2 z2 = Z.get(k == 0 ? 0 : a.Nrho - k);
    out[sidx(k, th0, a.Nth)] = make_float2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
    if (th1 >= 0) out[sidx(k, th1, a.Nth)] = make_float2(0.5f * (z1.y + z2.y), 0.5f * (z2.x - z1.x));
  }
}

// ---------------------------------------------------------------------------
// adjoint, per span: inverse FFT along rho for two theta columns, store the
// real log-polar columns [theta][rho] for the Cartesian gather (C2R :321).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256, 4) k_adj_lpcols(AdjLPColsArgs a) {
  extern __shared__ float smf[];
  CBuf A, B;
  carve(smf, a.Nrho, 1, A, B);
  const int s = blockIdx.x;
  const int th0 = a.lo2 + 2 * blockIdx.y;
  const int th1 = th0 + 1 <= a.hi2 ? th0 + 1 : -1;
  const float2* sp = a.spec + (size_t)s * spec_slice(a.Nk, a.Nth);
  for (int k = threadIdx.x; k < a.Nk; k += blockDim.x) {
    const float2 v0 = sp[sidx(k, th0, a.Nth)];
    const float2 v1 = th1 >= 0 ? sp[sidx(k, th1, a.Nth)] : make_float2(0.f, 0.f);
    put_pair(A, k, a.Nrho, v0, v1);
  }
  __syncthreads();
  const CBuf z = fft_block<1>(A, B, a.plan, 1, 0);
  float* g0 = a.G + ((size_t)s * a.W2 + (th0 - a.lo2)) * a.Nrho;
  for (int r = threadIdx.x; r < a.Nrho; r += blockDim.x) {
    const float2 v = z.get(r);
    if (a.surf) {
      surf2Dwrite(v.x, a.surf[s], r * (int)sizeof(float), th0 - a.lo2);
      if (th1 >= 0) surf2Dwrite(v.y, a.surf[s], r * (int)sizeof(float), th1 - a.lo2);
    } else {
      g0[r] = v.x;
      if (th1 >= 0) g0[a.Nrho + r] = v.y;
    }
  }
}

// ---------------------------------------------------------------------------
// adjoint: log-polar -> Cartesian gather summed over the three spans, written
// straight into the caller's N0 x N0 window (interp mode 5, lpRgpu.cu:328,
// copy3Dshifted :206).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float interp_cols(const float* __restrict__ G, int Nrho, int Nth, int lo2, int W2,
                                             int2 t, int F, float fsc, int cubic) {
  float wt[4], wr[4];
  const int ct = axis_weights_fx(t.x, F, fsc, cubic, wt);
  const int cr = axis_weights_fx(t.y, F, fsc, cubic, wr);
  const int nt = cubic ? 4 : 2;
  int rr[4];
  const bool inner = (cr >= 0 && cr + 3 < Nrho);
#pragma unroll
  for (int i = 0; i < 4; ++i) rr[i] = inner ? cr + i : wrapi(cr + i, Nrho);
  const bool tin = ct >= 0 && ct + 3 < Nth;
  float acc = 0.f;
  for (int j = 0; j < nt; ++j) {
    const int col = (tin ? ct + j : wrapi(ct + j, Nth)) - lo2;
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

// 8 resident blocks per SM (32 registers): the texture return path is the limit and more
// warps keep it busier (measured 8.3 ms per step at N=2048 against 8.9 with 5 blocks)
__global__ void __launch_bounds__(256, 8) k_adj_lp2cart(AdjLP2CartArgs a) {
  const int s = blockIdx.x;
  const int p = (blockIdx.z * gridDim.y + blockIdx.y) * blockDim.x + threadIdx.x;
  if (p >= a.npix) return;
  const size_t gs = (size_t)s * a.W2 * a.Nrho;
  float acc = 0.f;
  const int2 t0 = __ldg(a.c2lp0 + p);
  if (a.tex0) {
    // texture x = rho (wrap over Nrho), y = theta - lo2 (taps stay inside the stored band).
    // Straight-line: the three spans' twelve gathers are in flight together; pixels
    // outside the disk sample (0, 0) and are discarded, warps entirely outside skip.
    const bool ok = t0.x != LP_FX_NONE;
    if (__any_sync(__activemask(), ok)) {
      const float iw = 1.0f / (float)a.Nrho, ih = 1.0f / (float)a.W2;
      const int l2 = a.lo2 << a.F;
      const int2 t1 = __ldg(a.c2lp1 + p), t2 = __ldg(a.c2lp2 + p);
      const int2 q0 = ok ? make_int2(t0.y, t0.x - l2) : make_int2(0, 0);
      const int2 q1 = ok ? make_int2(t1.y, t1.x - l2) : make_int2(0, 0);
      const int2 q2 = ok ? make_int2(t2.y, t2.x - l2) : make_int2(0, 0);
      const float v = interp_tex_cubic_fx(a.tex0[s], iw, ih, q0.x, q0.y, a.F, a.fsc) +
                      interp_tex_cubic_fx(a.tex1[s], iw, ih, q1.x, q1.y, a.F, a.fsc) +
                      interp_tex_cubic_fx(a.tex2[s], iw, ih, q2.x, q2.y, a.F, a.fsc);
      acc = ok ? v : 0.f;
    }
    a.fout[(size_t)s * a.npix + p] = acc;
    return;
  }
  if (t0.x != LP_FX_NONE) {
    acc += interp_cols(a.G0 + gs, a.Nrho, a.Nth, a.lo2, a.W2, t0, a.F, a.fsc, a.cubic);
    acc += interp_cols(a.G1 + gs, a.Nrho, a.Nth, a.lo2, a.W2, __ldg(a.c2lp1 + p), a.F, a.fsc, a.cubic);
    acc += interp_cols(a.G2 + gs, a.Nrho, a.Nth, a.lo2, a.W2, __ldg(a.c2lp2 + p), a.F, a.fsc, a.cubic);
  }
  a.fout[(size_t)s * a.npix + p] = acc;
}

// ---------------------------------------------------------------------------
// launches
// ---------------------------------------------------------------------------
static const int kFFTThreads = 256;

static size_t fft_bytes(int L, int nfft) { return 4 * (size_t)nfft * fft_plane_floats(L) * sizeof(float); }
static size_t smem_c2lp(int Nrho) { return fft_bytes(Nrho, 1); }
static size_t smem_theta(int Nth) { return fft_bytes(Nth, 2); }
static size_t smem_adj_ingest(int N, bool filt) {
  return (filt ? fft_bytes(2 * N, 1) : 0) + 4 * (size_t)line_floats(N, 128) * sizeof(float);
}
static size_t smem_polar2lp(int Nrho, int N) { return fft_bytes(Nrho, 1) + 2 * (size_t)N * sizeof(float); }

static int g_smem_optin = 48 * 1024;
static cudaError_t smem_ok(size_t need);
bool smem_fits(size_t need) { return smem_ok(need) == cudaSuccess; }
// the register-FFT kernels: powers of two here, mixed lengths in lp_kernels_mr.cu
using Pow2Lengths = Lengths<256, 512, 1024, 2048, 4096, 8192>;
LP_DEFINE_LENGTH_SET(p2, Pow2Lengths)
// generic (any N) kernels are used when g_use_p2 is false or no register-FFT length fits
static bool g_use_p2 = true;
// the register-FFT launcher of FN for the length, from whichever length list holds it
#define LP_REGISTER_FFT(FN, A, S, ST, PE)                                                   \
  (g_use_p2 && (p2_##FN(A, S, ST, PE) || mr_##FN(A, S, ST, PE) || mr2_##FN(A, S, ST, PE) || \
                mr3_##FN(A, S, ST, PE) || mr4_##FN(A, S, ST, PE) || mr5_##FN(A, S, ST, PE)))

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
  e = p2_configure(optin);
  if (e == cudaSuccess) e = mr_configure(optin);
  if (e == cudaSuccess) e = mr2_configure(optin);
  if (e == cudaSuccess) e = mr3_configure(optin);
  if (e == cudaSuccess) e = mr4_configure(optin);
  return e == cudaSuccess ? mr5_configure(optin) : e;
}

void set_use_p2(bool on) { g_use_p2 = on; }

static cudaError_t smem_ok(size_t need) {
  return need <= (size_t)g_smem_optin ? cudaSuccess : cudaErrorInvalidConfiguration;
}

cudaError_t launch_fwd_ingest(const FwdIngestArgs& a, int S, cudaStream_t st) {
  const size_t sm = 2 * (size_t)line_floats(a.N, 128) * sizeof(float);
  if (smem_ok(sm) != cudaSuccess) return cudaErrorInvalidConfiguration;
  dim3 grid(S, a.N);
  k_fwd_ingest<<<grid, 128, sm, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_col_prefilter(const ColPrefilterArgs& a, int S, cudaStream_t st) {
  if (a.surf || a.out) {
    const int chunks = (a.H + kColC - 1) / kColC;
    dim3 grid((a.W + 31) / 32, (chunks + kColWarps - 1) / kColWarps, S);
    k_col_prefilter_staged<<<grid, 32 * kColWarps, 0, st>>>(a);
    return cudaGetLastError();
  }
  int nch = a.H / LP_WARM;
  if (nch > 32) nch = 32;
  if (nch < 1) nch = 1;
  dim3 block(32, nch);
  dim3 grid((a.W + 31) / 32, S);
  k_col_prefilter<<<grid, block, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_fwd_c2lp(const FwdC2LPArgs& a, int S, cudaStream_t st) {
  cudaError_t pe;
  if (LP_REGISTER_FFT(fwd_c2lp, a, S, st, &pe)) return pe;
  if (smem_ok(smem_c2lp(a.Nrho)) != cudaSuccess) return cudaErrorInvalidConfiguration;
  dim3 grid(S, (a.Nth + 1) / 2);
  k_fwd_c2lp<<<grid, kFFTThreads, smem_c2lp(a.Nrho), st>>>(a);
  return cudaGetLastError();
}

bool theta_conv_gathers(int Nth, int nrows) {
  if (!g_use_p2) return false;
  const size_t need = p2_has_length(Nth)    ? p2_gather_smem(Nth, nrows)
                      : mr_has_length(Nth)  ? mr_gather_smem(Nth, nrows)
                      : mr2_has_length(Nth) ? mr2_gather_smem(Nth, nrows)
                      : mr3_has_length(Nth) ? mr3_gather_smem(Nth, nrows)
                      : mr4_has_length(Nth) ? mr4_gather_smem(Nth, nrows)
                                            : mr5_gather_smem(Nth, nrows);
  return need > 0 && smem_fits(need);
}

cudaError_t launch_theta_conv(const ThetaConvArgs& a, int S, cudaStream_t st) {
  cudaError_t pe;
  if (LP_REGISTER_FFT(theta_conv, a, S, st, &pe)) return pe;
  if (a.rowspec) return cudaErrorNotSupported;  // the gathered input needs a register-FFT length
  if (smem_ok(smem_theta(a.Nth)) != cudaSuccess) return cudaErrorInvalidConfiguration;
  dim3 grid(S, (a.Nk + 1) / 2);
  k_theta_conv<<<grid, kFFTThreads, smem_theta(a.Nth), st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_fwd_lp2polar(const FwdLP2PolarArgs& a, int S, cudaStream_t st) {
  cudaError_t pe;
  if (LP_REGISTER_FFT(fwd_lp2polar, a, S, st, &pe)) return pe;
  if (a.nrows <= 0) return cudaSuccess;
  if (smem_ok(smem_c2lp(a.Nrho)) != cudaSuccess) return cudaErrorInvalidConfiguration;
  dim3 grid(S, (a.nrows + 1) / 2);
  k_fwd_lp2polar<<<grid, kFFTThreads, smem_c2lp(a.Nrho), st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_adj_ingest(const AdjIngestArgs& a, int S, cudaStream_t st) {
  cudaError_t pe;
  if (LP_REGISTER_FFT(adj_ingest, a, S, st, &pe)) return pe;
  if (smem_ok(smem_adj_ingest(a.N, a.H != nullptr)) != cudaSuccess) return cudaErrorInvalidConfiguration;
  dim3 grid(S, (a.Nproj0 + 1) / 2);
  k_adj_ingest<<<grid, kFFTThreads, smem_adj_ingest(a.N, a.H != nullptr), st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_adj_polar2lp(const AdjPolar2LPArgs& a, int S, cudaStream_t st) {
  cudaError_t pe;
  if (LP_REGISTER_FFT(adj_polar2lp, a, S, st, &pe)) return pe;
  if (a.chi < a.clo) return cudaSuccess;
  if (smem_ok(smem_polar2lp(a.Nrho, a.N)) != cudaSuccess) return cudaErrorInvalidConfiguration;
  dim3 grid(S, (a.chi - a.clo + 2) / 2);
  k_adj_polar2lp<<<grid, kFFTThreads, smem_polar2lp(a.Nrho, a.N), st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_adj_lpcols(const AdjLPColsArgs& a, int S, cudaStream_t st) {
  cudaError_t pe;
  if (LP_REGISTER_FFT(adj_lpcols, a, S, st, &pe)) return pe;
  if (smem_ok(smem_c2lp(a.Nrho)) != cudaSuccess) return cudaErrorInvalidConfiguration;
  dim3 grid(S, (a.hi2 - a.lo2 + 2) / 2);
  k_adj_lpcols<<<grid, kFFTThreads, smem_c2lp(a.Nrho), st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_adj_lp2cart(const AdjLP2CartArgs& a, int S, cudaStream_t st) {
  // pixel blocks over y and z (grid.y stops at 65535: N0 = 4096 has 65536 blocks of 256)
  const int nb = (a.npix + 255) / 256;
  dim3 grid(S, nb < 65535 ? nb : 65535, (nb + 65534) / 65535);
  k_adj_lp2cart<<<grid, 256, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace lpgb

// ===========================================================================
// Power-of-two sizes (N = 256 .. 4096): the same kernels on the register FFT
// of fft_reg.cuh.  A signal is transformed by T = L/16 threads; blocks of 256
// threads carry 256/T signals when L < 4096.
// ===========================================================================
namespace lpgb {

}  // namespace lpgb

// ===========================================================================
// Exact transpose of the forward operator (gradient of <fwd(f), g> in f).
// Stage by stage: transposed rho interpolation of every sinogram row, the
// transpose of C2R (a_k * R2C), the theta-tap combination scattered back to
// the columns, the theta convolution with conj(fZ), the transpose of R2C
// (C2R of b_k * Y), e^rho, the transposed Cartesian interpolation (scatter),
// and the transposed prefilter recursions.
// ===========================================================================
namespace lpgb {

// Rows: per pair of internal rows of a span, the transposed rho interpolation, one
// complex FFT along rho and the split into the two rows' half spectra (the
// transpose of the forward's C2R), written to the row-spectrum buffer.  The
// power-of-two and mixed lengths run k_fwdT_rows_p2 on the register FFT.
__global__ void __launch_bounds__(256) k_fwdT_rows(FwdTRowsArgs a) {
  extern __shared__ float smf[];
  CBuf A, B;
  float* u = carve(smf, a.Nrho, 1, A, B);  // 2 x Nrho transposed-interpolation accumulators
  const int s = blockIdx.x;
  const int i0 = 2 * blockIdx.y;
  const int r0 = a.rows[i0];
  const int r1 = i0 + 1 < a.nrows ? a.rows[i0 + 1] : -1;
  const int L = a.Nrho;
  for (int i = threadIdx.x; i < 2 * L; i += blockDim.x) u[i] = 0.f;
  __syncthreads();
  rho_scatter_T(a, s, r0, r1, threadIdx.x, blockDim.x, [&](int q, int bin) -> float& { return u[q * L + bin]; });
  for (int i = threadIdx.x; i < L; i += blockDim.x) A.set(i, make_float2(u[i], u[L + i]));
  __syncthreads();
  const CBuf Z = fft_block<-1>(A, B, a.plan, 1, 0);
  float2* o0 = a.rowspec + ((size_t)s * a.nrows + i0) * rowspec_stride(a.Nk);
  for (int k = threadIdx.x; k < a.Nk; k += blockDim.x) {
    float2 va, vb;
    split_rows_T(Z.get(k), Z.get(k == 0 ? 0 : L - k), k, L, &va, &vb);
    o0[k] = va;
    if (r1 >= 0) o0[rowspec_stride(a.Nk) + k] = vb;
  }
}

// Columns: per block of CW spectrum columns from lo, every rho frequency sums the
// half spectra of the rows whose theta taps reach the column, times the tap
// weight, in row order (no atomics: the same bits on every run).  Writes every
// column of [lo, hi], zero where no row reaches it.
constexpr int kColSumCW = 8;

__global__ void __launch_bounds__(256) k_fwdT_colsum(FwdTColSumArgs a) {
  const int s = blockIdx.x;
  const int c0 = a.lo + blockIdx.y * kColSumCW;
  const int2 rr = __ldg(a.blk + blockIdx.y);
  const int ntap = a.cubic ? 4 : 2;
  const float2* rs = a.rowspec + (size_t)s * a.nrows * rowspec_stride(a.Nk);
  float2* sp = a.spec + (size_t)s * spec_slice(a.Nk, a.Nth);
  for (int k = threadIdx.x; k < a.Nk; k += blockDim.x) {
    float2 acc[kColSumCW];
#pragma unroll
    for (int c = 0; c < kColSumCW; ++c) acc[c] = make_float2(0.f, 0.f);
    for (int i = rr.x; i < rr.y; ++i) {
      float w[4];
      const int t0 = axis_weights_fx(__ldg(a.thc + __ldg(a.rows + i)), a.F, a.fsc, a.cubic, w);
      const float2 z = __ldg(rs + (size_t)i * rowspec_stride(a.Nk) + k);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (j >= ntap) break;
        const int c = wrapi(t0 + j, a.Nth) - c0;
#pragma unroll
        for (int cc = 0; cc < kColSumCW; ++cc)
          if (c == cc) {
            acc[cc].x += w[j] * z.x;
            acc[cc].y += w[j] * z.y;
          }
      }
    }
#pragma unroll
    for (int cc = 0; cc < kColSumCW; ++cc)
      if (c0 + cc <= a.hi) sp[sidx(k, c0 + cc, a.Nth)] = acc[cc];
  }
}

// Transpose of the column stage of the forward: per pair of disk columns, the
// transposes of R2C (C2R of b_k * Y, b_k = 1/2 except at k = 0 and Nrho/2) and of
// the e^rho multiply, written slice-interleaved as real log-polar values for the
// gather below.
__global__ void __launch_bounds__(256) k_fwdT_cols(FwdTColsArgs a) {
  extern __shared__ float smf[];
  CBuf A, B;
  carve(smf, a.Nrho, 1, A, B);
  const int s = blockIdx.x;
  const int th0 = a.dlo + 2 * blockIdx.y;
  const int th1 = th0 + 1 <= a.dhi ? th0 + 1 : -1;
  const float2* sp = a.spec + (size_t)s * spec_slice(a.Nk, a.Nth);
  const int L = a.Nrho;
  for (int k = threadIdx.x; k < a.Nk; k += blockDim.x) {
    const float bk = (k == 0 || k == L / 2) ? 1.f : 0.5f;
    const float2 v0 = cscale(sp[sidx(k, th0, a.Nth)], bk);
    const float2 v1 = th1 >= 0 ? cscale(sp[sidx(k, th1, a.Nth)], bk) : make_float2(0.f, 0.f);
    put_pair(A, k, L, v0, v1);
  }
  __syncthreads();
  const CBuf z = fft_block<1>(A, B, a.plan, 1, 0);
  float* g0 = a.G + (size_t)(s / kGatherSlices) * a.npts * kGatherSlices + s % kGatherSlices;
  const int* pos = a.pos + (size_t)(th0 - a.dlo) * L;
  for (int r = threadIdx.x; r < L; r += blockDim.x) {
    const float2 zv = z.get(r);
    const float e = __ldg(a.erho + r);
    const int p0 = __ldg(pos + r);
    if (p0 >= 0) g0[(size_t)p0 * kGatherSlices] = e * zv.x;
    if (th1 >= 0) {
      const int p1 = __ldg(pos + L + r);
      if (p1 >= 0) g0[(size_t)p1 * kGatherSlices] = e * zv.y;
    }
  }
}

// Transposed Cartesian interpolation as a gather: output pixel (X, Y) of the padded
// grid sums, over the cells of the points whose taps reach it (cell = the integer
// part of a point's coordinates), each point's value times its tap weight, in a
// fixed order.  No atomics: the result is the same bits on every run.  A point with
// integer part (ix, iy) reaches columns ix - o .. ix - o + n - 1 (o = 1, n = 4 cubic;
// o = 0, n = 2 linear), so pixel X reads cells ix = X + o - i for tap i.  The n cells
// of one cell row are consecutive in the cell-sorted list unless they wrap at the
// image edge, so away from the edge a pixel walks n runs of points (one per tap row
// j) and takes each point's tap i from its own cell.  A thread computes one pixel for
// the kGatherSlices slices of a group.
constexpr int kGatherPixels = 2;  // pixels per thread of k_fwdT_gather (N is a multiple of 16)

__device__ __forceinline__ float pick_w(const float* w, int i) {
  return i == 0 ? w[0] : (i == 1 ? w[1] : (i == 2 ? w[2] : w[3]));
}

// PX consecutive pixels X0 .. X0 + PX - 1 of a row per thread: their cells of one cell
// row are one run of the list (X0 + o - n + 1 .. X0 + PX - 1 + o), walked once, each
// point adding to the pixels its taps reach -- the points and values are loaded once
// for the PX pixels instead of once per pixel.
template <int PX>
__global__ void __launch_bounds__(256) k_fwdT_gather(FwdTGatherArgs a, int S) {
  const int X0 = (blockIdx.x * 32 + (threadIdx.x & 31)) * PX;
  const int Y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (X0 >= a.N || Y >= a.N) return;
  const int s0 = blockIdx.z * kGatherSlices;
  const int ns = min(kGatherSlices, S - s0);
  const size_t plane = (size_t)a.N * a.N;
  float acc[PX][kGatherSlices];
#pragma unroll
  for (int x = 0; x < PX; ++x)
#pragma unroll
    for (int q = 0; q < kGatherSlices; ++q) acc[x][q] = 0.f;
  const int o = a.cubic ? 1 : 0;
  const int n = a.cubic ? 4 : 2;
  // this slice group's values, [npts][kGatherSlices] in list order
  const float* G = a.G + (size_t)blockIdx.z * a.npts * kGatherSlices;
  // point e (coordinates p) of cell column cx into the pixels whose tap it is, tap row j
  auto add = [&](int e, int2 p, int cx, int j) {
    float wx[4], wy[4];
    axis_weights_fx(p.x, a.F, a.fsc, a.cubic, wx);
    axis_weights_fx(p.y, a.F, a.fsc, a.cubic, wy);
    const float wyj = pick_w(wy, j);
    const float4* g = reinterpret_cast<const float4*>(G + (size_t)e * kGatherSlices);
    const float4 u = __ldg(g);
    const float4 v = ns > 4 ? __ldg(g + 1) : make_float4(0.f, 0.f, 0.f, 0.f);  // block-uniform
#pragma unroll
    for (int x = 0; x < PX; ++x) {
      const int i = X0 + x + o - cx;
      if (i >= 0 && i < n) {
        const float w = wyj * pick_w(wx, i);
        acc[x][0] += w * u.x;
        acc[x][1] += w * u.y;
        acc[x][2] += w * u.z;
        acc[x][3] += w * u.w;
        acc[x][4] += w * v.x;
        acc[x][5] += w * v.y;
        acc[x][6] += w * v.z;
        acc[x][7] += w * v.w;
      }
    }
  };
  const int xlo = X0 + o - (n - 1), xhi = X0 + PX - 1 + o;
  if (xlo >= 0 && xhi < a.N) {
    // the n runs walked side by side (independent load chains), run j in list order
    int e[4], e1[4], m = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      e[j] = e1[j] = 0;
      if (j < n) {
        const int* co = a.cell_off + (size_t)wrapi(Y + o - j, a.N) * a.N;
        e[j] = __ldg(co + xlo);
        e1[j] = __ldg(co + xhi + 1);
        m = max(m, e1[j] - e[j]);
      }
    }
    for (int step = 0; step < m; ++step) {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (e[j] < e1[j]) {
          const int2 p = __ldg(a.pts + e[j]);
          add(e[j], p, wrapi(fx_int(p.x, a.F), a.N), j);
          ++e[j];
        }
      }
    }
  } else {
    // image edge: each pixel's cells one at a time (wrapped); a point of cell cx adds
    // to pixel X0 + x through tap i = X0 + x + o - cx, taken modulo N here
    for (int x = 0; x < PX; ++x) {
      const int X = X0 + x;
      for (int j = 0; j < n; ++j) {
        const int* co = a.cell_off + (size_t)wrapi(Y + o - j, a.N) * a.N;
        for (int i = 0; i < n; ++i) {
          const int cx = wrapi(X + o - i, a.N);
          const int e1 = __ldg(co + cx + 1);
          for (int e = __ldg(co + cx); e < e1; ++e) {
            const int2 p = __ldg(a.pts + e);
            float wx[4], wy[4];
            axis_weights_fx(p.x, a.F, a.fsc, a.cubic, wx);
            axis_weights_fx(p.y, a.F, a.fsc, a.cubic, wy);
            const float w = pick_w(wy, j) * pick_w(wx, i);
            const float4* g = reinterpret_cast<const float4*>(G + (size_t)e * kGatherSlices);
            const float4 u = __ldg(g);
            const float4 v = ns > 4 ? __ldg(g + 1) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int xx = 0; xx < PX; ++xx) {
              if (xx == x) {
                acc[xx][0] += w * u.x;
                acc[xx][1] += w * u.y;
                acc[xx][2] += w * u.z;
                acc[xx][3] += w * u.w;
                acc[xx][4] += w * v.x;
                acc[xx][5] += w * v.y;
                acc[xx][6] += w * v.z;
                acc[xx][7] += w * v.w;
              }
            }
          }
        }
      }
    }
  }
  float* out = a.acc + (size_t)s0 * plane + (size_t)Y * a.N + X0;
#pragma unroll
  for (int q = 0; q < kGatherSlices; ++q) {
    if (q < ns) {
#pragma unroll
      for (int x = 0; x < PX; ++x) out[q * plane + x] = acc[x][q];
    }
  }
}

// ---------------------------------------------------------------------------
// Chunked transposed prefilter.  The transpose of one line's prefilter
// (ConvertToInterpolationCoefficients, main_kernels.cuh:97-142, with its
// boundary initialisations): y1 = causal pass t = x + z t with outputs -z t
// (q t = z/(z-1) t at the last sample), then w = y1 + z w backwards, then
// out = lambda w plus, for the first 12 samples, lambda z^(m+1) w(0) (the
// transposed causal boundary term).  Each chunk starts both recursions LP_WARM
// samples outside itself from a zero state (exact to |pole|^16 ~ 7e-10, as the
// forward prefilter's chunks are) and the line ends use the exact starts.
// ---------------------------------------------------------------------------

// columns: one warp per 32 columns x kColC rows staged in shared memory, out of place
__global__ void __launch_bounds__(32 * kColWarps) k_prefilter_T_cols(PrefilterTColsArgs a) {
  __shared__ float tile[kColWarps][kColRows][32];
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int H = a.H, W = a.W;
  const int b = (blockIdx.y * kColWarps + wp) * kColC;
  if (b >= H) return;  // warps are independent
  const int e = min(b + kColC, H);
  const int r0 = max(0, b - LP_WARM), r1 = min(H, e + LP_WARM);
  const int x = blockIdx.x * 32 + lane;
  const int s = blockIdx.z;
  const bool inx = x < W;
  float(*t)[32] = tile[wp];
  const float* col = a.in + (size_t)s * H * W + x;
  for (int r = r0; r < r1; ++r) {
    if (inx) cp_async4(&t[r - r0][lane], col + (size_t)r * W);
    else t[r - r0][lane] = 0.f;
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncwarp();
  const float z = LP_POLE, q = LP_POLE / (LP_POLE - 1.0f);
  float tc = 0.f;  // row 0 is the exact start; other chunks warm up from a zero state
  for (int m = r0; m < r1; ++m) {
    tc = t[m - r0][lane] + z * tc;
    t[m - r0][lane] = (m < H - 1) ? -z * tc : q * tc;
  }
  float w = 0.f;  // row H-1 is the exact start (w = y1 there); elsewhere a zero-state warm-up
  for (int m = r1 - 1; m >= b; --m) {
    w = t[m - r0][lane] + z * w;
    t[m - r0][lane] = w;
  }
  float* dst = a.out + (size_t)s * H * W + x;
  if (!inx) return;
  const int hor = b == 0 ? min(12, H) : 0;
  const float w0 = t[0][lane];
  float zn = z;
  for (int m = b; m < e; ++m) {
    float v = LP_LAMBDA * t[m - r0][lane];
    if (m < hor) {
      v += LP_LAMBDA * zn * w0;
      zn *= z;
    }
    dst[(size_t)m * W] = v;
  }
}

// rows: one warp per output row (kRowWarps rows per block), the padded row in shared
// memory, chunks of odd length per lane (distinct banks; at N = 512 chunks of 17
// against the recursions' 16-sample warm-ups), the window [off, off + N0) of it
// written into the caller's image (the crop of the forward's centring)
constexpr int kRowWarps = 4;

__global__ void __launch_bounds__(32 * kRowWarps) k_prefilter_T_rows_crop(PrefilterTRowsCropArgs a) {
  extern __shared__ float smf[];
  const int N = a.N;
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int s = blockIdx.x, yo = blockIdx.y * (blockDim.x >> 5) + wp;
  if (yo >= a.N0) return;  // warps are independent
  float* line = smf + (size_t)wp * 2 * N;
  float* y1 = line + N;
  const float* src = a.in + ((size_t)s * N + yo + a.off) * N;
  for (int x = lane; x < N; x += 32) line[x] = __ldg(src + x);
  __syncwarp();
  const float z = LP_POLE, q = LP_POLE / (LP_POLE - 1.0f);
  const int C = line_chunk(N, 32);
  const int b = lane * C, e = min(b + C, N);
  if (b < N) {
    float tc = 0.f;
    for (int m = max(0, b - LP_WARM); m < e; ++m) {
      tc = line[m] + z * tc;
      if (m >= b) y1[m] = (m < N - 1) ? -z * tc : q * tc;
    }
  }
  __syncwarp();
  if (b < N) {
    // the next chunks' causal outputs serve as this chunk's anticausal warm-up
    float w = 0.f;
    for (int m = min(N, e + LP_WARM) - 1; m >= b; --m) {
      w = y1[m] + z * w;
      if (m < e) line[m] = w;
    }
  }
  __syncwarp();
  const float w0 = line[0];
  float* dst = a.out + ((size_t)s * a.N0 + yo) * a.N0 - a.off;
  for (int x = a.off + lane; x < a.off + a.N0; x += 32) {
    float v = LP_LAMBDA * line[x];
    if (x < 12) {
      float zn = z;
      for (int i = 0; i < x; ++i) zn *= z;
      v += LP_LAMBDA * zn * w0;
    }
    dst[x] = v;
  }
}

__global__ void k_crop(CropArgs a) {
  const int s = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.N0 * a.N0) return;
  const int y = i / a.N0, x = i - y * a.N0;
  a.dst[(size_t)s * a.N0 * a.N0 + i] = a.src[((size_t)s * a.N + y + a.off) * a.N + x + a.off];
}

cudaError_t launch_fwdT_rows(const FwdTRowsArgs& a, int S, cudaStream_t st) {
  if (a.nrows <= 0) return cudaSuccess;
  cudaError_t pe;
  if (LP_REGISTER_FFT(fwdT_rows, a, S, st, &pe)) return pe;
  const size_t sm = fft_bytes(a.Nrho, 1) + 2 * (size_t)a.Nrho * sizeof(float);
  if (smem_ok(sm) != cudaSuccess) return cudaErrorInvalidConfiguration;
  cudaFuncSetAttribute(k_fwdT_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
  dim3 grid(S, (a.nrows + 1) / 2);
  k_fwdT_rows<<<grid, 256, sm, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_fwdT_colsum(const FwdTColSumArgs& a, int S, int nblk, cudaStream_t st) {
  if (nblk <= 0) return cudaSuccess;
  if (a.CW != kColSumCW) return cudaErrorInvalidValue;
  dim3 grid(S, nblk);
  k_fwdT_colsum<<<grid, 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_fwdT_cols(const FwdTColsArgs& a, int S, cudaStream_t st) {
  if (a.dhi < a.dlo) return cudaSuccess;
  cudaError_t pe;
  if (LP_REGISTER_FFT(fwdT_cols, a, S, st, &pe)) return pe;
  const size_t sm = fft_bytes(a.Nrho, 1);
  if (smem_ok(sm) != cudaSuccess) return cudaErrorInvalidConfiguration;
  cudaFuncSetAttribute(k_fwdT_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
  dim3 grid(S, (a.dhi - a.dlo + 2) / 2);
  k_fwdT_cols<<<grid, 256, sm, st>>>(a);
  return cudaGetLastError();
}

// the theta columns' tap weights of the exact transpose: entry (i, j) -> (i, bits of
// tap j's weight of the span's row i), the weight the forward's theta interpolation uses
__global__ void k_fwdT_tapw(int2* cent, int n, const int* rows, const int* thc, int F, float fsc, int cubic) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  int2 q = cent[e];
  float w[4];
  axis_weights_fx(__ldg(thc + __ldg(rows + q.x)), F, fsc, cubic, w);
  q.y = __float_as_int(w[q.y & 3]);
  cent[e] = q;
}

cudaError_t launch_fwdT_tapw(int2* cent, int n, const int* rows, const int* thc, int F, float fsc, int cubic,
                             cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_fwdT_tapw<<<(n + 255) / 256, 256, 0, st>>>(cent, n, rows, thc, F, fsc, cubic);
  return cudaGetLastError();
}

cudaError_t launch_fwdT_gather(const FwdTGatherArgs& a, int S, cudaStream_t st) {
  constexpr int PX = kGatherPixels;
  if (a.N % PX != 0) return cudaErrorInvalidValue;
  dim3 grid((a.N / PX + 31) / 32, (a.N + 7) / 8, (S + kGatherSlices - 1) / kGatherSlices);
  k_fwdT_gather<PX><<<grid, 256, 0, st>>>(a, S);
  return cudaGetLastError();
}

cudaError_t launch_prefilter_T_cols(const PrefilterTColsArgs& a, int S, cudaStream_t st) {
  const int chunks = (a.H + kColC - 1) / kColC;
  dim3 grid((a.W + 31) / 32, (chunks + kColWarps - 1) / kColWarps, S);
  k_prefilter_T_cols<<<grid, 32 * kColWarps, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_prefilter_T_rows_crop(const PrefilterTRowsCropArgs& a, int S, cudaStream_t st) {
  // up to kRowWarps rows per block, as many as the shared memory holds (2 N floats each)
  const size_t row = 2 * (size_t)a.N * sizeof(float);
  const int wpb = (int)std::max<size_t>(1, std::min<size_t>(kRowWarps, (size_t)g_smem_optin / row));
  const size_t sm = wpb * row;
  if (smem_ok(sm) != cudaSuccess) return cudaErrorInvalidConfiguration;
  cudaFuncSetAttribute(k_prefilter_T_rows_crop, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
  dim3 grid(S, (a.N0 + wpb - 1) / wpb);
  k_prefilter_T_rows_crop<<<grid, 32 * wpb, sm, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_crop(const CropArgs& a, int S, cudaStream_t st) {
  dim3 grid((a.N0 * a.N0 + 255) / 256, S);
  k_crop<<<grid, 256, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace lpgb
