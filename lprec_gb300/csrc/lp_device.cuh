// Device helpers shared by the kernel translation units: fixed-point
// coordinates, cubic B-spline weights, explicit interpolation with wrap
// addressing, the chunked prefilter recursion, and the packing of two real
// signals into one complex FFT.
#pragma once
#include <climits>

#include "lp_kernels.cuh"
#include "fft_mr.cuh"

namespace lpgb {

// cubic B-spline pole and gain (src/include/main_kernels.cuh:2, :124)
#define LP_POLE (-0.2679491924311228f)
#define LP_LAMBDA (6.0f)
#define LP_WARM 16  // warm-up length of the chunked recursions: |pole|^16 < 1e-9

__device__ __forceinline__ int wrapi(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

// ---------------------------------------------------------------------------
// Interpolation coordinates are stored as 32-bit fixed point: value = v * 2^-F
// with F chosen per handle from the largest coordinate (F = 17 at N = 2048:
// steps of 7.6e-6 texel, where float32 near 4096 steps by 4.9e-4).  The
// integer tap position is v >> F (an arithmetic shift, i.e. floor) and the
// fraction (v & (2^F - 1)) * 2^-F is exact in float32.  LP_FX_NONE marks a
// table entry without a point.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int fx_int(int v, int F) { return v >> F; }
__device__ __forceinline__ float fx_frac(int v, int F, float fsc) { return (float)(v & ((1 << F) - 1)) * fsc; }

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
__device__ __forceinline__ float interp2d_split(const float* __restrict__ img, int W, int H, int ix, float ax,
                                                int iy, float ay, int cubic) {
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

// 2-D interpolation at fixed-point index position (x, y)
__device__ __forceinline__ float interp2d_fx(const float* __restrict__ img, int W, int H, int vx, int vy, int F,
                                             float fsc, int cubic) {
  return interp2d_split(img, W, H, fx_int(vx, F), fx_frac(vx, F, fsc), fx_int(vy, F), fx_frac(vy, F, fsc), cubic);
}


// Cubic B-spline sample of a 2-D texture (N x N texels, normalised
// coordinates, wrap addressing) at index position (x, y) from four 2x2
// texel gathers.  A gather at integer texel coordinate (i, j) returns the
// raw texels of columns i-1, i and rows j-1, j -- no filtering weights are
// involved, the B-spline weights are applied here in float32.  The 0.5-texel
// margin of the integer position makes the quad selection insensitive to
// coordinate rounding.  Gather component order: w (i-1, j-1), z (i, j-1),
// x (i-1, j), y (i, j).
__device__ __forceinline__ float interp_tex_cubic_split(cudaTextureObject_t tx, float invW, float invH, int ix,
                                                       float ax, int iy, float ay) {
  float wx[4], wy[4];
  bspline_w(ax, wx);
  bspline_w(ay, wy);
  const float fx = (float)ix, fy = (float)iy;
  const float u0 = fx * invW, u1 = (fx + 2.0f) * invW;
  const float v0 = fy * invH, v1 = (fy + 2.0f) * invH;
  const float4 q00 = tex2Dgather<float4>(tx, u0, v0, 0);
  const float4 q10 = tex2Dgather<float4>(tx, u1, v0, 0);
  const float4 q01 = tex2Dgather<float4>(tx, u0, v1, 0);
  const float4 q11 = tex2Dgather<float4>(tx, u1, v1, 0);
  const float r0 = wx[0] * q00.w + wx[1] * q00.z + wx[2] * q10.w + wx[3] * q10.z;
  const float r1 = wx[0] * q00.x + wx[1] * q00.y + wx[2] * q10.x + wx[3] * q10.y;
  const float r2 = wx[0] * q01.w + wx[1] * q01.z + wx[2] * q11.w + wx[3] * q11.z;
  const float r3 = wx[0] * q01.x + wx[1] * q01.y + wx[2] * q11.x + wx[3] * q11.y;
  return wy[0] * r0 + wy[1] * r1 + wy[2] * r2 + wy[3] * r3;
}

// the same at fixed-point texel coordinates (x, y)
__device__ __forceinline__ float interp_tex_cubic_fx(cudaTextureObject_t tx, float invW, float invH, int vx, int vy,
                                                    int F, float fsc) {
  return interp_tex_cubic_split(tx, invW, invH, fx_int(vx, F), fx_frac(vx, F, fsc), fx_int(vy, F),
                                fx_frac(vy, F, fsc));
}

// 1-D interpolation along a shared-memory line of length L (wrap).
template <typename Get>
__device__ __forceinline__ float interp1d_split(Get get, int L, int ix, float ax, int cubic) {
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

// 1-D interpolation at fixed-point position v
template <typename Get>
__device__ __forceinline__ float interp1d_fx(Get get, int L, int v, int F, float fsc, int cubic) {
  return interp1d_split(get, L, fx_int(v, F), fx_frac(v, F, fsc), cubic);
}

// Interpolation weights along one axis at fixed-point coordinate v: returns the first tap.
__device__ __forceinline__ int axis_weights_fx(int v, int F, float fsc, int cubic, float* w) {
  const int it = fx_int(v, F);
  const float a = fx_frac(v, F, fsc);
  if (cubic) {
    bspline_w(a, w);
    return it - 1;
  }
  w[0] = 1.f - a;
  w[1] = a;
  w[2] = 0.f;
  w[3] = 0.f;
  return it;
}

// Two complex FFT buffers (nfft signals of length L each) at the start of
// dynamic shared memory; returns the first float after them.
__device__ __forceinline__ float* carve(float* sm, int L, int nfft, CBuf& a, CBuf& b) {
  const int pf = nfft * fft_plane_floats(L);
  a = CBuf{sm, sm + pf};
  b = CBuf{sm + 2 * pf, sm + 3 * pf};
  return sm + 4 * pf;
}

// ---------------------------------------------------------------------------
// Cubic B-spline prefilter of one line held in shared memory
// (ConvertToInterpolationCoefficients, src/include/main_kernels.cuh:97-142).
// The block splits the line into chunks; every chunk starts its causal and
// anticausal recursions LP_WARM samples early from a zero state, which is
// exact to |pole|^16 ~ 7e-10; the first and last chunk use the reference's
// boundary initialisations.  `cp` is scratch of L floats.
// ---------------------------------------------------------------------------
// Lines are split into chunks of odd length C, so the threads walking their
// chunks in lockstep (stride C) hit distinct shared-memory banks without any
// padding.  The last chunks may be short or empty.
__host__ __device__ inline int line_chunk(int L, int nth) { return ((L + nth - 1) / nth) | 1; }
__device__ __forceinline__ int lpos(int p, int C) { return p; }
// floats a line of L samples occupies
__host__ __device__ inline int line_floats(int L, int nth) { return L; }

static __device__ void prefilter_line(float* line, float* cp, int L, int tid, int nth) {
  const float z = LP_POLE;
  const int C = line_chunk(L, nth);
  const int b = tid * C;
  const int e = min(b + C, L);
  if (b < L) {
    float prev;
    const int n0 = b - LP_WARM;
    int n = 0;
    if (n0 <= 0) {
      const int hor = min(12, L);
      float sum = line[lpos(0, C)];
      float zn = z;
      for (int i = 0; i < hor; ++i) {
        sum += zn * line[lpos(i, C)];
        zn *= z;
      }
      prev = LP_LAMBDA * sum;
      if (b == 0) cp[lpos(0, C)] = prev;
      n = 1;
    } else {
      prev = LP_LAMBDA * line[lpos(n0, C)];
      n = n0 + 1;
    }
    for (; n < e; ++n) {
      prev = LP_LAMBDA * line[lpos(n, C)] + z * prev;
      if (n >= b) cp[lpos(n, C)] = prev;
    }
  }
  __syncthreads();
  if (b < L) {
    const int n1 = e - 1 + LP_WARM;
    float c;
    int n;
    if (n1 >= L - 1) {
      c = (z / (z - 1.0f)) * cp[lpos(L - 1, C)];
      if (L - 1 < e) line[lpos(L - 1, C)] = c;
      n = L - 2;
    } else {
      c = -z * cp[lpos(n1, C)];
      n = n1 - 1;
    }
    for (; n >= b; --n) {
      c = z * (c - cp[lpos(n, C)]);
      if (n < e) line[lpos(n, C)] = c;
    }
  }
  __syncthreads();
}


__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}

// Build the complex signal whose inverse FFT gives two real rho profiles
// from their half spectra V0, V1 (kr = 0..Nrho/2); C2R semantics: the
// imaginary parts at kr = 0 and kr = Nrho/2 are ignored.
__device__ __forceinline__ void put_pair(const CBuf& Z, int k, int Nrho, float2 v0, float2 v1) {
  const int half = Nrho / 2;
  if (k == 0 || k == half) {
    Z.set(k, make_float2(v0.x, v1.x));
  } else {
    Z.set(k, make_float2(v0.x - v1.y, v0.y + v1.x));
    Z.set(Nrho - k, make_float2(v0.x + v1.y, v1.x - v0.y));
  }
}


// element p of the complex signal whose inverse FFT gives two real profiles
// with half spectra V0, V1 (C2R semantics: imaginary parts at 0 and L/2 ignored)
__device__ __forceinline__ float2 pair_elem(int p, int L, float2 v0, float2 v1) {
  const int half = L / 2;
  if (p == 0 || p == half) return make_float2(v0.x, v1.x);
  if (p < half) return make_float2(v0.x - v1.y, v0.y + v1.x);
  return make_float2(v0.x + v1.y, v1.x - v0.y);  // conj(V0) + i conj(V1) at L - p
}

// Transposed 1-D interpolation along rho of the internal sinogram rows r0 and r1
// (r1 < 0: none) of slice s, added into acc(q, bin) for row q = 0, 1.  Called by
// all threads of the block (the same number of barriers on every path); thread
// tid of nth takes its share of the points.  With strictly monotone first taps
// (a.mono) the points of one residue class of x modulo the tap count and one window
// of first taps hit distinct bins with all their taps, so they are added in one
// pass without conflicts, in a fixed order; otherwise one thread per row adds its
// points' taps in x order.
template <class ArgsT, class Acc>
__device__ __forceinline__ void rho_scatter_T(const ArgsT& a, int s, int r0, int r1, int tid, int nth, Acc acc) {
  const int ntap = a.cubic ? 4 : 2;
  const int L = a.Nrho;
  if (a.mono) {
    // pass (p, h): the points x = p (mod ntap) whose first tap is below (h = 0) or from
    // (h = 1) the row's smallest first tap + L - ntap + 1, all taps of each.  First taps
    // strictly monotone in x put the points of one residue class at least ntap apart,
    // and a window spans at most L - ntap, so no two taps of a pass meet modulo L: each
    // bin takes at most one addition per pass, in a fixed pass order (rows that do not
    // wrap skip the second window; every thread still meets every barrier, and a block
    // none of whose rows wraps runs no second-window passes at all)
    const bool wraps = __syncthreads_or((r0 >= 0 && __ldg(a.rbase + r0) != kNoWrap) ||
                                        (r1 >= 0 && __ldg(a.rbase + r1) != kNoWrap));
    const int nwin = wraps ? 2 : 1;
    if (2 * ntap * nth >= a.N) {
      // at most two points per residue class and row per thread (N <= 2 ntap nth, as for
      // every register-FFT length, N = L / 2 = 8 T): the thread's points of both rows,
      // x = ntap tid + p + m ntap nth, are loaded once before the passes (no global
      // load waits inside the barrier-separated passes)
      float pv[2][2][4];
      int pc[2][2][4];
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int r = q == 0 ? r0 : r1;
        const float* row = r >= 0 ? a.Rin + ((size_t)s * a.Nproj0 + r / a.os) * a.N0 : a.Rin;
#pragma unroll
        for (int m = 0; m < 2; ++m)
#pragma unroll
          for (int p = 0; p < 4; ++p) {
            const int x = ntap * tid + p + m * ntap * nth;
            const int xo = x - a.cor_off;
            const bool ok = r >= 0 && p < ntap && x < a.N && xo >= 0 && xo < a.N0;
            pc[q][m][p] = ok ? __ldg(a.rhoc + (size_t)r * a.N + x) : LP_FX_NONE;
            pv[q][m][p] = ok ? __ldg(row + xo) : 0.f;
          }
      }
      for (int p = 0; p < ntap; ++p) {
        for (int h = 0; h < nwin; ++h) {
#pragma unroll
          for (int q = 0; q < 2; ++q) {
            const int r = q == 0 ? r0 : r1;
            if (r < 0) continue;
            const int base = __ldg(a.rbase + r);
            if (h == 1 && base == kNoWrap) continue;
            const int top = base == kNoWrap ? INT_MAX : base + L - ntap + 1;
#pragma unroll
            for (int m = 0; m < 2; ++m) {
              int rc = pc[q][m][0];
              float val = pv[q][m][0];
#pragma unroll
              for (int pp = 1; pp < 4; ++pp)
                if (p == pp) {
                  rc = pc[q][m][pp];
                  val = pv[q][m][pp];
                }
              if (rc == LP_FX_NONE) continue;
              float w[4];
              const int c = axis_weights_fx(rc, a.F, a.fsc, a.cubic, w);
              if ((c >= top) != (h == 1)) continue;
              for (int j = 0; j < ntap; ++j) acc(q, wrapi(c + j, L)) += w[j] * val;
            }
          }
          __syncthreads();
        }
      }
      return;
    }
    for (int p = 0; p < ntap; ++p) {
      for (int h = 0; h < nwin; ++h) {
        for (int q = 0; q < 2; ++q) {
          const int r = q == 0 ? r0 : r1;
          if (r < 0) continue;
          const int base = __ldg(a.rbase + r);
          if (h == 1 && base == kNoWrap) continue;  // every point went in the first window
          const float* row = a.Rin + ((size_t)s * a.Nproj0 + r / a.os) * a.N0;
          const int top = base == kNoWrap ? INT_MAX : base + L - ntap + 1;
          for (int x = p + ntap * tid; x < a.N; x += ntap * nth) {
            const int xo = x - a.cor_off;
            if (xo < 0 || xo >= a.N0) continue;
            float w[4];
            const int c = axis_weights_fx(__ldg(a.rhoc + (size_t)r * a.N + x), a.F, a.fsc, a.cubic, w);
            if ((c >= top) != (h == 1)) continue;
            const float val = __ldg(row + xo);
            for (int j = 0; j < ntap; ++j) acc(q, wrapi(c + j, L)) += w[j] * val;
          }
        }
        __syncthreads();
      }
    }
  } else {
    const int r = tid == 0 ? r0 : (tid == 1 ? r1 : -1);
    if (r >= 0) {
      const float* row = a.Rin + ((size_t)s * a.Nproj0 + r / a.os) * a.N0;
      for (int x = 0; x < a.N; ++x) {
        const int xo = x - a.cor_off;
        if (xo < 0 || xo >= a.N0) continue;
        float w[4];
        const int c = axis_weights_fx(__ldg(a.rhoc + (size_t)r * a.N + x), a.F, a.fsc, a.cubic, w);
        const float val = __ldg(row + xo);
        for (int j = 0; j < ntap; ++j) acc(tid, wrapi(c + j, L)) += w[j] * val;
      }
    }
    __syncthreads();
  }
}

// The two rows' half spectra from the complex FFT Z of (row 0) + i (row 1), each
// times a_k (1 at k = 0 and L/2, else 2; the imaginary parts of those two bins
// dropped): the transpose of the forward's C2R of one row.
__device__ __forceinline__ void split_rows_T(float2 z1, float2 z2, int k, int L, float2* va, float2* vb) {
  const float ak = (k == 0 || k == L / 2) ? 1.f : 2.f;
  float2 x = make_float2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
  float2 y = make_float2(0.5f * (z1.y + z2.y), 0.5f * (z2.x - z1.x));
  if (ak == 1.f) {
    x.y = 0.f;
    y.y = 0.f;
  }
  *va = cscale(x, ak);
  *vb = cscale(y, ak);
}

}  // namespace lpgb
