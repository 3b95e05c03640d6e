// Shared-memory complex FFT used by the log-polar convolution and the FBP filter.
//
// Stockham autosort formulation: every stage reads the whole signal with unit
// stride (conflict-free), applies one radix-r butterfly per group of r points,
// and writes in sorted order into the other buffer.  Radices 2, 3, 4, 5, 7 and
// 8 have hand-written butterflies; any other prime factor uses a direct DFT.
// Lengths are N = 16*m (log-polar grids) or 4N, 2N: any positive length works.
//
// Sign convention: dir = -1 is the forward transform exp(-2*pi*i*jk/L), dir =
// +1 the unnormalised inverse, as cuFFT defines them (reference call sites
// src/cuda/lpRgpu.cu:270,277,314,321,353,368).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace lpgb {

#define LP_FFT_MAX_STAGES 24

struct FFTPlan {
  int L;
  int nst;
  int radix[LP_FFT_MAX_STAGES];
};

// Factor L into stages, largest fast radix first.
inline FFTPlan make_fft_plan(int L) {
  FFTPlan p;
  p.L = L;
  p.nst = 0;
  int n = L;
  while (n % 8 == 0) { p.radix[p.nst++] = 8; n /= 8; }
  while (n % 4 == 0) { p.radix[p.nst++] = 4; n /= 4; }
  while (n % 2 == 0) { p.radix[p.nst++] = 2; n /= 2; }
  const int fast[] = {3, 5, 7};
  for (int f : fast)
    while (n % f == 0) { p.radix[p.nst++] = f; n /= f; }
  for (int f = 11; n > 1; f += 2)
    while (n % f == 0) { p.radix[p.nst++] = f; n /= f; }
  return p;
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by dir*i
template <int DIR>
__device__ __forceinline__ float2 mul_i(float2 a) {
  return DIR < 0 ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
}

template <int DIR>
__device__ __forceinline__ void bfly2(float2* v) {
  float2 a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <int DIR>
__device__ __forceinline__ void bfly4(float2* v) {
  float2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
  float2 b0 = cadd(v[1], v[3]), b1 = mul_i<DIR>(csub(v[1], v[3]));
  v[0] = cadd(a0, b0);
  v[2] = csub(a0, b0);
  v[1] = cadd(a1, b1);
  v[3] = csub(a1, b1);
}

template <int DIR>
__device__ __forceinline__ void bfly8(float2* v) {
  const float r = 0.70710678118654752440f;
  float2 e[4] = {v[0], v[2], v[4], v[6]};
  float2 o[4] = {v[1], v[3], v[5], v[7]};
  bfly4<DIR>(e);
  bfly4<DIR>(o);
  // twiddles w8^k, k = 0..3, w8 = exp(dir*i*pi/4)
  float2 t1 = make_float2(r * (o[1].x - DIR * o[1].y), r * (o[1].y + DIR * o[1].x));
  float2 t2 = mul_i<DIR>(o[2]);
  float2 t3 = make_float2(r * (-o[3].x - DIR * o[3].y), r * (-o[3].y + DIR * o[3].x));
  v[0] = cadd(e[0], o[0]);
  v[4] = csub(e[0], o[0]);
  v[1] = cadd(e[1], t1);
  v[5] = csub(e[1], t1);
  v[2] = cadd(e[2], t2);
  v[6] = csub(e[2], t2);
  v[3] = cadd(e[3], t3);
  v[7] = csub(e[3], t3);
}

template <int DIR>
__device__ __forceinline__ void bfly3(float2* v) {
  const float c = -0.5f, s = DIR * 0.86602540378443864676f;
  float2 t = cadd(v[1], v[2]);
  float2 d = csub(v[1], v[2]);
  float2 m = make_float2(v[0].x + c * t.x, v[0].y + c * t.y);
  float2 r = make_float2(-s * d.y, s * d.x);
  v[0] = cadd(v[0], t);
  v[1] = cadd(m, r);
  v[2] = csub(m, r);
}

template <int DIR>
__device__ __forceinline__ void bfly5(float2* v) {
  const float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;
  const float s1 = DIR * 0.95105651629515357212f, s2 = DIR * 0.58778525229247312917f;
  float2 t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
  float2 d1 = csub(v[1], v[4]), d2 = csub(v[2], v[3]);
  float2 m1 = make_float2(v[0].x + c1 * t1.x + c2 * t2.x, v[0].y + c1 * t1.y + c2 * t2.y);
  float2 m2 = make_float2(v[0].x + c2 * t1.x + c1 * t2.x, v[0].y + c2 * t1.y + c1 * t2.y);
  float2 r1 = make_float2(-(s1 * d1.y + s2 * d2.y), s1 * d1.x + s2 * d2.x);
  float2 r2 = make_float2(-(s2 * d1.y - s1 * d2.y), s2 * d1.x - s1 * d2.x);
  v[0] = cadd(v[0], cadd(t1, t2));
  v[1] = cadd(m1, r1);
  v[4] = csub(m1, r1);
  v[2] = cadd(m2, r2);
  v[3] = csub(m2, r2);
}

// Generic odd radix (7 and larger primes): direct DFT, O(r^2) per butterfly.
template <int DIR, int R>
__device__ __forceinline__ void bfly_direct(float2* v) {
  float2 out[R];
#pragma unroll
  for (int k = 0; k < R; ++k) {
    float2 acc = v[0];
#pragma unroll
    for (int j = 1; j < R; ++j) {
      float sn, cs;
      sincospif((float)(2 * DIR * ((j * k) % R)) / (float)R, &sn, &cs);
      acc.x += v[j].x * cs - v[j].y * sn;
      acc.y += v[j].x * sn + v[j].y * cs;
    }
    out[k] = acc;
  }
#pragma unroll
  for (int k = 0; k < R; ++k) v[k] = out[k];
}

// One Stockham stage with a compile-time radix over `nfft` signals of length L
// stored at `stride` apart.  Ns = product of the radices already applied.
template <int DIR, int R>
__device__ __forceinline__ void fft_stage(const float2* __restrict__ in, float2* __restrict__ out, int L,
                                          int Ns, int nfft, int stride) {
  const int Lr = L / R;
  const int total = nfft * Lr;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int f = t / Lr;
    const int j = t - f * Lr;
    const float2* src = in + f * stride;
    float2* dst = out + f * stride;
    const int k = j % Ns;
    float2 v[R];
#pragma unroll
    for (int i = 0; i < R; ++i) v[i] = src[j + i * Lr];
    if (Ns > 1) {
      // twiddle exp(dir*2*pi*i*i*k/(Ns*R))
      const float base = (float)(2 * DIR) * (float)k / (float)(Ns * R);
#pragma unroll
      for (int i = 1; i < R; ++i) {
        float sn, cs;
        sincospif(base * (float)i, &sn, &cs);
        v[i] = cmul(v[i], make_float2(cs, sn));
      }
    }
    if (R == 2) bfly2<DIR>(v);
    else if (R == 3) bfly3<DIR>(v);
    else if (R == 4) bfly4<DIR>(v);
    else if (R == 5) bfly5<DIR>(v);
    else if (R == 8) bfly8<DIR>(v);
    else bfly_direct<DIR, R>(v);
    const int base_o = (j - k) * R + k;
#pragma unroll
    for (int i = 0; i < R; ++i) dst[base_o + i * Ns] = v[i];
  }
}

// Generic prime radix not known at compile time (rare: N with a prime factor > 7).
template <int DIR>
__device__ void fft_stage_dyn(const float2* __restrict__ in, float2* __restrict__ out, int L, int Ns, int R,
                              int nfft, int stride) {
  const int Lr = L / R;
  const int total = nfft * Lr;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int f = t / Lr;
    const int j = t - f * Lr;
    const float2* src = in + f * stride;
    float2* dst = out + f * stride;
    const int k = j % Ns;
    const int base_o = (j - k) * R + k;
    for (int q = 0; q < R; ++q) {
      float2 acc = make_float2(0.f, 0.f);
      for (int i = 0; i < R; ++i) {
        // total phase: twiddle i*k/(Ns*R) + butterfly i*q/R
        const long long num = (long long)i * k + (long long)((i * q) % R) * Ns;
        const long long den = (long long)Ns * R;
        float sn, cs;
        sincospif((float)(2 * DIR) * (float)(num % den) / (float)den, &sn, &cs);
        const float2 x = src[j + i * Lr];
        acc.x += x.x * cs - x.y * sn;
        acc.y += x.x * sn + x.y * cs;
      }
      dst[base_o + q * Ns] = acc;
    }
  }
}

// Run the whole transform; data starts in `a`, `b` is scratch of the same
// size.  Returns the buffer that holds the result (a or b).  All threads of
// the block must call it; it ends with a __syncthreads().
template <int DIR>
__device__ float2* fft_block(float2* a, float2* b, const FFTPlan& p, int nfft, int stride) {
  int Ns = 1;
  float2* in = a;
  float2* out = b;
  for (int s = 0; s < p.nst; ++s) {
    const int R = p.radix[s];
    switch (R) {
      case 2: fft_stage<DIR, 2>(in, out, p.L, Ns, nfft, stride); break;
      case 3: fft_stage<DIR, 3>(in, out, p.L, Ns, nfft, stride); break;
      case 4: fft_stage<DIR, 4>(in, out, p.L, Ns, nfft, stride); break;
      case 5: fft_stage<DIR, 5>(in, out, p.L, Ns, nfft, stride); break;
      case 7: fft_stage<DIR, 7>(in, out, p.L, Ns, nfft, stride); break;
      case 8: fft_stage<DIR, 8>(in, out, p.L, Ns, nfft, stride); break;
      default: fft_stage_dyn<DIR>(in, out, p.L, Ns, R, nfft, stride); break;
    }
    __syncthreads();
    Ns *= R;
    float2* t = in;
    in = out;
    out = t;
  }
  return in;
}

}  // namespace lpgb
