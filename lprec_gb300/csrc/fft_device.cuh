// Shared-memory complex FFT used by the log-polar convolution and the FBP filter.
//
// Stockham autosort formulation, ping-pong between two shared buffers.  Data is
// planar (separate re / im float arrays) with one pad word after every 32, so
// both the unit-stride reads and the stride-R writes of a stage hit distinct
// banks.  Twiddles come from a table W[t] = exp(-2*pi*i*t/L) computed on the
// host in float64.  Radix 16, 8, 4, 2, 3, 5 and 7 have hand-written
// butterflies; other prime factors use a direct DFT from the same table, so
// any length works (N = 16*m log-polar grids allow any m).
//
// Sign convention: DIR = -1 is the forward transform exp(-2*pi*i*jk/L),
// DIR = +1 the unnormalised inverse, as cuFFT defines them (reference call
// sites src/cuda/lpRgpu.cu:270,277,314,321,353,368).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace lpgb {

#define LP_FFT_MAX_STAGES 24

struct FFTPlan {
  int L;
  int nst;
  int radix[LP_FFT_MAX_STAGES];
  const float2* tw;  // device table of L twiddles exp(-2*pi*i*t/L)
};

// Factor L into stages, largest fast radix first.
inline FFTPlan make_fft_plan(int L, const float2* tw) {
  FFTPlan p;
  p.L = L;
  p.nst = 0;
  p.tw = tw;
  int n = L;
  while (n % 16 == 0) { p.radix[p.nst++] = 16; n /= 16; }
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

// padded planar index
__device__ __forceinline__ int fpad(int p) { return p + (p >> 5); }
// floats needed for one planar plane of length L
__host__ __device__ inline int fft_plane_floats(int L) { return L + (L >> 5) + 1; }

// A complex array in shared memory: two padded planes.
struct CBuf {
  float* re;
  float* im;
  __device__ __forceinline__ float2 get(int p) const {
    const int q = fpad(p);
    return make_float2(re[q], im[q]);
  }
  __device__ __forceinline__ void set(int p, float2 v) const {
    const int q = fpad(p);
    re[q] = v.x;
    im[q] = v.y;
  }
  __device__ __forceinline__ CBuf offset(int n) const { return CBuf{re + n, im + n}; }
};

// floats of one complex buffer holding `nfft` signals of length L; signal f
// starts fft_plane_floats(L) * f floats into each plane (the `stride`
// argument of fft_block), so the padding of one signal never overlaps the next
__host__ __device__ inline int fft_buf_floats(int L, int nfft) { return 2 * nfft * fft_plane_floats(L); }

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by DIR*i
template <int DIR>
__device__ __forceinline__ float2 mul_i(float2 a) {
  return DIR < 0 ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
}
// multiply by exp(DIR*i*pi*m/8) given c = cos(pi*m/8), s = sin(pi*m/8)
template <int DIR>
__device__ __forceinline__ float2 rot(float2 a, float c, float s) {
  return make_float2(a.x * c - DIR * a.y * s, a.y * c + DIR * a.x * s);
}

template <int DIR>
__device__ __forceinline__ void bfly2(float2* v) {
  const float2 a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <int DIR>
__device__ __forceinline__ void bfly4(float2* v) {
  const float2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
  const float2 b0 = cadd(v[1], v[3]), b1 = mul_i<DIR>(csub(v[1], v[3]));
  v[0] = cadd(a0, b0);
  v[2] = csub(a0, b0);
  v[1] = cadd(a1, b1);
  v[3] = csub(a1, b1);
}

#define LP_C8 0.92387953251128675613f  // cos(pi/8)
#define LP_S8 0.38268343236508977173f  // sin(pi/8)
#define LP_R2 0.70710678118654752440f  // cos(pi/4)

template <int DIR>
__device__ __forceinline__ void bfly8(float2* v) {
  float2 e[4] = {v[0], v[2], v[4], v[6]};
  float2 o[4] = {v[1], v[3], v[5], v[7]};
  bfly4<DIR>(e);
  bfly4<DIR>(o);
  const float2 t1 = rot<DIR>(o[1], LP_R2, LP_R2);
  const float2 t2 = mul_i<DIR>(o[2]);
  const float2 t3 = rot<DIR>(o[3], -LP_R2, LP_R2);
  v[0] = cadd(e[0], o[0]);
  v[4] = csub(e[0], o[0]);
  v[1] = cadd(e[1], t1);
  v[5] = csub(e[1], t1);
  v[2] = cadd(e[2], t2);
  v[6] = csub(e[2], t2);
  v[3] = cadd(e[3], t3);
  v[7] = csub(e[3], t3);
}

// 16 = 4 x 4: X[c + 4d] = sum_b w4^(bd) w16^(bc) sum_a v[b + 4a] w4^(ac)
template <int DIR>
__device__ __forceinline__ void bfly16(float2* v) {
  float2 u[16];
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    float2 t[4] = {v[b], v[b + 4], v[b + 8], v[b + 12]};
    bfly4<DIR>(t);
#pragma unroll
    for (int c = 0; c < 4; ++c) u[4 * b + c] = t[c];
  }
  // twiddles w16^(b*c): exponents 0,1,2,3 / 2,4,6 / 3,6,9
  u[5] = rot<DIR>(u[5], LP_C8, LP_S8);
  u[6] = rot<DIR>(u[6], LP_R2, LP_R2);
  u[7] = rot<DIR>(u[7], LP_S8, LP_C8);
  u[9] = rot<DIR>(u[9], LP_R2, LP_R2);
  u[10] = mul_i<DIR>(u[10]);
  u[11] = rot<DIR>(u[11], -LP_R2, LP_R2);
  u[13] = rot<DIR>(u[13], LP_S8, LP_C8);
  u[14] = rot<DIR>(u[14], -LP_R2, LP_R2);
  u[15] = rot<DIR>(u[15], -LP_C8, -LP_S8);
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float2 t[4] = {u[c], u[4 + c], u[8 + c], u[12 + c]};
    bfly4<DIR>(t);
#pragma unroll
    for (int d = 0; d < 4; ++d) v[c + 4 * d] = t[d];
  }
}

template <int DIR>
__device__ __forceinline__ void bfly3(float2* v) {
  const float c = -0.5f, s = DIR * 0.86602540378443864676f;
  const float2 t = cadd(v[1], v[2]);
  const float2 d = csub(v[1], v[2]);
  const float2 m = make_float2(v[0].x + c * t.x, v[0].y + c * t.y);
  const float2 r = make_float2(-s * d.y, s * d.x);
  v[0] = cadd(v[0], t);
  v[1] = cadd(m, r);
  v[2] = csub(m, r);
}

template <int DIR>
__device__ __forceinline__ void bfly5(float2* v) {
  const float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;
  const float s1 = DIR * 0.95105651629515357212f, s2 = DIR * 0.58778525229247312917f;
  const float2 t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
  const float2 d1 = csub(v[1], v[4]), d2 = csub(v[2], v[3]);
  const float2 m1 = make_float2(v[0].x + c1 * t1.x + c2 * t2.x, v[0].y + c1 * t1.y + c2 * t2.y);
  const float2 m2 = make_float2(v[0].x + c2 * t1.x + c1 * t2.x, v[0].y + c2 * t1.y + c1 * t2.y);
  const float2 r1 = make_float2(-(s1 * d1.y + s2 * d2.y), s1 * d1.x + s2 * d2.x);
  const float2 r2 = make_float2(-(s2 * d1.y - s1 * d2.y), s2 * d1.x - s1 * d2.x);
  v[0] = cadd(v[0], cadd(t1, t2));
  v[1] = cadd(m1, r1);
  v[4] = csub(m1, r1);
  v[2] = cadd(m2, r2);
  v[3] = csub(m2, r2);
}

// twiddle exp(DIR*2*pi*i*t/L) from the table
template <int DIR>
__device__ __forceinline__ float2 twid(const float2* __restrict__ tw, int t) {
  float2 w = __ldg(tw + t);
  if (DIR > 0) w.y = -w.y;
  return w;
}

// Direct DFT of radix R with roots from the table (L/R * q steps).
template <int DIR>
__device__ __forceinline__ void bfly_direct(float2* v, int R, const float2* __restrict__ tw, int LoverR) {
  float2 out[7];
  for (int q = 0; q < R; ++q) {
    float2 acc = v[0];
    for (int i = 1; i < R; ++i) acc = cadd(acc, cmul(v[i], twid<DIR>(tw, ((i * q) % R) * LoverR)));
    out[q] = acc;
  }
  for (int q = 0; q < R; ++q) v[q] = out[q];
}

// One Stockham stage with compile-time radix R over `nfft` signals of length L
// whose planes start `stride` floats apart.  Ns = product of the radices already applied.
template <int DIR, int R>
__device__ __forceinline__ void fft_stage(const CBuf in, const CBuf out, const float2* __restrict__ tw, int L,
                                          int Ns, int nfft, int stride) {
  const int Lr = L / R;
  const int total = nfft * Lr;
  const int tstep = L / (Ns * R);
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int f = t / Lr;
    const int j = t - f * Lr;
    const int k = j % Ns;
    const CBuf src = in.offset(f * stride);
    const CBuf dst = out.offset(f * stride);
    float2 v[R];
#pragma unroll
    for (int i = 0; i < R; ++i) v[i] = src.get(j + i * Lr);
    if (Ns > 1) {
#pragma unroll
      for (int i = 1; i < R; ++i) v[i] = cmul(v[i], twid<DIR>(tw, i * k * tstep));
    }
    if (R == 2) bfly2<DIR>(v);
    else if (R == 4) bfly4<DIR>(v);
    else if (R == 8) bfly8<DIR>(v);
    else if (R == 16) bfly16<DIR>(v);
    else if (R == 3) bfly3<DIR>(v);
    else if (R == 5) bfly5<DIR>(v);
    else if (R == 7) bfly_direct<DIR>(v, 7, tw, L / R);
    const int base = (j - k) * R + k;
#pragma unroll
    for (int i = 0; i < R; ++i) dst.set(base + i * Ns, v[i]);
  }
}

// Odd radix 11 or 13, one thread per butterfly.  The thread's R
// inputs belong to its butterfly alone, so they are twiddled and folded in place in
// the source buffer: S_i = x_i + x_{R-i} and D_i = x_i - x_{R-i}, i = 1..h, h = (R-1)/2.
// With c = cos(2 pi i q / R) and s = sin(2 pi i q / R),
//   X_0 = x_0 + sum_i S_i,  X_q = x_0 + A_q + DIR i B_q,  X_{R-q} = x_0 + A_q - DIR i B_q,
// A_q = sum_i S_i c, B_q = sum_i D_i s, so an output pair costs h complex-by-real
// products of each kind.  The root index i q mod R advances by additions; the roots
// come from the length-L table (exp(-2 pi i t / L) at t = m L / R).
template <int DIR>
__device__ void fft_stage_dyn_serial(const CBuf in, const CBuf out, const float2* __restrict__ tw, int L, int Ns, int R,
                              int nfft, int stride) {
  const int Lr = L / R;
  const int total = nfft * Lr;
  const int tstep = L / (Ns * R);
  const int h = (R - 1) / 2;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int f = t / Lr;
    const int j = t - f * Lr;
    const int k = j % Ns;
    const CBuf src = in.offset(f * stride);
    const CBuf dst = out.offset(f * stride);
    const int base = (j - k) * R + k;
    if (Ns > 1)
      for (int i = 1; i < R; ++i) src.set(j + i * Lr, cmul(src.get(j + i * Lr), twid<DIR>(tw, i * k * tstep)));
    const float2 x0 = src.get(j);
    float2 sum = x0;
    for (int i = 1; i <= h; ++i) {
      const float2 a = src.get(j + i * Lr), b = src.get(j + (R - i) * Lr);
      const float2 si = cadd(a, b);
      src.set(j + i * Lr, si);
      src.set(j + (R - i) * Lr, csub(a, b));
      sum = cadd(sum, si);
    }
    dst.set(base, sum);
    for (int q = 1; q <= h; ++q) {
      float2 A = make_float2(0.f, 0.f), B = make_float2(0.f, 0.f);
      int m = 0;
      for (int i = 1; i <= h; ++i) {
        m += q;
        if (m >= R) m -= R;
        const float2 w = __ldg(tw + m * Lr);  // (cos, -sin) of 2 pi m / R
        const float2 si = src.get(j + i * Lr), di = src.get(j + (R - i) * Lr);
        A.x += si.x * w.x;
        A.y += si.y * w.x;
        B.x -= di.x * w.y;
        B.y -= di.y * w.y;
      }
      // DIR i B = (-DIR B.y, DIR B.x)
      const float2 iB = make_float2(-DIR * B.y, DIR * B.x);
      dst.set(base + q * Ns, cadd(cadd(x0, A), iB));
      dst.set(base + (R - q) * Ns, csub(cadd(x0, A), iB));
    }
  }
}

// A prime radix above 13 the planner leaves (17, 19, ...), output-parallel (with few
// butterflies per signal, one thread per butterfly would leave most threads idle).
// Phase 1, one (signal, butterfly, i) item per thread step: twiddle x_i and x_{R-i}
// in place and fold them into S_i = x_i + x_{R-i} (at i) and D_i = x_i - x_{R-i} (at
// R - i), i = 1..h, h = (R-1)/2.  Phase 2, one (signal, butterfly, q) unit per thread
// step: with c = cos(2 pi i q / R) and s = sin(2 pi i q / R),
//   X_0 = x_0 + sum_i S_i,  X_q = x_0 + A_q + DIR i B_q,  X_{R-q} = x_0 + A_q - DIR i B_q,
// A_q = sum_i S_i c, B_q = sum_i D_i s, written straight to the output buffer (the
// stage is out of place).  The root index i q mod R advances by additions; the roots
// come from the length-L table (exp(-2 pi i t / L) at t = m L / R).  Every thread of
// the block calls it (one barrier between the phases).
template <int DIR>
__device__ void fft_stage_dyn(const CBuf in, const CBuf out, const float2* __restrict__ tw, int L, int Ns, int R,
                              int nfft, int stride) {
  const int Lr = L / R;
  const int tstep = L / (Ns * R);
  const int h = (R - 1) / 2;
  // items and units are numbered with i (q) outermost, so the lanes of a warp work on
  // consecutive butterflies with the same i (q): conflict-free shared loads and one
  // root for the whole warp
  const int nb = nfft * Lr;
  for (int it = threadIdx.x; it < nb * h; it += blockDim.x) {
    const int i = 1 + it / nb;
    const int t = it - (i - 1) * nb;
    const int f = t / Lr;
    const int j = t - f * Lr;
    const int k = j % Ns;
    const CBuf src = in.offset(f * stride);
    float2 a = src.get(j + i * Lr), b = src.get(j + (R - i) * Lr);
    if (Ns > 1) {
      a = cmul(a, twid<DIR>(tw, i * k * tstep));
      b = cmul(b, twid<DIR>(tw, (R - i) * k * tstep));
    }
    src.set(j + i * Lr, cadd(a, b));
    src.set(j + (R - i) * Lr, csub(a, b));
  }
  __syncthreads();
  for (int u = threadIdx.x; u < nb * (h + 1); u += blockDim.x) {
    const int q = u / nb;
    const int t = u - q * nb;
    const int f = t / Lr;
    const int j = t - f * Lr;
    const int k = j % Ns;
    const CBuf src = in.offset(f * stride);
    const CBuf dst = out.offset(f * stride);
    const int base = (j - k) * R + k;
    const float2 x0 = src.get(j);
    if (q == 0) {
      float2 sum = x0;
      for (int i = 1; i <= h; ++i) sum = cadd(sum, src.get(j + i * Lr));
      dst.set(base, sum);
      continue;
    }
    float2 A = make_float2(0.f, 0.f), B = make_float2(0.f, 0.f);
    int m = 0;
    for (int i = 1; i <= h; ++i) {
      m += q;
      if (m >= R) m -= R;
      const float2 w = __ldg(tw + m * Lr);  // (cos, -sin) of 2 pi m / R
      const float2 si = src.get(j + i * Lr), di = src.get(j + (R - i) * Lr);
      A.x += si.x * w.x;
      A.y += si.y * w.x;
      B.x -= di.x * w.y;
      B.y -= di.y * w.y;
    }
    // DIR i B = (-DIR B.y, DIR B.x)
    const float2 iB = make_float2(-DIR * B.y, DIR * B.x);
    dst.set(base + q * Ns, cadd(cadd(x0, A), iB));
    dst.set(base + (R - q) * Ns, csub(cadd(x0, A), iB));
  }
}

// Run the transform on `nfft` signals; data starts in `a`, `b` is scratch of
// the same shape.  Returns the buffer holding the result.  All threads of the
// block must call it; it ends with a __syncthreads().
template <int DIR>
__device__ CBuf fft_block(CBuf a, CBuf b, const FFTPlan& p, int nfft, int stride) {
  int Ns = 1;
  CBuf in = a, out = b;
  for (int s = 0; s < p.nst; ++s) {
    const int R = p.radix[s];
    switch (R) {
      case 16: fft_stage<DIR, 16>(in, out, p.tw, p.L, Ns, nfft, stride); break;
      case 8: fft_stage<DIR, 8>(in, out, p.tw, p.L, Ns, nfft, stride); break;
      case 4: fft_stage<DIR, 4>(in, out, p.tw, p.L, Ns, nfft, stride); break;
      case 2: fft_stage<DIR, 2>(in, out, p.tw, p.L, Ns, nfft, stride); break;
      case 3: fft_stage<DIR, 3>(in, out, p.tw, p.L, Ns, nfft, stride); break;
      case 5: fft_stage<DIR, 5>(in, out, p.tw, p.L, Ns, nfft, stride); break;
      case 7: fft_stage<DIR, 7>(in, out, p.tw, p.L, Ns, nfft, stride); break;
      default:
        if (R <= 13) fft_stage_dyn_serial<DIR>(in, out, p.tw, p.L, Ns, R, nfft, stride);
        else fft_stage_dyn<DIR>(in, out, p.tw, p.L, Ns, R, nfft, stride);
        break;
    }
    __syncthreads();
    Ns *= R;
    const CBuf t = in;
    in = out;
    out = t;
  }
  return in;
}

}  // namespace lpgb
