// The hot-path kernels on the register FFT (fft_reg.cuh for powers of two,
// fft_mr.cuh for mixed lengths), templated on the FFT length L.  A signal is
// transformed by T = L/16 threads; blocks carry as many signals as fit in 256
// threads.  Each translation unit instantiates them for its list of lengths
// (LP_DEFINE_LENGTH_SET), so the power-of-two and the mixed lengths compile in
// parallel.
#pragma once
#include <type_traits>

#include "lp_device.cuh"

namespace lpgb {

template <int L>
struct P2 {
  static constexpr bool POW2 = (L & (L - 1)) == 0;
  static constexpr int T = L / 16;                  // threads per signal
  static constexpr int NSIG = T >= 256 ? 1 : 256 / T;
  static constexpr int BLOCK = T * NSIG;
  static constexpr int SLOTS = reg_fft_slots(L);
  // resident blocks per SM to size registers for: as many threads as k blocks of 256
  // (mixed lengths: at most 4, since their odd-radix stages hold up to 26 elements)
  static constexpr int blocks(int k) {
    return (k * 256 / BLOCK > 0 ? k * 256 / BLOCK : 1) > 4 && !POW2 ? 4
         : (k * 256 / BLOCK > 0 ? k * 256 / BLOCK : 1);
  }
};

// forward, per span: Cartesian -> log-polar gather for column pairs, e^rho, FFT along rho.
// The disk points of a column form one rho interval (a.ival), so the two
// columns' points are enumerated as one compact list and gathered in
// straight-line groups of kGatherUnroll per thread (the four quads of a sample
// in flight together) and no fetch is spent outside the disk.  Values land in
// the zeroed shared buffer at their rho position (real part: column th,
// imaginary part: column th+1), from which the register FFT takes its inputs.
// Measured at N=2048: one sample per group with 6 resident blocks per SM
// (40 registers, the shared-memory limit; 8.7 ms per step against 9.0 at 5
// and 9.3 at 4) beats 2, 4 or 8 samples per group with 2-4 blocks: the
// gathers' latency is hidden by more warps rather than by depth per thread.
constexpr int kGatherUnroll = 1;

template <int L>
__global__ void __launch_bounds__(P2<L>::BLOCK, P2<L>::blocks(6)) k_fwd_c2lp_p2(FwdC2LPArgs a) {
  extern __shared__ float2 sm2[];
  constexpr int T = P2<L>::T;
  const int sig = threadIdx.x / T, t = threadIdx.x % T;
  float2* sm = sm2 + sig * P2<L>::SLOTS;
  const int s = blockIdx.x;
  const int th = 2 * ((a.col_lo >> 1) + blockIdx.y * P2<L>::NSIG + sig);
  const bool live = th <= a.col_hi && th < a.Nth;
  const bool has_b = live && th + 1 < a.Nth;
  const int2 ia = live ? __ldg(a.ival + th) : make_int2(1, 0);
  const int2 ib = has_b ? __ldg(a.ival + th + 1) : make_int2(1, 0);
  const int na = max(0, ia.y - ia.x + 1), nb = max(0, ib.y - ib.x + 1);
  const int n = na + nb;
  const float* img = a.fbuf + (size_t)s * a.N * a.N;
  const bool use_tex = a.tex != nullptr;
  const cudaTextureObject_t tx = use_tex ? a.tex[s] : 0;
  const float invN = 1.0f / (float)a.N;
#pragma unroll
  for (int i = 0; i < 16; ++i) sm[spad(t + i * T)] = make_float2(0.f, 0.f);
  __syncthreads();
  float* smf = reinterpret_cast<float*>(sm);
  for (int j0 = 0; j0 < n; j0 += kGatherUnroll * T) {
    float val[kGatherUnroll];
    int pos[kGatherUnroll];
#pragma unroll
    for (int u = 0; u < kGatherUnroll; ++u) {
      const int j = j0 + u * T + t;
      const bool inb = j < n;
      const bool isa = j < na;
      const int r = inb ? (isa ? ia.x + j : ib.x + (j - na)) : 0;
      const int col = (inb && !isa) ? th + 1 : th;
      int2 p = __ldg(a.c2lp + (size_t)col * L + r);
      const bool ok = inb && p.x != LP_FX_NONE;
      if (!ok) p = make_int2(0, 0);
      const float e = __ldg(a.erho + r);
      const float v = use_tex ? interp_tex_cubic_fx(tx, invN, invN, p.x, p.y, a.F, a.fsc)
                              : interp2d_fx(img, a.N, a.N, p.x, p.y, a.F, a.fsc, a.cubic);
      val[u] = ok ? e * v : 0.f;
      pos[u] = inb ? 2 * spad(r) + (isa ? 0 : 1) : -1;
    }
#pragma unroll
    for (int u = 0; u < kGatherUnroll; ++u)
      if (pos[u] >= 0) smf[pos[u]] = val[u];
  }
  __syncthreads();
  float2 v[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = sm[spad(t + i * T)];
  __syncthreads();
  any_fft<L, -1>(v, sm, t);
  if (!live) return;
  float2* out = a.spec + (size_t)s * spec_slice(a.Nk, a.Nth);
  // two consecutive rho frequencies per thread and column: 16-byte stores (the
  // pair k, k+1 of a column is adjacent in the tiled layout; k + 1 = Nk lands
  // in the tile's padding)
  for (int k = 2 * t; k < a.Nk; k += 2 * T) {
    const float2 z1 = sm[spad(k)], z2 = sm[spad(k == 0 ? 0 : L - k)];
    const float2 y1 = sm[spad(k + 1)], y2 = sm[spad(L - k - 1)];
    *reinterpret_cast<float4*>(out + sidx(k, th, a.Nth)) =
        make_float4(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y), 0.5f * (y1.x + y2.x), 0.5f * (y1.y - y2.y));
    if (has_b)
      *reinterpret_cast<float4*>(out + sidx(k, th + 1, a.Nth)) =
          make_float4(0.5f * (z1.y + z2.y), 0.5f * (z2.x - z1.x), 0.5f * (y1.y + y2.y), 0.5f * (y2.x - y1.x));
  }
}

// Theta convolution launch shape: BLK threads (256 or 512, picked per
// geometry by the autotuner) carry NSIG = BLK / T rows (rho frequencies).  Threads are assigned so that the KT = min(4, NSIG) rows of one
// spectrum tile alternate fastest: lane l works on row (l % KT) of the tile and
// theta position t = l / KT, so a warp access covers 32 / KT consecutive theta
// columns of all KT rows -- one contiguous run in the tiled layout.  The rows'
// shared buffers are spaced by 32 / KT extra banks so that the KT rows' accesses
// of one half-warp fall in distinct banks.
template <int L, int BLK>
struct TC {
  static constexpr int T = L / 16;
  static constexpr int NSIG0 = BLK > T ? BLK / T : 1;
  static constexpr int KT = NSIG0 < kSpecTile ? NSIG0 : kSpecTile;
  static constexpr int NSIG = NSIG0 / KT * KT;       // a multiple of KT
  static constexpr int BLOCK = NSIG * T;
  static constexpr int MINB = (L & (L - 1)) == 0 ? 768 / BLOCK : (768 / BLOCK > 4 ? 4 : 768 / BLOCK);
  static constexpr int SLOTS = reg_fft_slots(L) + (KT > 1 ? 16 / KT : 0);
};

// per rho frequency: FFT along theta, multiply by the kernel (which carries the
// 1/(Nrho*Ntheta) of the two unnormalised transforms), inverse; NSIG rows per block
template <int L, int BLK, bool GATHER = false>
__global__ void __launch_bounds__(TC<L, BLK>::BLOCK, TC<L, BLK>::MINB) k_theta_conv_p2(ThetaConvArgs a) {
  extern __shared__ float2 sm2[];
  using C = TC<L, BLK>;
  constexpr int T = C::T, KT = C::KT;
  const int g = threadIdx.x / (KT * T), r = threadIdx.x % (KT * T);
  const int sig = g * KT + r % KT, t = r / KT;
  float2* sm = sm2 + sig * C::SLOTS;
  const int s = blockIdx.x;
  const int k = blockIdx.y * C::NSIG + sig;
  const bool live = k < a.Nk;
  float2* sp = a.spec + (size_t)s * spec_slice(a.Nk, L);
  float2 v[16];
  if constexpr (GATHER) {
    // the block's NSIG frequencies of every row of the span are staged in shared memory
    // after the signals' buffers ([nrows][NSIG]); each column's sum goes through the
    // signal's own buffer slots, so no input register is live across the gather loops
    float2* stg = sm2 + C::NSIG * C::SLOTS;
    const int k0 = blockIdx.y * C::NSIG;
    const float2* rs = a.rowspec + (size_t)s * a.nrows * rowspec_stride(a.Nk);
    for (int q = threadIdx.x; q < a.nrows * C::NSIG; q += C::BLOCK) {
      const int i = q / C::NSIG, kk = k0 + q % C::NSIG;
      stg[q] = kk < a.Nk ? __ldg(rs + (size_t)i * rowspec_stride(a.Nk) + kk) : make_float2(0.f, 0.f);
    }
    __syncthreads();
    // four columns' lists walked side by side (independent load chains)
#pragma unroll 1
    for (int i0 = 0; i0 < 16; i0 += 4) {
      int e[4], e1[4], m = 0;
      float2 acc[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int c = t + (i0 + u) * T;
        const bool in = c >= a.in_lo && c <= a.in_hi;
        e[u] = in ? __ldg(a.coff + c) : 0;
        e1[u] = in ? __ldg(a.coff + c + 1) : 0;
        m = max(m, e1[u] - e[u]);
        acc[u] = make_float2(0.f, 0.f);
      }
      for (int step = 0; step < m; ++step) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          if (e[u] < e1[u]) {
            const int2 q = __ldg(a.cent + e[u]);
            const float w = __int_as_float(q.y);
            const float2 z = stg[q.x * C::NSIG + sig];
            acc[u].x = fmaf(w, z.x, acc[u].x);
            acc[u].y = fmaf(w, z.y, acc[u].y);
            ++e[u];
          }
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) sm[spad(t + (i0 + u) * T)] = acc[u];
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = sm[spad(t + i * T)];
    __syncthreads();  // the transform's first stage writes other threads' slots
  } else {
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int c = t + i * T;
      v[i] = (live && c >= a.in_lo && c <= a.in_hi) ? sp[sidx(k, c, L)] : make_float2(0.f, 0.f);
    }
  }
  // the forward transform leaves X[t + i*T] in v[i]: the kernel multiply needs no
  // shared-memory round trip
  any_fft<L, -1, kOutRegs>(v, sm, t);
  const int kf = live ? k : 0;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const int c = t + i * T;
    float2 w = __ldg(a.fz + sidx(kf, c, L));
    if (a.conj_fz) w.y = -w.y;
    v[i] = cmul(v[i], w);
  }
  any_fft<L, 1>(v, sm, t);
  if (!live) return;
  for (int c = a.out_lo + t; c <= a.out_hi; c += T) sp[sidx(k, c, L)] = sm[spad(c)];
}

// Two rows per thread (used for L <= 4096; at L = 8192 the two rows spill and the
// one-row kernel runs): the thread owns rho frequencies k, k+1 (k even, the same
// tile, adjacent in memory), so one 16-byte access moves both rows' element of a
// theta column, and the two transforms share their twiddles (reg_fft2).  256
// threads carry NP = 256/T row pairs; KP = min(2, NP) pairs alternate fastest
// across lanes (lane l: pair l % KP, position l / KP), so a warp access covers
// 32/KP consecutive columns of 2*KP rows -- contiguous in the tiled layout.  The
// 2*NP row buffers are signal-major (buffer j*NP + p for signal j of pair p) and
// spaced by SLOTS (padded by 8 float2 when KP = 2) so that the pairs of a
// half-warp fall in distinct banks.
template <int L>
struct TC2 {
  static constexpr int T = L / 16;
  static constexpr int NP0 = 256 > T ? 256 / T : 1;
  static constexpr int KP = NP0 < 2 ? NP0 : 2;
  static constexpr int NP = NP0 / KP * KP;           // a multiple of KP
  static constexpr int BLOCK = NP * T;
  static constexpr int SLOTS = reg_fft_slots(L) + (KP > 1 ? 8 : 0);
  static constexpr size_t SMEM = (size_t)2 * NP * SLOTS * sizeof(float2);
};

template <int L>
__global__ void __launch_bounds__(TC2<L>::BLOCK, 512 / TC2<L>::BLOCK) k_theta_conv2_p2(ThetaConvArgs a) {
  extern __shared__ float2 sm2[];
  using C = TC2<L>;
  constexpr int T = C::T, KP = C::KP;
  const int g = threadIdx.x / (KP * T), r = threadIdx.x % (KP * T);
  const int pr = g * KP + r % KP, t = r / KP;
  float2* sm0 = sm2 + pr * C::SLOTS;
  float2* sm1 = sm2 + (C::NP + pr) * C::SLOTS;
  const int s = blockIdx.x;
  const int k = (blockIdx.y * C::NP + pr) * 2;
  const bool live0 = k < a.Nk, live1 = k + 1 < a.Nk;
  float2* sp = a.spec + (size_t)s * spec_slice(a.Nk, L);
  float2 v0[16], v1[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const int c = t + i * T;
    float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
    if (live0 && c >= a.in_lo && c <= a.in_hi) q = *reinterpret_cast<const float4*>(sp + sidx(k, c, L));
    v0[i] = make_float2(q.x, q.y);
    v1[i] = live1 ? make_float2(q.z, q.w) : make_float2(0.f, 0.f);
  }
  any_fft2<L, -1, kOutRegs>(v0, v1, sm0, sm1, t);
  const int kf = live0 ? k : 0;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const int c = t + i * T;
    float4 w = __ldg(reinterpret_cast<const float4*>(a.fz + sidx(kf, c, L)));
    if (a.conj_fz) {
      w.y = -w.y;
      w.w = -w.w;
    }
    v0[i] = cmul(v0[i], make_float2(w.x, w.y));
    v1[i] = cmul(v1[i], make_float2(w.z, w.w));
  }
  any_fft2<L, 1>(v0, v1, sm0, sm1, t);
  if (!live0) return;
  for (int c = a.out_lo + t; c <= a.out_hi; c += T) {
    const float2 y0 = sm0[spad(c)];
    if (live1) {
      const float2 y1 = sm1[spad(c)];
      *reinterpret_cast<float4*>(sp + sidx(k, c, L)) = make_float4(y0.x, y0.y, y1.x, y1.y);
    } else {
      sp[sidx(k, c, L)] = y0;
    }
  }
}


// forward, per span: two angle rows per signal, theta taps combined in frequency,
// inverse FFT along rho, rho interpolation into the caller's sinogram
template <int L>
__global__ void __launch_bounds__(P2<L>::BLOCK, P2<L>::blocks(3)) k_fwd_lp2polar_p2(FwdLP2PolarArgs a) {
  extern __shared__ float2 sm2[];
  constexpr int T = P2<L>::T;
  const int sig = threadIdx.x / T, t = threadIdx.x % T;
  float2* sm = sm2 + sig * P2<L>::SLOTS;
  const int s = blockIdx.x;
  const int i0 = 2 * (blockIdx.y * P2<L>::NSIG + sig);
  const bool live = i0 < a.nrows;
  const int r0 = live ? a.rows[i0] : 0;
  const int r1 = (live && i0 + 1 < a.nrows) ? a.rows[i0 + 1] : -1;
  float w0[4], w1[4];
  const int c0 = axis_weights_fx(__ldg(a.thc + r0), a.F, a.fsc, a.cubic, w0);
  int c1 = 0;
  if (r1 >= 0) {
    c1 = axis_weights_fx(__ldg(a.thc + r1), a.F, a.fsc, a.cubic, w1);
  } else {
    w1[0] = w1[1] = w1[2] = w1[3] = 0.f;
  }
  if (!live) w0[0] = w0[1] = w0[2] = w0[3] = 0.f;
  int t0[4], t1[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    t0[j] = wrapi(c0 + j, a.Nth);
    t1[j] = wrapi(c1 + j, a.Nth);
  }
  const int ntap = a.cubic ? 4 : 2;
  const float2* sp = a.spec + (size_t)s * spec_slice(a.Nk, a.Nth);
  // both rows' taps as offsets into one run of consecutive columns starting at cu
  const int cu = min(c0, r1 >= 0 ? c1 : c0);
  const int nu = max(c0, r1 >= 0 ? c1 : c0) - cu + ntap;
  const bool run = nu <= 8 && cu >= 0 && cu + nu <= a.Nth;
  float u0[8], u1[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int j0 = cu + q - c0, j1 = cu + q - c1;
    u0[q] = (j0 >= 0 && j0 < ntap) ? w0[j0] : 0.f;
    u1[q] = (r1 >= 0 && j1 >= 0 && j1 < ntap) ? w1[j1] : 0.f;
  }
  // two consecutive rho frequencies per thread: one 16-byte load per column
  // (frequencies kk, kk+1 of a column are adjacent in the tiled layout)
#pragma unroll 1
  for (int kk = 2 * t; kk <= L / 2; kk += 2 * T) {
    float4 v0 = make_float4(0.f, 0.f, 0.f, 0.f), v1 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (run) {
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        if (q < nu) {
          const float4 z = *reinterpret_cast<const float4*>(sp + sidx(kk, cu + q, a.Nth));
          v0.x += u0[q] * z.x; v0.y += u0[q] * z.y; v0.z += u0[q] * z.z; v0.w += u0[q] * z.w;
          v1.x += u1[q] * z.x; v1.y += u1[q] * z.y; v1.z += u1[q] * z.z; v1.w += u1[q] * z.w;
        }
      }
    } else {
      for (int j = 0; j < ntap; ++j) {
        const float4 q0 = *reinterpret_cast<const float4*>(sp + sidx(kk, t0[j], a.Nth));
        v0.x += w0[j] * q0.x; v0.y += w0[j] * q0.y; v0.z += w0[j] * q0.z; v0.w += w0[j] * q0.w;
        if (r1 >= 0) {
          const float4 q1 = *reinterpret_cast<const float4*>(sp + sidx(kk, t1[j], a.Nth));
          v1.x += w1[j] * q1.x; v1.y += w1[j] * q1.y; v1.z += w1[j] * q1.z; v1.w += w1[j] * q1.w;
        }
      }
    }
    const float2 a0 = make_float2(v0.x, v0.y), a1 = make_float2(v1.x, v1.y);
    sm[spad(kk)] = pair_elem(kk, L, a0, a1);
    if (kk > 0) sm[spad(L - kk)] = pair_elem(L - kk, L, a0, a1);
    if (kk + 1 <= L / 2) {  // kk + 1 < L / 2 here since kk is even and L / 2 is even
      const float2 b0 = make_float2(v0.z, v0.w), b1 = make_float2(v1.z, v1.w);
      sm[spad(kk + 1)] = pair_elem(kk + 1, L, b0, b1);
      sm[spad(L - kk - 1)] = pair_elem(L - kk - 1, L, b0, b1);
    }
  }
  __syncthreads();
  float2 v[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = sm[spad(t + i * T)];
  __syncthreads();
  // rho coordinates of both rows' N = 8 T polar points, loaded while the FFT runs
  int tr0[8], tr1[8];
#pragma unroll
  for (int m = 0; m < 8; ++m) {
    tr0[m] = __ldg(a.rhoc + (size_t)r0 * a.N + t + m * T);
    tr1[m] = __ldg(a.rhoc + (size_t)max(r1, 0) * a.N + t + m * T);
  }
  any_fft<L, 1>(v, sm, t);
  if (!live) return;
  const bool o0 = r0 % a.os == 0, o1 = r1 >= 0 && r1 % a.os == 0;
  float* out0 = a.Rout + ((size_t)s * a.Nproj0 + r0 / a.os) * a.N0;
  float* out1 = a.Rout + ((size_t)s * a.Nproj0 + max(r1, 0) / a.os) * a.N0;
#pragma unroll
  for (int m = 0; m < 8; ++m) {
    const int x = t + m * T;
    const int xo = x - a.cor_off;
    if (xo < 0 || xo >= a.N0) continue;
    if (o0) out0[xo] = interp1d_fx([&](int i) { return sm[spad(i)].x; }, L, tr0[m], a.F, a.fsc, a.cubic);
    if (o1) out1[xo] = interp1d_fx([&](int i) { return sm[spad(i)].y; }, L, tr1[m], a.F, a.fsc, a.cubic);
  }
}

// adjoint ingest for N = L/2: one pair of input rows per block of T threads
template <int L>
__global__ void __launch_bounds__(P2<L>::BLOCK, P2<L>::blocks(3)) k_adj_ingest_p2(AdjIngestArgs a) {
  extern __shared__ float2 sm2[];
  constexpr int T = P2<L>::T;
  const int N = L / 2;
  const bool filt = a.H != nullptr;
  float2* sm = sm2;
  const int half = T / 2;
  const int C = line_chunk(N, half);
  const int LF = line_floats(N, half);
  float* lines = reinterpret_cast<float*>(sm2 + (filt ? P2<L>::SLOTS : 0));  // 2 rows, chunked layout
  float* cp = lines + 2 * LF;
  const int t = threadIdx.x;
  const int s = blockIdx.x;
  const int q0 = 2 * blockIdx.y;
  const int q1 = q0 + 1 < a.Nproj0 ? q0 + 1 : -1;
  const float* in0 = a.Rin + ((size_t)s * a.Nproj0 + q0) * a.N0;
  const float* in1 = a.Rin + ((size_t)s * a.Nproj0 + max(q1, 0)) * a.N0;
  if (filt) {
    float2 v[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int x = t + i * T;
      const int xi = min(max(x - a.cor_off, 0), a.N0 - 1);
      v[i] = x < N ? make_float2(__ldg(in0 + xi), q1 >= 0 ? __ldg(in1 + xi) : 0.f) : make_float2(0.f, 0.f);
    }
    // filter spectrum multiply and line stores straight from registers (v[i] = X[t + i*T])
    any_fft<L, -1, kOutRegs>(v, sm, t);
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = cscale(v[i], __ldg(a.H + t + i * T));
    any_fft<L, 1, kOutRegs>(v, sm, t);
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int x = t + i * T;
      if (x < N) {
        lines[lpos(x, C)] = v[i].x;
        lines[LF + lpos(x, C)] = v[i].y;
      }
    }
  } else {
    for (int x = t; x < N; x += T) {
      const int xi = min(max(x - a.cor_off, 0), a.N0 - 1);
      lines[lpos(x, C)] = __ldg(in0 + xi);
      lines[LF + lpos(x, C)] = q1 >= 0 ? __ldg(in1 + xi) : 0.f;
    }
  }
  __syncthreads();
  if (a.cubic) {
    const int which = t >= half;
    prefilter_line(lines + which * LF, cp + which * LF, N, t - which * half, half);
  }
  for (int rr = 0; rr < 2; ++rr) {
    const int q = rr == 0 ? q0 : q1;
    if (q < 0) break;
    for (int j = 0; j < a.os; ++j) {
      float* dst = a.rbuf + ((size_t)s * a.Nproj + (size_t)q * a.os + j) * N;
      for (int x = t; x < N; x += T) dst[x] = j == 0 ? lines[rr * LF + lpos(x, C)] : 0.f;
    }
  }
}

// adjoint, per span: polar -> log-polar for a column pair per signal, FFT along rho
template <int L>
__global__ void __launch_bounds__(P2<L>::BLOCK, P2<L>::blocks(4)) k_adj_polar2lp_p2(AdjPolar2LPArgs a) {
  extern __shared__ float2 sm2[];
  constexpr int T = P2<L>::T;
  const int N = L / 2;
  const int sig = threadIdx.x / T, t = threadIdx.x % T;
  float2* sm = sm2 + sig * P2<L>::SLOTS;
  float* prof = reinterpret_cast<float*>(sm2 + P2<L>::NSIG * P2<L>::SLOTS) + sig * 2 * N;
  const int s = blockIdx.x;
  const int th0 = a.clo + 2 * (blockIdx.y * P2<L>::NSIG + sig);
  const bool live = th0 <= a.chi;
  const int th1 = (live && th0 + 1 <= a.chi) ? th0 + 1 : -1;
  const float* img = a.rbuf + (size_t)s * a.Nproj * N;
  const int ta0 = live ? __ldg(a.ta + th0) : LP_FX_NONE;
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
  // N / T = 8 profile points per thread; the loads of all taps are issued
  // before any is used (straight-line, no per-point branches)
  if (!has0) w0[0] = w0[1] = w0[2] = w0[3] = 0.f;
  if (!has1) w1[0] = w1[1] = w1[2] = w1[3] = 0.f;
#pragma unroll
  for (int m = 0; m < N / T; ++m) {
    const int x = t + m * T;
    float p0 = 0.f, p1 = 0.f;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (j < ntap) {
        p0 += w0[j] * (has0 ? __ldg(img + (size_t)rw0[j] * N + x) : 0.f);
        p1 += w1[j] * (has1 ? __ldg(img + (size_t)rw1[j] * N + x) : 0.f);
      }
    }
    prof[x] = p0;
    prof[N + x] = p1;
  }
  __syncthreads();
  const int* sx0 = a.sx + (size_t)(live ? th0 : 0) * L;
  const int* sx1 = a.sx + (size_t)max(th1, 0) * L;
  int xs0[16], xs1[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    xs0[i] = live ? __ldg(sx0 + t + i * T) : LP_FX_NONE;
    xs1[i] = th1 >= 0 ? __ldg(sx1 + t + i * T) : LP_FX_NONE;
  }
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const bool ok0 = xs0[i] != LP_FX_NONE, ok1 = xs1[i] != LP_FX_NONE;
    const float v0 = interp1d_fx([&](int q) { return prof[q]; }, N, ok0 ? xs0[i] : 0, a.F, a.fsc, a.cubic);
    const float v1 = interp1d_fx([&](int q) { return prof[N + q]; }, N, ok1 ? xs1[i] : 0, a.F, a.fsc, a.cubic);
    sm[spad(t + i * T)] = make_float2(ok0 ? v0 : 0.f, ok1 ? v1 : 0.f);
  }
  __syncthreads();
  // wrap points (distinct rho within a column) add a direct 2-D sample
  for (int c = 0; c < 2; ++c) {
    const int th = c == 0 ? th0 : th1;
    if (!live || th < 0) continue;
    const int wb = __ldg(a.woff + th), we = __ldg(a.woff + th + 1);
    for (int w = wb + t; w < we; w += T) {
      const int4 p = __ldg(a.wpt + w);
      const int r = p.x;
      const float val = interp2d_fx(img, N, a.Nproj, p.y, p.z, a.F, a.fsc, a.cubic);
      if (c == 0) sm[spad(r)].x += val;
      else sm[spad(r)].y += val;
    }
  }
  __syncthreads();
  float2 v[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = sm[spad(t + i * T)];
  __syncthreads();
  any_fft<L, -1>(v, sm, t);
  if (!live) return;
  float2* out = a.spec + (size_t)s * spec_slice(a.Nk, a.Nth);
  // frequencies k, k+1 of a column in one 16-byte store (k + 1 = Nk: tile padding)
  for (int k = 2 * t; k < a.Nk; k += 2 * T) {
    const float2 z1 = sm[spad(k)], z2 = sm[spad(k == 0 ? 0 : L - k)];
    const float2 y1 = sm[spad(k + 1)], y2 = sm[spad(L - k - 1)];
    *reinterpret_cast<float4*>(out + sidx(k, th0, a.Nth)) =
        make_float4(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y), 0.5f * (y1.x + y2.x), 0.5f * (y1.y - y2.y));
    if (th1 >= 0)
      *reinterpret_cast<float4*>(out + sidx(k, th1, a.Nth)) =
          make_float4(0.5f * (z1.y + z2.y), 0.5f * (z2.x - z1.x), 0.5f * (y1.y + y2.y), 0.5f * (y2.x - y1.x));
  }
}

// adjoint, per span: inverse FFT along rho for a column pair per signal
template <int L>
__global__ void __launch_bounds__(P2<L>::BLOCK, P2<L>::blocks(4)) k_adj_lpcols_p2(AdjLPColsArgs a) {
  extern __shared__ float2 sm2[];
  constexpr int T = P2<L>::T;
  const int sig = threadIdx.x / T, t = threadIdx.x % T;
  float2* sm = sm2 + sig * P2<L>::SLOTS;
  const int s = blockIdx.x;
  const int th0 = a.lo2 + 2 * (blockIdx.y * P2<L>::NSIG + sig);
  const bool live = th0 <= a.hi2;
  const int th1 = (live && th0 + 1 <= a.hi2) ? th0 + 1 : -1;
  const float2* sp = a.spec + (size_t)s * spec_slice(a.Nk, a.Nth);
  // frequencies kk, kk+1 of each column in one 16-byte load (kk even)
#pragma unroll
  for (int m = 0; m <= L / 4 / T; ++m) {
    const int kk = 2 * (t + m * T);
    if (kk > L / 2) break;
    float4 q0 = make_float4(0.f, 0.f, 0.f, 0.f), q1 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (live) q0 = *reinterpret_cast<const float4*>(sp + sidx(kk, th0, a.Nth));
    if (th1 >= 0) q1 = *reinterpret_cast<const float4*>(sp + sidx(kk, th1, a.Nth));
    const float2 a0 = make_float2(q0.x, q0.y), a1 = make_float2(q1.x, q1.y);
    sm[spad(kk)] = pair_elem(kk, L, a0, a1);
    if (kk > 0) sm[spad(L - kk)] = pair_elem(L - kk, L, a0, a1);
    if (kk + 1 <= L / 2) {
      const float2 b0 = make_float2(q0.z, q0.w), b1 = make_float2(q1.z, q1.w);
      sm[spad(kk + 1)] = pair_elem(kk + 1, L, b0, b1);
      sm[spad(L - kk - 1)] = pair_elem(L - kk - 1, L, b0, b1);
    }
  }
  __syncthreads();
  float2 v[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = sm[spad(t + i * T)];
  __syncthreads();
  any_fft<L, 1>(v, sm, t);
  if (!live) return;
  float* g0 = a.G + ((size_t)s * a.W2 + (th0 - a.lo2)) * L;
  for (int r = t; r < L; r += T) {
    const float2 z = sm[spad(r)];
    if (a.surf) {
      surf2Dwrite(z.x, a.surf[s], r * (int)sizeof(float), th0 - a.lo2);
      if (th1 >= 0) surf2Dwrite(z.y, a.surf[s], r * (int)sizeof(float), th1 - a.lo2);
    } else {
      g0[r] = z.x;
      if (th1 >= 0) g0[L + r] = z.y;
    }
  }
}


// exact transpose, row stage (k_fwdT_rows) on the register FFT: per signal one
// pair of internal rows of the span; N = L/2 = 8T detector points per row
template <int L>
__global__ void __launch_bounds__(P2<L>::BLOCK, P2<L>::blocks(4)) k_fwdT_rows_p2(FwdTRowsArgs a) {
  extern __shared__ float2 sm2[];
  constexpr int T = P2<L>::T;
  const int sig = threadIdx.x / T, t = threadIdx.x % T;
  float2* sm = sm2 + sig * P2<L>::SLOTS;
  float* smf = reinterpret_cast<float*>(sm);
  const int s = blockIdx.x;
  const int i0 = 2 * (blockIdx.y * P2<L>::NSIG + sig);
  const bool live = i0 < a.nrows;
  const int r0 = live ? a.rows[i0] : -1;
  const int r1 = (live && i0 + 1 < a.nrows) ? a.rows[i0 + 1] : -1;
#pragma unroll
  for (int i = 0; i < 16; ++i) sm[spad(t + i * T)] = make_float2(0.f, 0.f);
  __syncthreads();
  // row 0 accumulates in the real parts, row 1 in the imaginary parts
  rho_scatter_T(a, s, r0, r1, t, T, [&](int q, int bin) -> float& { return smf[2 * spad(bin) + q]; });
  float2 v[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = sm[spad(t + i * T)];
  __syncthreads();
  any_fft<L, -1>(v, sm, t);
  if (!live) return;
  float2* o0 = a.rowspec + ((size_t)s * a.nrows + i0) * rowspec_stride(a.Nk);
  for (int k = t; k < a.Nk; k += T) {
    float2 va, vb;
    split_rows_T(sm[spad(k)], sm[spad(k == 0 ? 0 : L - k)], k, L, &va, &vb);
    o0[k] = va;
    if (r1 >= 0) o0[rowspec_stride(a.Nk) + k] = vb;
  }
}

// exact transpose, column stage (k_fwdT_cols) on the register FFT.  The block's
// NSIG signals (up to 1024 threads) are SL consecutive slices (a power of two
// dividing kGatherSlices) of PAIRS column pairs, so each point's values of the SL
// slices go out as one vector store into the slice-interleaved point list instead
// of SL scattered 4-byte stores.
template <int L>
struct TCols {
  static constexpr int T = L / 16;
  // powers of two: up to kGatherSlices slices in blocks of up to 1024 threads at 64
  // registers; mixed lengths (whose odd stages hold more values) keep the other
  // kernels' blocks, SL the largest power of two dividing their signal count
  static constexpr int FIT = 1024 / T > kGatherSlices ? kGatherSlices : 1024 / T;
  static constexpr int NS0 = P2<L>::NSIG;
  static constexpr int SL = P2<L>::POW2 ? (FIT >= 8 ? 8 : FIT >= 4 ? 4 : FIT >= 2 ? 2 : 1)
                          : (NS0 % 8 == 0 ? 8 : NS0 % 4 == 0 ? 4 : NS0 % 2 == 0 ? 2 : 1);
  static constexpr int NSIG = P2<L>::POW2 ? SL : NS0;
  static constexpr int PAIRS = NSIG / SL;
  static constexpr int BLOCK = NSIG * T;
  static constexpr int MINB = P2<L>::POW2 ? (1024 / BLOCK > 0 ? 1024 / BLOCK : 1) : P2<L>::blocks(4);
};

template <int N>
__device__ __forceinline__ void store_vec(float* p, const float* v) {
  if constexpr (N == 8) {
    reinterpret_cast<float4*>(p)[0] = make_float4(v[0], v[1], v[2], v[3]);
    reinterpret_cast<float4*>(p)[1] = make_float4(v[4], v[5], v[6], v[7]);
  } else if constexpr (N == 4) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  } else if constexpr (N == 2) {
    *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
  } else {
    *p = v[0];
  }
}

template <int L>
__global__ void __launch_bounds__(TCols<L>::BLOCK, TCols<L>::MINB)
    k_fwdT_cols_p2(FwdTColsArgs a, int S) {
  extern __shared__ float2 sm2[];
  using C = TCols<L>;
  constexpr int T = P2<L>::T, SL = C::SL;
  const int sig = threadIdx.x / T, t = threadIdx.x % T;
  float2* sm = sm2 + sig * P2<L>::SLOTS;
  const int s0 = blockIdx.x * SL;  // the block's first slice (SL divides kGatherSlices)
  const int s = s0 + sig % SL;
  const int pr = blockIdx.y * C::PAIRS + sig / SL;
  const int th0 = a.dlo + 2 * pr;
  const bool live = th0 <= a.dhi && s < S;
  const int th1 = (live && th0 + 1 <= a.dhi) ? th0 + 1 : -1;
  const float2* sp = a.spec + (size_t)(live ? s : 0) * spec_slice(a.Nk, a.Nth);
#pragma unroll
  for (int m = 0; m <= L / 4 / T; ++m) {
    const int kk = 2 * (t + m * T);
    if (kk > L / 2) break;
    float4 q0 = make_float4(0.f, 0.f, 0.f, 0.f), q1 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (live) q0 = *reinterpret_cast<const float4*>(sp + sidx(kk, th0, a.Nth));
    if (th1 >= 0) q1 = *reinterpret_cast<const float4*>(sp + sidx(kk, th1, a.Nth));
    // b_k: 1 at k = 0 and L/2 (kk + 1 < L/2 always), 1/2 elsewhere
    const float b0 = kk == 0 || kk == L / 2 ? 1.f : 0.5f;
    const float2 a0 = cscale(make_float2(q0.x, q0.y), b0), a1 = cscale(make_float2(q1.x, q1.y), b0);
    sm[spad(kk)] = pair_elem(kk, L, a0, a1);
    if (kk > 0) sm[spad(L - kk)] = pair_elem(L - kk, L, a0, a1);
    if (kk + 1 <= L / 2) {
      const float2 c0 = cscale(make_float2(q0.z, q0.w), 0.5f), c1 = cscale(make_float2(q1.z, q1.w), 0.5f);
      sm[spad(kk + 1)] = pair_elem(kk + 1, L, c0, c1);
      sm[spad(L - kk - 1)] = pair_elem(L - kk - 1, L, c0, c1);
    }
  }
  __syncthreads();
  float2 v[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = sm[spad(t + i * T)];
  __syncthreads();
  any_fft<L, 1>(v, sm, t);
  __syncthreads();  // the stores below read every signal's buffer
  // each point's values of the SL slices to its place in the cell-sorted list (slices
  // past S write their slots too: padding of the group, never read)
  float* g0 = a.G + (size_t)(s0 / kGatherSlices) * a.npts * kGatherSlices + s0 % kGatherSlices;
  for (int q = threadIdx.x; q < C::PAIRS * 2 * L; q += C::BLOCK) {
    const int p = q / (2 * L), c = (q / L) & 1, r = q % L;
    const int th = a.dlo + 2 * (blockIdx.y * C::PAIRS + p) + c;
    if (th > a.dhi) continue;
    const int e = __ldg(a.pos + (size_t)(th - a.dlo) * L + r);
    if (e < 0) continue;
    const float er = __ldg(a.erho + r);
    float vals[SL];
#pragma unroll
    for (int j = 0; j < SL; ++j) {
      const float2 z = sm2[(p * SL + j) * P2<L>::SLOTS + spad(r)];
      vals[j] = er * (c == 0 ? z.x : z.y);
    }
    store_vec<SL>(g0 + (size_t)e * kGatherSlices, vals);
  }
}

// ---- launchers: one per kernel, for any length of a compile-time list ---------
template <int... Ls>
struct Lengths {};

template <class F>
bool with_length(int, Lengths<>, F&&) {
  return false;
}
template <int L0, int... Ls, class F>
bool with_length(int L, Lengths<L0, Ls...>, F&& f) {
  if (L == L0) {
    f(std::integral_constant<int, L0>());
    return true;
  }
  return with_length(L, Lengths<Ls...>(), f);
}

bool smem_fits(size_t need);

template <int L>
void set_len_attrs(int optin) {
  cudaFuncSetAttribute(k_fwd_c2lp_p2<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  cudaFuncSetAttribute(k_theta_conv_p2<L, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  cudaFuncSetAttribute(k_theta_conv_p2<L, 512>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  cudaFuncSetAttribute(k_theta_conv_p2<L, 256, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  if constexpr (L <= 4096) cudaFuncSetAttribute(k_theta_conv2_p2<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  cudaFuncSetAttribute(k_fwd_lp2polar_p2<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  if constexpr (L >= 512) cudaFuncSetAttribute(k_adj_ingest_p2<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  cudaFuncSetAttribute(k_adj_polar2lp_p2<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  cudaFuncSetAttribute(k_adj_lpcols_p2<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  cudaFuncSetAttribute(k_fwdT_rows_p2<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  cudaFuncSetAttribute(k_fwdT_cols_p2<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
}
template <int... Ls>
cudaError_t set_attrs(Lengths<Ls...>, int optin) {
  (set_len_attrs<Ls>(optin), ...);
  return cudaGetLastError();
}

template <class LS>
bool run_fwd_c2lp(const FwdC2LPArgs& a, int S, cudaStream_t st, cudaError_t* err) {
  if (a.ival == nullptr) return false;
  return with_length(a.Nrho, LS(), [&](auto len) {
    constexpr int LL = decltype(len)::value;
    if (a.col_lo < 0 || a.col_hi >= a.Nth) { *err = cudaErrorInvalidValue; return; }
    const int npairs = a.col_hi < a.col_lo ? 0 : (a.col_hi >> 1) - (a.col_lo >> 1) + 1;
    if (npairs == 0) { *err = cudaSuccess; return; }
    const size_t sm = (size_t)P2<LL>::NSIG * P2<LL>::SLOTS * sizeof(float2);
    if (!smem_fits(sm)) { *err = cudaErrorInvalidConfiguration; return; }
    dim3 grid(S, (npairs + P2<LL>::NSIG - 1) / P2<LL>::NSIG);
    k_fwd_c2lp_p2<LL><<<grid, P2<LL>::BLOCK, sm, st>>>(a);
    *err = cudaGetLastError();
  });
}

// shared memory of the exact transpose's theta convolution (0: not a length of the list)
template <class LS>
size_t theta_gather_smem(int L, int nrows) {
  size_t r = 0;
  with_length(L, LS(), [&](auto len) {
    using C = TC<decltype(len)::value, 256>;
    r = ((size_t)C::NSIG * C::SLOTS + (size_t)nrows * C::NSIG) * sizeof(float2);
  });
  return r;
}

template <class LS>
bool run_theta_conv(const ThetaConvArgs& a, int S, cudaStream_t st, cudaError_t* err) {
  return with_length(a.Nth, LS(), [&](auto len) {
    constexpr int LL = decltype(len)::value;
    // mixed lengths whose FFT ends in an odd stage (T odd: 528, 1008): one row per
    // thread (measured at N = 528: 1.00 against 1.21 ms with two rows per thread; at
    // N = 2016 two rows per thread are faster, 1.29x against 1.40x the power-of-two
    // rate per pixel)
    if (a.rowspec) {
      // exact transpose: the input gathered from the row spectra (one row per thread)
      using C = TC<LL, 256>;
      const size_t sm = ((size_t)C::NSIG * C::SLOTS + (size_t)a.nrows * C::NSIG) * sizeof(float2);
      if (!smem_fits(sm)) { *err = cudaErrorInvalidConfiguration; return; }
      dim3 grid(S, (a.Nk + C::NSIG - 1) / C::NSIG);
      k_theta_conv_p2<LL, 256, true><<<grid, C::BLOCK, sm, st>>>(a);
      *err = cudaGetLastError();
    } else if (a.block == 512 || LL > 4096 || (!P2<LL>::POW2 && pow2_part(LL / 16) == 1)) {
      auto go = [&](auto blk) {
        constexpr int B = decltype(blk)::value;
        using C = TC<LL, B>;
        const size_t sm = (size_t)C::NSIG * C::SLOTS * sizeof(float2);
        if (!smem_fits(sm)) { *err = cudaErrorInvalidConfiguration; return; }
        dim3 grid(S, (a.Nk + C::NSIG - 1) / C::NSIG);
        k_theta_conv_p2<LL, B><<<grid, C::BLOCK, sm, st>>>(a);
        *err = cudaGetLastError();
      };
      if (a.block == 512) go(std::integral_constant<int, 512>());
      else go(std::integral_constant<int, 256>());
    } else {
      if constexpr (LL <= 4096) {
        using C = TC2<LL>;
        if (!smem_fits(C::SMEM)) { *err = cudaErrorInvalidConfiguration; return; }
        dim3 grid(S, (a.Nk + 2 * C::NP - 1) / (2 * C::NP));
        k_theta_conv2_p2<LL><<<grid, C::BLOCK, C::SMEM, st>>>(a);
        *err = cudaGetLastError();
      }
    }
  });
}

template <class LS>
bool run_fwd_lp2polar(const FwdLP2PolarArgs& a, int S, cudaStream_t st, cudaError_t* err) {
  return with_length(a.Nrho, LS(), [&](auto len) {
    constexpr int LL = decltype(len)::value;
    if (a.nrows <= 0) { *err = cudaSuccess; return; }
    const size_t sm = (size_t)P2<LL>::NSIG * P2<LL>::SLOTS * sizeof(float2);
    if (!smem_fits(sm)) { *err = cudaErrorInvalidConfiguration; return; }
    const int pairs = (a.nrows + 1) / 2;
    dim3 grid(S, (pairs + P2<LL>::NSIG - 1) / P2<LL>::NSIG);
    k_fwd_lp2polar_p2<LL><<<grid, P2<LL>::BLOCK, sm, st>>>(a);
    *err = cudaGetLastError();
  });
}

template <class LS>
bool run_adj_ingest(const AdjIngestArgs& a, int S, cudaStream_t st, cudaError_t* err) {
  const int L = 2 * a.N;
  if (L < 512) return false;  // T = L/16 >= 32: a warp per row pair, 16 threads per line's prefilter
  return with_length(L, LS(), [&](auto len) {
    constexpr int LL = decltype(len)::value;
    if constexpr (LL >= 512) {
      const size_t sm = (a.H ? (size_t)P2<LL>::SLOTS * sizeof(float2) : 0) +
                        4 * (size_t)line_floats(LL / 2, P2<LL>::T / 2) * sizeof(float);
      if (!smem_fits(sm)) { *err = cudaErrorInvalidConfiguration; return; }
      dim3 grid(S, (a.Nproj0 + 1) / 2);
      k_adj_ingest_p2<LL><<<grid, P2<LL>::T, sm, st>>>(a);
      *err = cudaGetLastError();
    }
  });
}

template <class LS>
bool run_adj_polar2lp(const AdjPolar2LPArgs& a, int S, cudaStream_t st, cudaError_t* err) {
  return with_length(a.Nrho, LS(), [&](auto len) {
    constexpr int LL = decltype(len)::value;
    if (a.chi < a.clo) { *err = cudaSuccess; return; }
    const size_t sm = (size_t)P2<LL>::NSIG * (P2<LL>::SLOTS * sizeof(float2) + (size_t)LL * sizeof(float));
    if (!smem_fits(sm)) { *err = cudaErrorInvalidConfiguration; return; }
    const int pairs = (a.chi - a.clo + 2) / 2;
    dim3 grid(S, (pairs + P2<LL>::NSIG - 1) / P2<LL>::NSIG);
    k_adj_polar2lp_p2<LL><<<grid, P2<LL>::BLOCK, sm, st>>>(a);
    *err = cudaGetLastError();
  });
}

template <class LS>
bool run_adj_lpcols(const AdjLPColsArgs& a, int S, cudaStream_t st, cudaError_t* err) {
  return with_length(a.Nrho, LS(), [&](auto len) {
    constexpr int LL = decltype(len)::value;
    const size_t sm = (size_t)P2<LL>::NSIG * P2<LL>::SLOTS * sizeof(float2);
    if (!smem_fits(sm)) { *err = cudaErrorInvalidConfiguration; return; }
    const int pairs = (a.hi2 - a.lo2 + 2) / 2;
    dim3 grid(S, (pairs + P2<LL>::NSIG - 1) / P2<LL>::NSIG);
    k_adj_lpcols_p2<LL><<<grid, P2<LL>::BLOCK, sm, st>>>(a);
    *err = cudaGetLastError();
  });
}

template <class LS>
bool run_fwdT_rows(const FwdTRowsArgs& a, int S, cudaStream_t st, cudaError_t* err) {
  return with_length(a.Nrho, LS(), [&](auto len) {
    constexpr int LL = decltype(len)::value;
    const int pairs = (a.nrows + 1) / 2;
    const size_t sm = (size_t)P2<LL>::NSIG * P2<LL>::SLOTS * sizeof(float2);
    if (!smem_fits(sm)) { *err = cudaErrorInvalidConfiguration; return; }
    dim3 grid(S, (pairs + P2<LL>::NSIG - 1) / P2<LL>::NSIG);
    k_fwdT_rows_p2<LL><<<grid, P2<LL>::BLOCK, sm, st>>>(a);
    *err = cudaGetLastError();
  });
}

template <class LS>
bool run_fwdT_cols(const FwdTColsArgs& a, int S, cudaStream_t st, cudaError_t* err) {
  return with_length(a.Nrho, LS(), [&](auto len) {
    constexpr int LL = decltype(len)::value;
    using C = TCols<LL>;
    const int npairs = (a.dhi - a.dlo + 2) / 2;
    const size_t sm = (size_t)C::NSIG * P2<LL>::SLOTS * sizeof(float2);
    if (!smem_fits(sm)) { *err = cudaErrorInvalidConfiguration; return; }
    dim3 grid((S + C::SL - 1) / C::SL, (npairs + C::PAIRS - 1) / C::PAIRS);
    k_fwdT_cols_p2<LL><<<grid, C::BLOCK, sm, st>>>(a, S);
    *err = cudaGetLastError();
  });
}

// the register-FFT kernels of one list of lengths (lp_kernels.cu: powers of two;
// lp_kernels_mr.cu: mixed lengths); false when the list does not hold the length
#define LP_DECLARE_LENGTH_SET(PFX)                                                            \
  cudaError_t PFX##_configure(int optin);                                                     \
  bool PFX##_fwd_c2lp(const FwdC2LPArgs& a, int S, cudaStream_t st, cudaError_t* err);        \
  bool PFX##_theta_conv(const ThetaConvArgs& a, int S, cudaStream_t st, cudaError_t* err);    \
  bool PFX##_fwd_lp2polar(const FwdLP2PolarArgs& a, int S, cudaStream_t st, cudaError_t* err); \
  bool PFX##_adj_ingest(const AdjIngestArgs& a, int S, cudaStream_t st, cudaError_t* err);    \
  bool PFX##_adj_polar2lp(const AdjPolar2LPArgs& a, int S, cudaStream_t st, cudaError_t* err); \
  bool PFX##_adj_lpcols(const AdjLPColsArgs& a, int S, cudaStream_t st, cudaError_t* err);    \
  bool PFX##_fwdT_rows(const FwdTRowsArgs& a, int S, cudaStream_t st, cudaError_t* err);      \
  bool PFX##_fwdT_cols(const FwdTColsArgs& a, int S, cudaStream_t st, cudaError_t* err);      \
  bool PFX##_has_length(int L);                                                               \
  size_t PFX##_gather_smem(int L, int nrows);

#define LP_DEFINE_LENGTH_SET(PFX, LIST)                                                           \
  cudaError_t PFX##_configure(int optin) { return set_attrs(LIST(), optin); }                    \
  bool PFX##_fwd_c2lp(const FwdC2LPArgs& a, int S, cudaStream_t st, cudaError_t* err) {          \
    return run_fwd_c2lp<LIST>(a, S, st, err);                                                   \
  }                                                                                              \
  bool PFX##_theta_conv(const ThetaConvArgs& a, int S, cudaStream_t st, cudaError_t* err) {      \
    return run_theta_conv<LIST>(a, S, st, err);                                                 \
  }                                                                                              \
  bool PFX##_fwd_lp2polar(const FwdLP2PolarArgs& a, int S, cudaStream_t st, cudaError_t* err) {  \
    return run_fwd_lp2polar<LIST>(a, S, st, err);                                               \
  }                                                                                              \
  bool PFX##_adj_ingest(const AdjIngestArgs& a, int S, cudaStream_t st, cudaError_t* err) {      \
    return run_adj_ingest<LIST>(a, S, st, err);                                                 \
  }                                                                                              \
  bool PFX##_adj_polar2lp(const AdjPolar2LPArgs& a, int S, cudaStream_t st, cudaError_t* err) {  \
    return run_adj_polar2lp<LIST>(a, S, st, err);                                               \
  }                                                                                              \
  bool PFX##_adj_lpcols(const AdjLPColsArgs& a, int S, cudaStream_t st, cudaError_t* err) {      \
    return run_adj_lpcols<LIST>(a, S, st, err);                                                 \
  }                                                                                              \
  bool PFX##_fwdT_rows(const FwdTRowsArgs& a, int S, cudaStream_t st, cudaError_t* err) {        \
    return run_fwdT_rows<LIST>(a, S, st, err);                                                  \
  }                                                                                              \
  bool PFX##_fwdT_cols(const FwdTColsArgs& a, int S, cudaStream_t st, cudaError_t* err) {        \
    return run_fwdT_cols<LIST>(a, S, st, err);                                                  \
  }                                                                                              \
  bool PFX##_has_length(int L) { return with_length(L, LIST(), [](auto) {}); }                  \
  size_t PFX##_gather_smem(int L, int nrows) { return theta_gather_smem<LIST>(L, nrows); }

LP_DECLARE_LENGTH_SET(p2)
LP_DECLARE_LENGTH_SET(mr)
LP_DECLARE_LENGTH_SET(mr2)
LP_DECLARE_LENGTH_SET(mr3)
LP_DECLARE_LENGTH_SET(mr4)
LP_DECLARE_LENGTH_SET(mr5)

}  // namespace lpgb
