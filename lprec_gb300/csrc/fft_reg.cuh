// Register-resident complex FFT for power-of-two lengths 256..8192.
//
// Each thread of a signal's T = L/16 threads holds 16 elements in registers,
// thread t holding x[t + i*T], i = 0..15.  Every stage is a Stockham step:
// the thread's elements form 16/R butterflies of radix R (elements m, m+NB,
// m+2NB, ... with NB = 16/R), twiddled and transformed in registers, then
// written to their sorted positions in one shared buffer; the next stage
// reads the same natural positions t + i*T back.  The schedule is radix 16
// followed by at most one radix 2/4/8 stage, so L = 4096 takes three stages.
// Index arithmetic is resolved at compile time.  Shared positions carry one
// pad element per 16 (`spad`), which keeps the radix-16 scatter of the first
// stage and the unit-stride reads conflict-free for 64-bit accesses.
//
// Twiddles exp(DIR*2*pi*i*a*k/(Ns*R)) are built per butterfly from two
// sincospif() calls (powers 1 and 4) and short products (depth <= 3), so no
// table is gathered.  On return the transform is in shared memory in
// natural order at spad(k); registers are free.
//
// DIR = -1 forward exp(-2*pi*i*jk/L), DIR = +1 unnormalised inverse.
#pragma once
#include "fft_device.cuh"

namespace lpgb {

__device__ __forceinline__ int spad(int p) { return p + (p >> 4); }
// float2 slots of one padded signal buffer
__host__ __device__ constexpr int reg_fft_slots(int L) { return L + (L >> 4); }

template <int R, int DIR>
__device__ __forceinline__ void reg_bfly(float2* x) {
  if constexpr (R == 16) bfly16<DIR>(x);
  else if constexpr (R == 8) bfly8<DIR>(x);
  else if constexpr (R == 4) bfly4<DIR>(x);
  else bfly2<DIR>(x);
}

// twiddle powers w^i, i < R, from w1 = w and (R >= 8) w4 = w^4
template <int R>
__device__ __forceinline__ void twiddle_powers_from(float2 w1, float2 w4, float2* w) {
  w[0] = make_float2(1.f, 0.f);
  w[1] = w1;
  if constexpr (R >= 4) {
    w[2] = cmul(w1, w1);
    w[3] = cmul(w[2], w1);
  }
  if constexpr (R >= 8) {
    w[4] = w4;
    w[5] = cmul(w4, w1);
    w[6] = cmul(w4, w[2]);
    w[7] = cmul(w4, w[3]);
    if constexpr (R == 16) {
      const float2 w8 = cmul(w4, w4);
      const float2 w12 = cmul(w8, w4);
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        w[8 + a] = a == 0 ? w8 : cmul(w8, w[a]);
        w[12 + a] = a == 0 ? w12 : cmul(w12, w[a]);
      }
    }
  }
}

// twiddle powers w^i, i < R, of w = exp(DIR*2*pi*i*f) with f = k/(Ns*R)
template <int R, int DIR>
__device__ __forceinline__ void twiddle_powers(float f, float2* w) {
  float s1, c1;
  sincospif(2.0f * f, &s1, &c1);
  float2 w4 = make_float2(1.f, 0.f);
  if constexpr (R >= 8) {
    float s4, c4;
    sincospif(8.0f * f, &s4, &c4);
    w4 = make_float2(c4, DIR * s4);
  }
  twiddle_powers_from<R>(make_float2(c1, DIR * s1), w4, w);
}

// cos(pi*m/8) and sin(pi*m/8), m = 0..7 (m is a compile-time constant at every use)
__device__ __forceinline__ float cos_pi8(int m) {
  return m == 0 ? 1.f : m == 1 ? LP_C8 : m == 2 ? LP_R2 : m == 3 ? LP_S8
       : m == 4 ? 0.f : m == 5 ? -LP_S8 : m == 6 ? -LP_R2 : -LP_C8;
}
__device__ __forceinline__ float sin_pi8(int m) {
  return m == 0 ? 0.f : m == 1 ? LP_S8 : m == 2 ? LP_R2 : m == 3 ? LP_C8
       : m == 4 ? 1.f : m == 5 ? LP_C8 : m == 6 ? LP_R2 : LP_S8;
}

// where the last stage leaves the transform
enum RegFftOut { kOutSmem = 0, kOutPlanar = 1, kOutRegs = 2, kOutCall = 3 };

struct NoSink {
  __device__ __forceinline__ void operator()(int, float2) const {}
};

template <int L, int DIR, int R, int NS, bool LAST, int OUT = kOutSmem, class Sink = NoSink>
__device__ __forceinline__ void reg_stage(float2 (&v)[16], float2* sm, int t, const Sink& sink = Sink()) {
  constexpr int T = L / 16;
  constexpr int NB = 16 / R;
  static_assert((OUT != kOutRegs && OUT != kOutCall) || (LAST && NS * R == L),
                "register or sink output only from a last stage spanning L");
  float2 w1_0 = make_float2(1.f, 0.f), w4_0 = make_float2(1.f, 0.f);  // butterfly 0's w and w^4
#pragma unroll
  for (int m = 0; m < NB; ++m) {
    const int jp = t + m * T;
    const int k = (int)((unsigned)jp % (unsigned)NS);  // NS: any product of radices
    float2 x[R];
#pragma unroll
    for (int i = 0; i < R; ++i) x[i] = v[m + i * NB];
    if constexpr (NS > 1) {
      float2 w[R];
      if constexpr (NB > 1) {
        // NB > 1 only in a last stage (R < 16, NS*R = L), where k = t + m*T: butterfly m's
        // base twiddle is butterfly 0's times exp(DIR*i*pi*m/8), its fourth power butterfly
        // 0's times (DIR*i)^m -- one product instead of two sincospif
        static_assert(NS * R == L, "multi-butterfly stages end the transform");
        if (m == 0) {
          twiddle_powers<R, DIR>((float)k * (1.0f / (float)(NS * R)), w);
          w1_0 = w[1];
          if constexpr (R >= 8) w4_0 = w[4];
        } else {
          const float2 w1 = rot<DIR>(w1_0, cos_pi8(m), sin_pi8(m));
          float2 w4 = w4_0;
          if constexpr (R >= 8) {
#pragma unroll
            for (int j = 0; j < (m & 3); ++j) w4 = mul_i<DIR>(w4);
          }
          twiddle_powers_from<R>(w1, w4, w);
        }
      } else {
        twiddle_powers<R, DIR>((float)k * (1.0f / (float)(NS * R)), w);
      }
#pragma unroll
      for (int i = 1; i < R; ++i) x[i] = cmul(x[i], w[i]);
    }
    reg_bfly<R, DIR>(x);
    const int base = (jp - k) * R + k;
    if constexpr (OUT == kOutRegs) {
      // jp < NS here, so output i of this butterfly is element jp + i*NS = t + (m + i*NB)*T:
      // back into the register it came from
#pragma unroll
      for (int i = 0; i < R; ++i) v[m + i * NB] = x[i];
    } else if constexpr (OUT == kOutCall) {
      // the same elements handed to the caller as soon as they exist
#pragma unroll
      for (int i = 0; i < R; ++i) sink(jp + i * NS, x[i]);
    } else if constexpr (OUT == kOutPlanar) {
      float* re = reinterpret_cast<float*>(sm);
      float* im = re + reg_fft_slots(L);
#pragma unroll
      for (int i = 0; i < R; ++i) {
        re[spad(base + i * NS)] = x[i].x;
        im[spad(base + i * NS)] = x[i].y;
      }
    } else {
#pragma unroll
      for (int i = 0; i < R; ++i) sm[spad(base + i * NS)] = x[i];
    }
  }
  if constexpr (OUT != kOutRegs && OUT != kOutCall) __syncthreads();
  if constexpr (!LAST) {
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = sm[spad(t + i * T)];
    __syncthreads();
  }
}

// Transform one signal.  v: this thread's 16 elements x[t + i*T]; sm: the
// signal's shared buffer of reg_fft_slots(L) float2.  All threads of the
// block must call it (it synchronises the block).  OUT:
//   kOutSmem   -- the result in sm in natural order at spad(k), registers free;
//   kOutPlanar -- the same as two float planes (real parts at ((float*)sm)[spad(k)],
//                 imaginary parts reg_fft_slots(L) floats further), so that 4-byte
//                 reads of one part by neighbouring threads fall in distinct banks;
//   kOutRegs   -- the result in registers, v[q] = X[t + q*T]: the distribution the
//                 input had, so a pointwise multiply and another transform (or
//                 stores of a chosen range) follow without a shared-memory round
//                 trip.  sm is free on return (no final barrier).
//   kOutCall   -- the same elements X[t + q*T] passed to sink(t + q*T, value) as the
//                 last stage produces them (registers are released as it goes).
template <int L, int DIR, int OUT = kOutSmem, class Sink = NoSink>
__device__ __forceinline__ void reg_fft(float2 (&v)[16], float2* sm, int t, const Sink& sink = Sink()) {
  static_assert(L == 256 || L == 512 || L == 1024 || L == 2048 || L == 4096 || L == 8192, "size");
  reg_stage<L, DIR, 16, 1, false>(v, sm, t);
  if constexpr (L == 256) {
    reg_stage<L, DIR, 16, 16, true, OUT>(v, sm, t, sink);
  } else if constexpr (L == 8192) {
    reg_stage<L, DIR, 16, 16, false>(v, sm, t);
    reg_stage<L, DIR, 16, 256, false>(v, sm, t);
    reg_stage<L, DIR, 2, 4096, true, OUT>(v, sm, t, sink);
  } else {
    reg_stage<L, DIR, 16, 16, false>(v, sm, t);
    constexpr int R3 = L / 256;
    reg_stage<L, DIR, R3, 256, true, OUT>(v, sm, t, sink);
  }
}

}  // namespace lpgb

namespace lpgb {

// Two signals of the same length on the same threads: thread t holds x0[t + i*T]
// in v0[i] and x1[t + i*T] in v1[i].  Each stage computes its twiddles once and
// applies them to both signals before either butterfly, then transforms and
// writes one signal after the other (so only one butterfly's temporaries are
// live at a time).  Same arithmetic per signal as reg_stage / reg_fft, so each
// result equals the one-signal transform's bit for bit.
template <int L, int DIR, int R, int NS, bool LAST, int OUT>
__device__ __forceinline__ void reg_stage2(float2 (&v0)[16], float2 (&v1)[16], float2* sm0, float2* sm1, int t) {
  constexpr int T = L / 16;
  constexpr int NB = 16 / R;
  static_assert(OUT == kOutSmem || OUT == kOutRegs, "two-signal stages write shared memory or registers");
  static_assert(OUT != kOutRegs || (LAST && NS * R == L), "register output only from a last stage spanning L");
  float2 w1_0 = make_float2(1.f, 0.f), w4_0 = make_float2(1.f, 0.f);
#pragma unroll
  for (int m = 0; m < NB; ++m) {
    const int jp = t + m * T;
    const int k = (int)((unsigned)jp % (unsigned)NS);  // NS: any product of radices
    if constexpr (NS > 1) {
      float2 w[R];
      if constexpr (NB > 1) {
        static_assert(NS * R == L, "multi-butterfly stages end the transform");
        if (m == 0) {
          twiddle_powers<R, DIR>((float)k * (1.0f / (float)(NS * R)), w);
          w1_0 = w[1];
          if constexpr (R >= 8) w4_0 = w[4];
        } else {
          const float2 w1 = rot<DIR>(w1_0, cos_pi8(m), sin_pi8(m));
          float2 w4 = w4_0;
          if constexpr (R >= 8) {
#pragma unroll
            for (int j = 0; j < (m & 3); ++j) w4 = mul_i<DIR>(w4);
          }
          twiddle_powers_from<R>(w1, w4, w);
        }
      } else {
        twiddle_powers<R, DIR>((float)k * (1.0f / (float)(NS * R)), w);
      }
#pragma unroll
      for (int i = 1; i < R; ++i) {
        v0[m + i * NB] = cmul(v0[m + i * NB], w[i]);
        v1[m + i * NB] = cmul(v1[m + i * NB], w[i]);
      }
    }
    const int base = (jp - k) * R + k;
#pragma unroll
    for (int sg = 0; sg < 2; ++sg) {
      float2(&v)[16] = sg == 0 ? v0 : v1;
      float2* sm = sg == 0 ? sm0 : sm1;
      float2 x[R];
#pragma unroll
      for (int i = 0; i < R; ++i) x[i] = v[m + i * NB];
      reg_bfly<R, DIR>(x);
      if constexpr (OUT == kOutRegs) {
#pragma unroll
        for (int i = 0; i < R; ++i) v[m + i * NB] = x[i];
      } else {
#pragma unroll
        for (int i = 0; i < R; ++i) sm[spad(base + i * NS)] = x[i];
      }
    }
  }
  if constexpr (OUT != kOutRegs) __syncthreads();
  if constexpr (!LAST) {
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      v0[i] = sm0[spad(t + i * T)];
      v1[i] = sm1[spad(t + i * T)];
    }
    __syncthreads();
  }
}

// Two-signal transform (see reg_stage2); OUT kOutSmem or kOutRegs as in reg_fft.
template <int L, int DIR, int OUT = kOutSmem>
__device__ __forceinline__ void reg_fft2(float2 (&v0)[16], float2 (&v1)[16], float2* sm0, float2* sm1, int t) {
  static_assert(L == 256 || L == 512 || L == 1024 || L == 2048 || L == 4096 || L == 8192, "size");
  reg_stage2<L, DIR, 16, 1, false, kOutSmem>(v0, v1, sm0, sm1, t);
  if constexpr (L == 256) {
    reg_stage2<L, DIR, 16, 16, true, OUT>(v0, v1, sm0, sm1, t);
  } else if constexpr (L == 8192) {
    reg_stage2<L, DIR, 16, 16, false, kOutSmem>(v0, v1, sm0, sm1, t);
    reg_stage2<L, DIR, 16, 256, false, kOutSmem>(v0, v1, sm0, sm1, t);
    reg_stage2<L, DIR, 2, 4096, true, OUT>(v0, v1, sm0, sm1, t);
  } else {
    reg_stage2<L, DIR, 16, 16, false, kOutSmem>(v0, v1, sm0, sm1, t);
    constexpr int R3 = L / 256;
    reg_stage2<L, DIR, R3, 256, true, OUT>(v0, v1, sm0, sm1, t);
  }
}

}  // namespace lpgb
