// Register FFT for padded lengths that are not powers of two.
//
// The reference pads the image to N = 16 m (src/lprec/initsgl.py:29), so its
// log-polar grids have Ntheta = 16 m and Nrho = 32 m for any m: an off-centre
// rotation axis or an odd detector width gives factors 3, 5, 7, 11, 13.  This
// extends fft_reg.cuh's register Stockham FFT (T = L/16 threads per signal,
// thread t holding x[t + i*T], i < 16) to L = 16 T with T = 2^a * odd, the odd
// part a product of 3, 5, 7, 11 and 13:
//
//   1. radix 16 in registers (stride T: valid for any T);
//   2. one stage per odd prime factor, through the shared buffer: the stage's
//      L/R butterflies of radix R are spread over the T threads (butterfly
//      jp = t + b*T), each loads its R inputs, syncs, twiddles, transforms and
//      writes its R outputs to their sorted positions;
//   3. the remaining power-of-two factor as the usual uniform register stages
//      (radix 16, then 2/4/8), the last one able to leave the result in
//      registers (kOutRegs) as fft_reg.cuh's does.
//
// Odd butterflies fold the inputs into sums and differences of mirrored pairs
// (x_i +- x_{R-i}) so an output pair costs (R-1)/2 real-by-complex products of
// each kind; their roots cos/sin(2 pi m / R) are compile-time constants.  A
// prime factor above 13 (N = 2064 = 16 * 3 * 43 for an axis 3 pixels off centre
// at N0 = 2048) would hold 2R values per thread that way, so it runs output-
// parallel instead (mr_big_stage): the folded sums and differences are formed in
// the shared buffer, then each butterfly's output pairs are split between
// threads that each read the R folded values once and accumulate their pairs
// with compile-time roots.
// Stage twiddles are built from two sincospif() calls per butterfly and short
// products, as in fft_reg.cuh.  Same sign convention (DIR = -1 forward).
#pragma once
#include "fft_reg.cuh"

namespace lpgb {

__host__ __device__ constexpr int pow2_part(int n) {
  int p = 1;
  while (n > 0 && n % 2 == 0) {
    n /= 2;
    p *= 2;
  }
  return p;
}

// smallest of 3, 5, 7, 11, 13 dividing n (0: none)
__host__ __device__ constexpr int small_odd_factor(int n) {
  return n % 3 == 0 ? 3 : n % 5 == 0 ? 5 : n % 7 == 0 ? 7 : n % 11 == 0 ? 11 : n % 13 == 0 ? 13 : 0;
}

// smallest prime factor of odd n > 1
__host__ __device__ constexpr int odd_prime_factor(int n) {
  for (int f = 3; f * f <= n; f += 2)
    if (n % f == 0) return f;
  return n;
}

// the largest prime factor above 13 the output-parallel stage takes (instantiated and
// checked against the oracle at 43; a thread holds about R float2 of accumulators)
constexpr int kBigPrimeMax = 43;

// L = 16 T with T not a power of two, T's odd part a product of primes up to
// kBigPrimeMax, those above 13 each leaving at least one thread per butterfly
__host__ __device__ constexpr bool mr_length(int L) {
  if (L < 32 || L % 16 != 0) return false;
  const int T = L / 16;
  int o = T / pow2_part(T);
  if (o == 1) return false;
  while (o > 1) {
    const int f = odd_prime_factor(o);
    if (f > kBigPrimeMax || (f > 13 && L / f > T)) return false;
    o /= f;
  }
  return true;
}

// cos and sin of 2 pi m / R in double precision, at compile time (Taylor series
// after reducing the angle to [-pi, pi])
__host__ __device__ constexpr double ct_sin_red(double x) {
  double term = x, sum = x;
  for (int n = 1; n < 30; ++n) {
    term *= -x * x / ((2.0 * n) * (2.0 * n + 1.0));
    sum += term;
  }
  return sum;
}
__host__ __device__ constexpr double ct_cos_red(double x) {
  double term = 1.0, sum = 1.0;
  for (int n = 1; n < 30; ++n) {
    term *= -x * x / ((2.0 * n - 1.0) * (2.0 * n));
    sum += term;
  }
  return sum;
}
__host__ __device__ constexpr double ct_angle(int m, int R) {
  const double pi = 3.14159265358979323846264338327950288;
  const int mm = ((m % R) + R) % R;
  return 2.0 * pi * (2 * mm > R ? mm - R : mm) / R;
}
template <int R>
struct PrimeRoots {
  float c[R], s[R];
  constexpr PrimeRoots() : c(), s() {
    for (int m = 0; m < R; ++m) {
      c[m] = (float)ct_cos_red(ct_angle(m, R));
      s[m] = (float)ct_sin_red(ct_angle(m, R));
    }
  }
};

// cos(2 pi m / R), sin(2 pi m / R) for 1 <= m <= (R-1)/2 (m a compile-time constant at every use)
template <int R>
__device__ __forceinline__ float odd_cos(int m) {
  if constexpr (R == 7) {
    return m == 1 ? 0.62348980185873359439f : m == 2 ? -0.22252093395631433737f : -0.90096886790241903498f;
  } else if constexpr (R == 11) {
    return m == 1 ? 0.84125353283118120551f : m == 2 ? 0.41541501300188643508f : m == 3 ? -0.14231483827328500480f
         : m == 4 ? -0.65486073394528498959f : -0.95949297361449736865f;
  } else {
    static_assert(R == 13, "odd radix");
    return m == 1 ? 0.88545602565320991051f : m == 2 ? 0.56806474673115592289f : m == 3 ? 0.12053668025532300601f
         : m == 4 ? -0.35460488704253545489f : m == 5 ? -0.74851074817110119231f : -0.97094181742605201180f;
  }
}
template <int R>
__device__ __forceinline__ float odd_sin(int m) {
  if constexpr (R == 7) {
    return m == 1 ? 0.78183148246802980363f : m == 2 ? 0.97492791218182361934f : 0.43388373911755823142f;
  } else if constexpr (R == 11) {
    return m == 1 ? 0.54064081745559755543f : m == 2 ? 0.90963199535451833011f : m == 3 ? 0.98982144188093279524f
         : m == 4 ? 0.75574957435425826890f : 0.28173255684142967104f;
  } else {
    static_assert(R == 13, "odd radix");
    return m == 1 ? 0.46472317204376850652f : m == 2 ? 0.82298386589365635224f : m == 3 ? 0.99270887409805397272f
         : m == 4 ? 0.93501624268541483342f : m == 5 ? 0.66312265824079519305f : 0.23931566428755768339f;
  }
}

// X_q = sum_n x_n exp(DIR 2 pi i n q / R) for odd prime R, in place
template <int R, int DIR>
__device__ __forceinline__ void bfly_odd(float2* v) {
  if constexpr (R == 3) {
    bfly3<DIR>(v);
  } else if constexpr (R == 5) {
    bfly5<DIR>(v);
  } else {
    constexpr int h = (R - 1) / 2;
    float2 S[h], D[h];
    const float2 x0 = v[0];
    float2 sum = x0;
#pragma unroll
    for (int i = 1; i <= h; ++i) {
      S[i - 1] = cadd(v[i], v[R - i]);
      D[i - 1] = csub(v[i], v[R - i]);
      sum = cadd(sum, S[i - 1]);
    }
    v[0] = sum;
#pragma unroll
    for (int q = 1; q <= h; ++q) {
      float2 A = make_float2(0.f, 0.f), B = make_float2(0.f, 0.f);
#pragma unroll
      for (int i = 1; i <= h; ++i) {
        const int m = (i * q) % R;  // root index; cos is even, sin odd about R/2
        const float c = m <= h ? odd_cos<R>(m) : odd_cos<R>(R - m);
        const float s = m <= h ? odd_sin<R>(m) : -odd_sin<R>(R - m);
        A.x += S[i - 1].x * c;
        A.y += S[i - 1].y * c;
        B.x += D[i - 1].x * s;
        B.y += D[i - 1].y * s;
      }
      const float2 iB = make_float2(-DIR * B.y, DIR * B.x);  // DIR * i * B
      const float2 m0 = cadd(x0, A);
      v[q] = cadd(m0, iB);
      v[R - q] = csub(m0, iB);
    }
  }
}

// w^i, 0 <= i < R, of w = exp(DIR 2 pi i f): two sincospif() calls, products of depth <= 3
template <int R, int DIR>
__device__ __forceinline__ void twiddle_powers_any(float f, float2* w) {
  float s1, c1;
  sincospif(2.0f * f, &s1, &c1);
  const float2 w1 = make_float2(c1, DIR * s1);
  w[0] = make_float2(1.f, 0.f);
  if constexpr (R > 1) w[1] = w1;
  if constexpr (R > 2) w[2] = cmul(w1, w1);
  if constexpr (R > 3) w[3] = cmul(w[2], w1);
  if constexpr (R > 4) {
    float s4, c4;
    sincospif(8.0f * f, &s4, &c4);
    const float2 w4 = make_float2(c4, DIR * s4);
    w[4] = w4;
#pragma unroll
    for (int i = 5; i < R; ++i) {
      if (i < 8) w[i] = cmul(w4, w[i - 4]);
      else if (i == 8) w[i] = cmul(w4, w4);
      else w[i] = cmul(w[8], w[i - 8]);
    }
  }
}

// One odd-radix stage through the shared buffer (see the file comment).  NS is
// the product of the radices already applied.  Ends with a barrier.
template <int L, int DIR, int R, int NS>
__device__ __forceinline__ void mr_odd_stage(float2* sm, int t) {
  constexpr int T = L / 16;
  constexpr int NBUT = L / R;
  constexpr int NBF = (NBUT + T - 1) / T;
  float2 x[NBF][R];
#pragma unroll
  for (int b = 0; b < NBF; ++b) {
    const int jp = t + b * T;
    if (jp < NBUT) {
#pragma unroll
      for (int i = 0; i < R; ++i) x[b][i] = sm[spad(jp + i * NBUT)];
    }
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < NBF; ++b) {
    const int jp = t + b * T;
    if (jp < NBUT) {
      const int k = jp % NS;
      if constexpr (NS > 1) {
        float2 w[R];
        twiddle_powers_any<R, DIR>((float)k * (1.0f / (float)(NS * R)), w);
#pragma unroll
        for (int i = 1; i < R; ++i) x[b][i] = cmul(x[b][i], w[i]);
      }
      bfly_odd<R, DIR>(x[b]);
      const int base = (jp - k) * R + k;
#pragma unroll
      for (int i = 0; i < R; ++i) sm[spad(base + i * NS)] = x[b][i];
    }
  }
  __syncthreads();
}

// output pairs q = Q0 .. Q1 of one folded butterfly (x_0 at p0, S_i at p0 + i stride,
// D_i at p0 + (R - i) stride, i = 1 .. h, in the shared buffer) into out[]: with
// Q0 = 0, out[0] = X_0 and X_q, X_{R-q} at out[2q - 1], out[2q]; otherwise X_q,
// X_{R-q} at out[2 (q - Q0)], out[2 (q - Q0) + 1]
template <int R, int DIR, int Q0, int Q1>
__device__ __forceinline__ void big_prime_pairs(const float2* sm, int p0, int stride, float2* out) {
  constexpr int h = (R - 1) / 2;
  constexpr int NQ = Q1 - Q0 + 1;
  constexpr PrimeRoots<R> rt{};
  float2 A[NQ], B[NQ];
#pragma unroll
  for (int u = 0; u < NQ; ++u) A[u] = B[u] = make_float2(0.f, 0.f);
  const float2 x0 = sm[spad(p0)];
#pragma unroll
  for (int i = 1; i <= h; ++i) {
    const float2 S = sm[spad(p0 + i * stride)], D = sm[spad(p0 + (R - i) * stride)];
#pragma unroll
    for (int u = 0; u < NQ; ++u) {
      const int q = Q0 + u;
      if (q == 0) {
        A[u] = cadd(A[u], S);
      } else {
        const int m = (i * q) % R;
        const float c = rt.c[m], sn = rt.s[m];
        A[u].x = fmaf(S.x, c, A[u].x);
        A[u].y = fmaf(S.y, c, A[u].y);
        B[u].x = fmaf(D.x, sn, B[u].x);
        B[u].y = fmaf(D.y, sn, B[u].y);
      }
    }
  }
#pragma unroll
  for (int u = 0; u < NQ; ++u) {
    const int q = Q0 + u;
    const float2 m0 = cadd(x0, A[u]);
    if (q == 0) {
      out[0] = m0;
    } else {
      const float2 iB = make_float2(-DIR * B[u].y, DIR * B[u].x);  // DIR * i * B
      const int o = Q0 == 0 ? 2 * q - 1 : 2 * (q - Q0);
      out[o] = cadd(m0, iB);
      out[o + 1] = csub(m0, iB);
    }
  }
}

// One stage of a prime radix R > 13 through the shared buffer, output-parallel (see
// the file comment).  Phase 1: the PB threads of a butterfly twiddle x_i and x_{R-i}
// over runs of i and store S_i = x_i + x_{R-i} at i and D_i = x_i - x_{R-i} at R - i.  Phase 2: PB
// threads per butterfly (consecutive lanes take consecutive butterflies) each form
// their share of the output pairs in registers.  Phase 3: the outputs go to their
// sorted positions.  NS is the product of the radices already applied.  Ends with
// a barrier.
template <int L, int DIR, int R, int NS>
__device__ __forceinline__ void mr_big_stage(float2* sm, int t) {
  constexpr int T = L / 16;
  constexpr int NBUT = L / R;
  static_assert(NBUT <= T, "one thread per butterfly at least");
  constexpr int h = (R - 1) / 2;
  constexpr int PB = T / NBUT >= 2 ? 2 : 1;  // threads per butterfly
  constexpr int QA = PB == 2 ? h / 2 : h;    // thread 0 of a butterfly: q = 0 .. QA; thread 1: QA + 1 .. h
  // phase 1: twiddle and fold, the PB threads of a butterfly on consecutive runs of i;
  // the twiddles w^i and w^(R-i) of a run start from sincospif and step by w and
  // conj(w) (at most IRUN - 1 products)
  constexpr int IRUN = (h + PB - 1) / PB;
  if (t < PB * NBUT) {
    const int jp = t % NBUT, i0 = 1 + (t / NBUT) * IRUN;
    const int k = jp % NS;
    float2 w = make_float2(1.f, 0.f), wa = w, wb = w;
    if constexpr (NS > 1) {
      constexpr float inv = 1.0f / (float)(NS * R);
      float s1, c1, sa, ca, sb, cb;
      sincospif(2.0f * (float)k * inv, &s1, &c1);
      sincospif(2.0f * (float)((i0 * k) % (NS * R)) * inv, &sa, &ca);
      sincospif(2.0f * (float)(((R - i0) * k) % (NS * R)) * inv, &sb, &cb);
      w = make_float2(c1, DIR * s1);
      wa = make_float2(ca, DIR * sa);
      wb = make_float2(cb, DIR * sb);
    }
#pragma unroll
    for (int r = 0; r < IRUN; ++r) {
      const int i = i0 + r;
      if (i <= h) {
        float2 a = sm[spad(jp + i * NBUT)], b = sm[spad(jp + (R - i) * NBUT)];
        if constexpr (NS > 1) {
          a = cmul(a, wa);
          b = cmul(b, wb);
          wa = cmul(wa, w);
          wb = cmul(wb, make_float2(w.x, -w.y));
        }
        sm[spad(jp + i * NBUT)] = cadd(a, b);
        sm[spad(jp + (R - i) * NBUT)] = csub(a, b);
      }
    }
  }
  __syncthreads();
  // phase 2: output pairs in registers
  constexpr int NOUT0 = 1 + 2 * QA, NOUT1 = 2 * (h - QA);
  constexpr int NOUT = NOUT0 > NOUT1 ? NOUT0 : NOUT1;
  float2 out[NOUT];
  const int jp = t % NBUT, part = t / NBUT;
  const bool act = t < PB * NBUT;
  if (act) {
    if (part == 0) big_prime_pairs<R, DIR, 0, QA>(sm, jp, NBUT, out);
    else if constexpr (PB == 2) big_prime_pairs<R, DIR, QA + 1, h>(sm, jp, NBUT, out);
  }
  __syncthreads();
  // phase 3: sorted positions
  if (act) {
    const int k = jp % NS;
    const int base = (jp - k) * R + k;
    if (part == 0) {
      sm[spad(base)] = out[0];
#pragma unroll
      for (int q = 1; q <= QA; ++q) {
        sm[spad(base + q * NS)] = out[2 * q - 1];
        sm[spad(base + (R - q) * NS)] = out[2 * q];
      }
    } else if constexpr (PB == 2) {
#pragma unroll
      for (int q = QA + 1; q <= h; ++q) {
        sm[spad(base + q * NS)] = out[2 * (q - QA - 1)];
        sm[spad(base + (R - q) * NS)] = out[2 * (q - QA - 1) + 1];
      }
    }
  }
  __syncthreads();
}

// the odd part O of T, one prime stage at a time (NS: radices applied so far)
template <int L, int DIR, int O, int NS>
__device__ __forceinline__ void mr_odd_stages(float2* sm, int t) {
  if constexpr (O > 1) {
    constexpr int R = odd_prime_factor(O);
    if constexpr (R <= 13) mr_odd_stage<L, DIR, R, NS>(sm, t);
    else mr_big_stage<L, DIR, R, NS>(sm, t);
    mr_odd_stages<L, DIR, O / R, NS * R>(sm, t);
  }
}

// the power-of-two part P after the odd stages, uniform register stages; the data
// is in the shared buffer in natural stage order on entry, read back by the caller
template <int L, int DIR, int P, int NS, int OUT>
__device__ __forceinline__ void mr_pow2_stages(float2 (&v)[16], float2* sm, int t) {
  constexpr int R = P >= 16 ? 16 : P;
  constexpr bool LAST = P / R == 1;
  reg_stage<L, DIR, R, NS, LAST, LAST ? OUT : kOutSmem>(v, sm, t);
  if constexpr (!LAST) mr_pow2_stages<L, DIR, P / R, NS * R, OUT>(v, sm, t);
}

// Transform one signal of mixed length L (mr_length(L)); same contract as reg_fft
// for OUT = kOutSmem and kOutRegs.
template <int L, int DIR, int OUT = kOutSmem>
__device__ __forceinline__ void mr_fft(float2 (&v)[16], float2* sm, int t) {
  static_assert(mr_length(L), "mixed-radix length");
  static_assert(OUT == kOutSmem || OUT == kOutRegs, "output form");
  constexpr int T = L / 16;
  constexpr int P = pow2_part(T);
  constexpr int O = T / P;
  // stage 1: radix 16 from the registers (Stockham with NS = 1: outputs at 16 t + i)
  {
    float2 x[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) x[i] = v[i];
    bfly16<DIR>(x);
#pragma unroll
    for (int i = 0; i < 16; ++i) sm[spad(t * 16 + i)] = x[i];
    __syncthreads();
  }
  mr_odd_stages<L, DIR, O, 16>(sm, t);
  if constexpr (P > 1) {
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = sm[spad(t + i * T)];
    __syncthreads();
    mr_pow2_stages<L, DIR, P, 16 * O, OUT>(v, sm, t);
  } else if constexpr (OUT == kOutRegs) {
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = sm[spad(t + i * T)];
    __syncthreads();  // the caller may reuse the buffer at once
  }
}

// two signals on the same threads (reg_fft2's contract), one after the other
template <int L, int DIR, int OUT = kOutSmem>
__device__ __forceinline__ void mr_fft2(float2 (&v0)[16], float2 (&v1)[16], float2* sm0, float2* sm1, int t) {
  mr_fft<L, DIR, OUT>(v0, sm0, t);
  mr_fft<L, DIR, OUT>(v1, sm1, t);
}

// any supported length: power of two (fft_reg.cuh) or mixed
template <int L, int DIR, int OUT = kOutSmem>
__device__ __forceinline__ void any_fft(float2 (&v)[16], float2* sm, int t) {
  if constexpr ((L & (L - 1)) == 0) reg_fft<L, DIR, OUT>(v, sm, t);
  else mr_fft<L, DIR, OUT>(v, sm, t);
}
template <int L, int DIR, int OUT = kOutSmem>
__device__ __forceinline__ void any_fft2(float2 (&v0)[16], float2 (&v1)[16], float2* sm0, float2* sm1, int t) {
  if constexpr ((L & (L - 1)) == 0) reg_fft2<L, DIR, OUT>(v0, v1, sm0, sm1, t);
  else mr_fft2<L, DIR, OUT>(v0, v1, sm0, sm1, t);
}

}  // namespace lpgb
