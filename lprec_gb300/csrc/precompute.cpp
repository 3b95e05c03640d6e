// Host precompute of the log-polar geometry, coordinate tables, convolution
// kernels and FBP filter, written into lprec's packed parameter arrays.
//
// Restates src/lprec/initsgl.py:25-99 (create_gl), src/lprec/initsfwd.py:15-126
// (create_fwd, fzeta_loop_weights, savePfwdpars) and src/lprec/initsadj.py:19-244
// (create_adj, fzeta_loop_weights_adj, take_filter, wint, savePadjpars).
//
// Two precisions:
//  * LP_PRECISION_REFERENCE repeats the reference's float32 steps (float32
//    log-polar grids, float32 exp/cos/log on them, float32 comparisons where the
//    reference compares a float32 array with a Python scalar, complex64 kernel
//    rows), so index sets and values match the reference precompute.
//  * LP_PRECISION_FP64 keeps exactly the same index sets and evaluates every
//    value in float64, rounding once when packing.
// Compile with -ffp-contract=off: the float steps must not fuse into FMAs.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <complex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/lprec_gb300.h"
#include "host_fft.h"

typedef std::complex<double> cd;
using lpgb_host::HostFFT;

int lp_internal_set_err(int code, const char* msg);  // lp_handle.cu

namespace {

const double PI = 3.14159265358979311600;  // numpy.pi (nearest double to pi)

inline double f32(double x) { return (double)(float)x; }
inline float expf_ref(float x) { return (float)exp((double)x); }
inline float cosf_ref(float x) { return (float)cos((double)x); }
inline float sinf_ref(float x) { return (float)sin((double)x); }
inline float logf_ref(float x) { return (float)log((double)x); }

template <typename F>
void parallel_for(int n, int nthreads, F fn) {
  if (nthreads <= 1 || n < 2) {
    for (int i = 0; i < n; ++i) fn(i);
    return;
  }
  std::vector<std::thread> th;
  const int nt = std::min(nthreads, n);
  for (int t = 0; t < nt; ++t)
    th.emplace_back([=, &fn]() {
      for (int i = t; i < n; i += nt) fn(i);
    });
  for (auto& x : th) x.join();
}

// ---------------------------------------------------------------------------
// geometry (initsgl.py:25-70)
// ---------------------------------------------------------------------------
struct Geo {
  int N0, N, os, Nproj0, Nproj, Nslices, Nth, Nrho, cubic;
  double cor;
  double beta, aR, am, g, dtheta, drho;
  std::vector<double> proj, s;
  std::vector<float> thsp, rhosp;
  bool ok = true;
  std::string err;
};

double osg(double aR, double theta) {  // initsgl.py:73-77
  const int n = 1000;
  const double a = -PI / 2, b = PI / 2;
  const double step = (b - a) / (n - 1);
  double best = -INFINITY;
  for (int i = 0; i < n; ++i) {
    const double t = (i == n - 1) ? b : i * step + a;
    const double wr = aR * cos(t) + (1 - aR);
    const double wi = aR * sin(t);
    const double v = log(hypot(wr, wi)) + log(cos(theta - atan2(wi, wr)));
    if (v > best) best = v;
  }
  return best;
}

std::vector<double> linspace(double a, double b, int n) {
  std::vector<double> y(n);
  const double step = (b - a) / (n - 1);
  for (int i = 0; i < n; ++i) y[i] = i * step + a;
  if (n > 1) y[n - 1] = b;
  return y;
}

int round_half_even(double x) {
  double r = nearbyint(x);  // default rounding mode: ties to even, as Python's round
  return (int)r;
}

Geo make_geo(int N0, int Nproj, int Nslices, double cor, int cubic) {
  Geo G;
  G.N0 = N0;
  G.Nproj0 = Nproj;
  G.Nslices = Nslices;
  G.cor = cor;
  G.cubic = cubic;
  G.beta = PI / 3;
  G.N = (int)(ceil((N0 + fabs(N0 / 2.0 - cor) * 2.0) / 16.0) * 16);
  G.os = std::max(round_half_even(3.0 * G.N / 2.0 / Nproj), 1);
  G.Nproj = G.os * Nproj;
  const double b = G.beta;
  G.proj.resize(G.Nproj);
  for (int i = 0; i < G.Nproj; ++i) G.proj[i] = (double)i * PI / G.Nproj - b / 2;
  G.s = linspace(-1, 1, G.N);
  G.aR = sin(b / 2) / (1 + sin(b / 2));
  G.am = (cos(b / 2) - sin(b / 2)) / (1 + sin(b / 2));
  G.g = osg(G.aR, b / 2);
  G.Nth = G.N;
  G.Nrho = 2 * G.N;
  G.dtheta = (2 * b) / G.Nth;
  G.drho = (G.g - log(G.am)) / G.Nrho;
  G.thsp.resize(G.Nth);
  const double dth32 = f32(G.dtheta);
  for (int i = 0; i < G.Nth; ++i) G.thsp[i] = (float)((double)(i - G.Nth / 2) * dth32);
  G.rhosp.resize(G.Nrho);
  for (int i = 0; i < G.Nrho; ++i) G.rhosp[i] = (float)((double)(i - G.Nrho) * G.drho);
  return G;
}

// cubic B-spline samples (initsgl.py:80-99) and their DFT; ref: float32 steps
std::vector<cd> b3_dft(const std::vector<float>& grid, bool ref) {
  const int n = (int)grid.size();
  std::vector<double> x2(n);
  if (ref) {
    const float mid = (grid[n - 1] + grid[0]) / 2.0f;
    for (int i = 0; i < n; ++i) x2[i] = (double)(float)(grid[i] - mid);
  } else {
    const double mid = ((double)grid[n - 1] + (double)grid[0]) / 2.0;
    for (int i = 0; i < n; ++i) x2[i] = (double)grid[i] - mid;
  }
  const int c = (int)ceil((n + 1) / 2.0) - 1;
  std::vector<double> B(n, 0.0);
  if (ref) {
    const float step = (float)x2[1] - (float)x2[0];
    const float r = 1.0f * step;
    for (int ix = -2; ix <= 2; ++ix) {
      const float d = fabsf((float)x2[c + ix] - (float)x2[c]) / r;
      float v = 0.f;
      const float d2 = d * d, d3 = (float)pow((double)d, 3.0);
      if (d < 1) v = (3 * d3 - 6 * d2 + 4) / 6;
      else if (d < 2) v = (-d3 + 6 * d2 - 12 * d + 8) / 6;
      B[c + ix] = v;
    }
  } else {
    const double step = x2[1] - x2[0];
    for (int ix = -2; ix <= 2; ++ix) {
      const double d = fabs(x2[c + ix] - x2[c]) / step;
      double v = 0.0;
      if (d < 1) v = (3 * d * d * d - 6 * d * d + 4) / 6;
      else if (d < 2) v = (-d * d * d + 6 * d * d - 12 * d + 8) / 6;
      B[c + ix] = v;
    }
  }
  // ifftshift then DFT: sample at index m moves to (m - n/2) mod n
  std::vector<cd> out(n);
  for (int k = 0; k < n; ++k) {
    cd acc = 0;
    for (int ix = -2; ix <= 2; ++ix) {
      const int m = c + ix;
      const int pos = ((m - n / 2) % n + n) % n;
      const double ang = -2.0 * PI * (double)(((int64_t)pos * k) % n) / n;
      acc += B[m] * cd(cos(ang), sin(ang));
    }
    if (ref) acc = cd((double)(float)acc.real(), (double)(float)acc.imag());
    out[k] = acc;
  }
  return out;
}

// numpy's complex128 division (Smith's algorithm, as in numpy's loops)
inline cd cdiv(cd a, cd b) {
  const double br = b.real(), bi = b.imag(), ar = a.real(), ai = a.imag();
  if (fabs(br) >= fabs(bi)) {
    if (br == 0 && bi == 0) return cd(ar / fabs(br), ai / fabs(bi));
    const double rat = bi / br;
    const double scl = 1.0 / (br + bi * rat);
    return cd((ar + ai * rat) * scl, (ai - ar * rat) * scl);
  }
  const double rat = br / bi;
  const double scl = 1.0 / (bi + br * rat);
  return cd((ar * rat + ai) * scl, (ai * rat - ar) * scl);
}

// ---------------------------------------------------------------------------
// convolution kernel (initsfwd.py:69-93, initsadj.py:119-143), returned as the
// packed half spectrum fZ[Nrho][Nth/2+1] after fftshift, const and B3com.
// ---------------------------------------------------------------------------
std::vector<cd> kernel_half(const Geo& G, bool adjoint, bool ref, int nthreads) {
  const int Nth = G.Nth, Nrho = G.Nrho, NL = 4 * Nth;
  const double betas = 2 * G.beta;
  const double rhos = G.g - log(G.am);
  std::vector<double> lc(NL), h(NL, 1.0);
  double dthL;
  if (ref) {
    std::vector<float> thL(NL);
    for (int i = 0; i < NL; ++i) thL[i] = ((float)(i - NL / 2) / (float)NL) * (float)betas;
    for (int i = 0; i < NL; ++i) lc[i] = log((double)cosf_ref(thL[i]));
    dthL = (double)(thL[1] - thL[0]);
  } else {
    for (int i = 0; i < NL; ++i) lc[i] = log(cos((double)(i - NL / 2) / NL * betas));
    dthL = ((double)(1 - NL / 2) / NL * betas) - ((double)(-NL / 2) / NL * betas);
  }
  static const double num[11] = {-216254335, 679543284, -1412947389, 2415881496, -3103579086, 2939942400,
                                 -2023224114, 984515304, -321455811, 63253516, -5675265};
  double corr[11];
  for (int j = 0; j < 11; ++j) corr[j] = 1 + num[j] / 958003200.0;
  corr[0] = 2 * (corr[0] - 0.5);
  h[0] *= corr[0];
  for (int j = 1; j < 11; ++j) {
    h[j] *= corr[j];
    h[NL - j] *= corr[j];
  }
  if (ref)
    for (int i = 0; i < NL; ++i) h[i] = f32(h[i]);
  // centred rows krho = -Nrho/2 .. Nrho/2-1, columns kt = -Nth/2 .. Nth/2-1
  std::vector<cd> cen((size_t)Nrho * Nth);
  const float twopi32 = (float)(2.0 * PI);
  HostFFT fft(NL);
  // exp(er * log cos) does not depend on the rho row: once per sample
  const double er = adjoint ? 0.0 : -1.0;
  std::vector<double> mag(NL);
  for (int i = 0; i < NL; ++i) mag[i] = exp(er * lc[i]);
  parallel_for(Nrho, nthreads, [&](int j) {
    const double kj = (double)(j - Nrho / 2);
    double ei;
    if (ref) {
      const double im32 = (double)(twopi32 * (float)kj);
      // NumPy divides the complex64 product by the float64 scalar with
      // Smith's method, i.e. multiplies by the reciprocal
      ei = (adjoint ? im32 : -im32) * (1.0 / rhos);
    } else {
      ei = (adjoint ? 2 * PI * kj : -2 * PI * kj) / rhos;
    }
    std::vector<cd> a(NL), b(NL);
    for (int i = 0; i < NL; ++i) {
      const double L = lc[i];
      const double ph = ei * L;
      const cd v = cd(mag[i] * cos(ph), mag[i] * sin(ph)) * h[i];
      a[(i + NL / 2) % NL] = v;  // fftshift before the FFT
    }
    fft.run(a.data(), b.data());
    for (int q = 0; q < Nth; ++q) {
      cd v = a[(size_t)((q - Nth / 2 + NL) % NL)];
      if (ref) {
        const float re = (float)v.real(), im = (float)v.imag();
        const float d = (float)dthL;
        v = cd((double)(re * d), (double)(im * d));
      } else {
        v *= dthL;
      }
      cen[(size_t)j * Nth + q] = v;
    }
  });
  for (int q = 0; q < Nth; ++q) cen[q] = 0;                    // fZ[0] = 0
  for (int j = 0; j < Nrho; ++j) cen[(size_t)j * Nth] = 0;     // fZ[:, 0] = 0
  double cst;
  if (adjoint)
    cst = (double)((G.N + 1) * (G.N - 1)) / ((double)G.N * G.N) / 2 * sqrt((double)G.os * G.Nproj / G.N / 2);
  else
    cst = sqrt((double)G.N * G.os / G.Nproj) * PI / 4 / G.aR / sqrt(2.0);
  std::vector<cd> b3th, b3rho;
  if (G.cubic) {
    b3th = b3_dft(G.thsp, ref);
    b3rho = b3_dft(G.rhosp, ref);
  }
  const int nh = Nth / 2 + 1;
  std::vector<cd> out((size_t)Nrho * nh);
  for (int r = 0; r < Nrho; ++r)
    for (int c = 0; c < nh; ++c) {
      cd v = cen[(size_t)((r + Nrho / 2) % Nrho) * Nth + (c + Nth / 2) % Nth];  // fftshift
      v = cd(v.real() * cst, v.imag() * cst);
      if (G.cubic) {
        cd b;
        if (ref) {
          const float ar = (float)b3rho[r].real(), ai = (float)b3rho[r].imag();
          const float br = (float)b3th[c].real(), bi = (float)b3th[c].imag();
          b = cd((double)(ar * br - ai * bi), (double)(ar * bi + ai * br));
        } else {
          b = b3rho[r] * b3th[c];
        }
        v = cdiv(v, b);
      }
      out[(size_t)r * nh + c] = v;
    }
  return out;
}

// ---------------------------------------------------------------------------
// FBP filter (initsadj.py:146-203)
// ---------------------------------------------------------------------------
bool invert(std::vector<double>& A, int n) {  // Gauss-Jordan with partial pivoting
  std::vector<double> I((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) I[(size_t)i * n + i] = 1.0;
  for (int c = 0; c < n; ++c) {
    int p = c;
    for (int r = c + 1; r < n; ++r)
      if (fabs(A[(size_t)r * n + c]) > fabs(A[(size_t)p * n + c])) p = r;
    if (A[(size_t)p * n + c] == 0) return false;
    if (p != c)
      for (int j = 0; j < n; ++j) {
        std::swap(A[(size_t)p * n + j], A[(size_t)c * n + j]);
        std::swap(I[(size_t)p * n + j], I[(size_t)c * n + j]);
      }
    const double d = A[(size_t)c * n + c];
    for (int j = 0; j < n; ++j) {
      A[(size_t)c * n + j] /= d;
      I[(size_t)c * n + j] /= d;
    }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = A[(size_t)r * n + c];
      if (f == 0) continue;
      for (int j = 0; j < n; ++j) {
        A[(size_t)r * n + j] -= f * A[(size_t)c * n + j];
        I[(size_t)r * n + j] -= f * I[(size_t)c * n + j];
      }
    }
  }
  A = I;
  return true;
}

std::vector<double> wint(int n, const std::vector<double>& t) {
  const int N = (int)t.size();
  std::vector<double> s = linspace(1e-40, 1, n);
  std::vector<double> V((size_t)n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) V[(size_t)i * n + j] = exp(i * log(s[j]));
  invert(V, n);
  // u[i][j] = X[i][j+1]-X[i][j], X[i][j] = exp((i+1) log s_j) / (i+1), i=0..n
  std::vector<double> X((size_t)(n + 1) * n), u((size_t)(n + 1) * (n - 1));
  for (int i = 0; i <= n; ++i)
    for (int j = 0; j < n; ++j) X[(size_t)i * n + j] = exp((i + 1) * log(s[j])) * (1.0 / (i + 1));
  for (int i = 0; i <= n; ++i)
    for (int j = 0; j < n - 1; ++j) u[(size_t)i * (n - 1) + j] = X[(size_t)i * n + j + 1] - X[(size_t)i * n + j];
  std::vector<double> W1((size_t)n * (n - 1), 0.0), W2((size_t)n * (n - 1), 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n - 1; ++j) {
      double a = 0, b = 0;
      for (int m = 0; m < n; ++m) {
        a += V[(size_t)i * n + m] * u[(size_t)(m + 1) * (n - 1) + j];
        b += V[(size_t)i * n + m] * u[(size_t)m * (n - 1) + j];
      }
      W1[(size_t)i * (n - 1) + j] = a;
      W2[(size_t)i * (n - 1) + j] = b;
    }
  std::vector<double> p;
  for (int i = 1; i < n; ++i) p.push_back(1.0 / i);
  for (int i = 0; i < N - 2 * (n - 1) - 1; ++i) p.push_back(1.0 / (n - 1));
  for (int i = n - 1; i > 0; --i) p.push_back(1.0 / i);
  std::vector<double> w(N, 0.0);
  for (int j = 0; j < N - n + 1; ++j) {
    const double dt = t[j + n - 1] - t[j];
    for (int k = 0; k < n - 1; ++k)
      for (int i = 0; i < n; ++i) {
        const double Wik = (dt * dt) * W1[(size_t)i * (n - 1) + k] + dt * t[j] * W2[(size_t)i * (n - 1) + k];
        w[j + i] = w[j + i] + p[j + k] * Wik;
      }
  }
  const double w40 = w[N - 40];
  for (int i = 0; i < 40; ++i) w[N - 40 + i] = w40 / (N - 40) * (double)(N - 40 + i);
  return w;
}

bool take_filter(int N, const std::string& name, std::vector<double>& out) {
  const int Ne = 4 * N;
  const double d = 0.5;
  const int nt = Ne / 2 + 1;
  std::vector<double> t(nt);
  for (int i = 0; i < nt; ++i) t[i] = (double)i / Ne;
  std::vector<double> w = wint(12, t);
  std::vector<double> wfa(nt);
  for (int i = 0; i < nt; ++i) {
    const double base = Ne * 0.5 * w[i];
    const double x = t[i];
    double v;
    if (name == "ramp") v = base;
    else if (name == "shepp-logan") {
      const double y = x / (2 * d);
      const double sc = (y == 0) ? 1.0 : sin(PI * y) / (PI * y);
      v = base * sc * ((x / d <= 2) ? 1.0 : 0.0);
    } else if (name == "cosine") v = base * cos(PI * x / (2 * d)) * ((x / d <= 1) ? 1.0 : 0.0);
    else if (name == "cosine2") {
      const double c = cos(PI * x / (2 * d));
      v = base * (c * c) * ((x / d <= 1) ? 1.0 : 0.0);
    } else if (name == "hamming") v = base * (.54 + .46 * cos(PI * x / d)) * ((x / d <= 1) ? 1.0 : 0.0);
    else if (name == "hann") v = base * (1 + cos(PI * x / d)) / 2.0 * ((x / d <= 1) ? 1.0 : 0.0);
    else if (name == "parzen") {
      const double q = 1 - x / d;
      v = base * pow(q, 3.0) * ((x / d <= 1) ? 1.0 : 0.0);
    } else return false;
    wfa[i] = v * ((v >= 0) ? 1.0 : 0.0);
  }
  out.assign(4 * (size_t)N, 0.0);
  // [flipud(wfa[1:]), 2*wfa[0], wfa[1:]][:-1]
  size_t o = 0;
  for (int i = nt - 1; i >= 1; --i) out[o++] = wfa[i];
  out[o++] = 2 * wfa[0];
  for (int i = 1; i < nt - 1; ++i) out[o++] = wfa[i];
  return true;
}

struct Sizes {
  int64_t gl, fi, ff, ai, af;
};

struct Tables {
  Geo G;
  // fwd
  std::vector<int32_t> pids[3], fcids;
  std::vector<double> lp2C1[3], lp2C2[3], p2lp1[3], p2lp2[3];
  // adj
  std::vector<int32_t> acids, lpids, wids;
  std::vector<double> C2lp1[3], C2lp2[3], lp2p1[3], lp2p2[3], lp2p1w[3], lp2p2w[3];
};

// Rows r of a (row, column) grid processed in parallel, each appending to its own
// buffers; the buffers are then concatenated in row order, so the result is the
// serial loop's, element for element.
template <typename T>
void concat_rows(std::vector<std::vector<T>>& rows, std::vector<T>& out) {
  size_t n = out.size();
  for (const auto& v : rows) n += v.size();
  out.reserve(n);
  for (auto& v : rows) {
    out.insert(out.end(), v.begin(), v.end());
    std::vector<T>().swap(v);
  }
}

// index sets and coordinates (no kernels); `ref` selects the value precision
bool build_fwd_coords(Tables& T, bool ref, std::string& err, int nthreads) {
  const Geo& G = T.G;
  const int Nth = G.Nth, Nrho = G.Nrho, N = G.N;
  const double b = G.beta, aR = G.aR;
  std::vector<float> e32(Nrho), c32(Nth), s32(Nth);
  for (int r = 0; r < Nrho; ++r) e32[r] = expf_ref(G.rhosp[r]);
  for (int t = 0; t < Nth; ++t) {
    c32[t] = cosf_ref(G.thsp[t]);
    s32[t] = sinf_ref(G.thsp[t]);
  }
  // float64 grid values for the fp64 coordinates (the same expressions, hoisted)
  std::vector<double> e64(Nrho), c64(Nth), s64(Nth);
  for (int r = 0; r < Nrho; ++r) e64[r] = exp((double)G.rhosp[r]);
  for (int t = 0; t < Nth; ++t) {
    c64[t] = cos((double)G.thsp[t]);
    s64[t] = sin((double)G.thsp[t]);
  }
  std::vector<int32_t> cids_k[3];
  for (int k = 0; k < 3; ++k) {
    const double c = cos(k * b + b / 2), sn = sin(k * b + b / 2);
    std::vector<std::vector<int32_t>> rid(Nrho);
    std::vector<std::vector<double>> rx(Nrho), ry(Nrho);
    parallel_for(Nrho, nthreads, [&](int r) {
      for (int t = 0; t < Nth; ++t) {
        // mask from the float32 products, as the reference
        const double t1 = (double)(e32[r] * c32[t]), t2 = (double)(e32[r] * s32[t]);
        const double X = ((t1 - (1 - aR)) * c - t2 * sn) / aR;
        double Y = ((t1 - (1 - aR)) * sn + t2 * c) / aR;
        Y *= -1;
        if (X * X + Y * Y <= 1) {
          rid[r].push_back((int32_t)((size_t)r * Nth + t));
          double x = X, y = Y;
          if (!ref) {
            const double ee = e64[r];
            const double u1 = ee * c64[t], u2 = ee * s64[t];
            x = ((u1 - (1 - aR)) * c - u2 * sn) / aR;
            y = ((u1 - (1 - aR)) * sn + u2 * c) / aR;
            y *= -1;
          }
          rx[r].push_back((x + 1) / 2 * (N - 1));
          ry[r].push_back((y + 1) / 2 * (N - 1));
        }
      }
    });
    concat_rows(rid, cids_k[k]);
    concat_rows(rx, T.lp2C1[k]);
    concat_rows(ry, T.lp2C2[k]);
  }
  if (cids_k[0] != cids_k[1] || cids_k[0] != cids_k[2]) {
    err = "disk index sets differ between spans";
    return false;
  }
  T.fcids = cids_k[2];
  const double thden = (double)(G.thsp[Nth - 1] - G.thsp[0]);
  const double rhoden = (double)(G.rhosp[Nrho - 1] - G.rhosp[0]);
  for (int k = 0; k < 3; ++k) {
    for (int p = 0; p < G.Nproj; ++p) {
      const double th = G.proj[p];
      if (!(th >= k * b - b / 2 && th < k * b + b / 2)) continue;
      const double th00 = th - k * b;
      const double cth = cos(th00);
      const double tc = (th00 - (double)G.thsp[0]) / thden * (Nth - 1);
      for (int x = 0; x < N; ++x) {
        T.pids[k].push_back((int32_t)(p * N + x));
        T.p2lp1[k].push_back(tc);
        const double rr = log(G.s[x] * aR + (1 - aR) * cth);
        T.p2lp2[k].push_back((rr - (double)G.rhosp[0]) / rhoden * (Nrho - 1));
      }
    }
  }
  return true;
}

bool build_adj_coords(Tables& T, bool ref, std::string& err, int nthreads) {
  const Geo& G = T.G;
  const int Nth = G.Nth, Nrho = G.Nrho, N = G.N;
  const double b = G.beta, aR = G.aR, am = G.am, g = G.g;
  std::vector<double> lin = linspace(-1, 1, N);
  for (int i = 0; i < N * N; ++i) {
    const double x1 = lin[i % N], x2 = -lin[i / N];
    if (x1 * x1 + x2 * x2 <= 1) T.acids.push_back(i);
  }
  const double thden = (double)(G.thsp[Nth - 1] - G.thsp[0]);
  const double rhoden = (double)(G.rhosp[Nrho - 1] - G.rhosp[0]);
  const int na = (int)T.acids.size();
  const int nblk = (na + 4095) / 4096;
  for (int k = 0; k < 3; ++k) {
    const double c = cos(k * b + b / 2), sn = sin(k * b + b / 2);
    T.C2lp1[k].resize(na);
    T.C2lp2[k].resize(na);
    parallel_for(nblk, nthreads, [&](int blk) {
      for (int j = blk * 4096; j < std::min(na, (blk + 1) * 4096); ++j) {
        const int32_t i = T.acids[j];
        const double x1 = lin[i % N], x2 = -lin[i / N];
        const double z1 = aR * (x1 * c + x2 * sn) + (1 - aR);
        const double z2 = aR * (-x1 * sn + x2 * c);
        T.C2lp1[k][j] = (atan2(z2, z1) - (double)G.thsp[0]) / thden * (Nth - 1);
        T.C2lp2[k][j] = (log(sqrt(z1 * z1 + z2 * z2)) - (double)G.rhosp[0]) / rhoden * (Nrho - 1);
      }
    });
  }
  // log-polar grid in float32 as the reference, for the index sets
  const float lo32 = (float)(-b / 2), hi32 = (float)(b / 2);
  const double drho32 = (double)(G.rhosp[1] - G.rhosp[0]);
  std::vector<double> z2n_v;
  std::vector<int32_t> wr, wl;          // wrap candidates (right: log z2 > g; left)
  std::vector<double> wrv, wlv;
  {
    // per theta column: cos in float32 (masks) and in the value precision (hoisted)
    std::vector<double> cm(Nth), cv(Nth);
    for (int t = 0; t < Nth; ++t) {
      cm[t] = (double)cosf_ref(G.thsp[t]);
      cv[t] = ref ? cm[t] : cos((double)G.thsp[t]);
    }
    std::vector<std::vector<int32_t>> r_lp(Nrho), r_wr(Nrho), r_wl(Nrho);
    std::vector<std::vector<double>> r_z2n(Nrho), r_wrv(Nrho), r_wlv(Nrho);
    parallel_for(Nrho, nthreads, [&](int r) {
      const float z2f = expf_ref(G.rhosp[r]);
      const double z2 = ref ? (double)z2f : exp((double)G.rhosp[r]);
      const float lz2f = logf_ref(z2f);
      const double lz2 = ref ? (double)lz2f : log(z2);
      const bool right = (double)lz2f > g, left = (double)lz2f < log(am) - g + drho32;
      const double vrm = right ? exp((double)lz2f + log(am) - g) : 0, vr = right ? exp(lz2 + log(am) - g) : 0;
      const double vlm = left ? exp((double)lz2f - log(am) + g) : 0, vl = left ? exp(lz2 - log(am) + g) : 0;
      for (int t = 0; t < Nth; ++t) {
        const float z1f = G.thsp[t];
        const double cz1 = cv[t];
        // masks always from the float32 (reference) values
        const double z2n_m = ((double)z2f - (1 - aR) * cm[t]) / aR;
        const double z2n = (z2 - (1 - aR) * cz1) / aR;
        const int idx = r * Nth + t;
        const bool inspan = (z1f >= lo32) && (z1f < hi32);
        if (inspan && fabs(z2n_m) <= 1) {
          r_lp[r].push_back(idx);
          r_z2n[r].push_back(z2n);
        }
        if (right) {
          r_wr[r].push_back(idx);
          const double vm = (vrm - (1 - aR) * cm[t]) / aR;
          const double v = (vr - (1 - aR) * cz1) / aR;
          r_wrv[r].push_back(inspan && fabs(vm) <= 1 ? v : NAN);
        }
        if (left) {
          r_wl[r].push_back(idx);
          const double vm = (vlm - (1 - aR) * cm[t]) / aR;
          const double v = (vl - (1 - aR) * cz1) / aR;
          r_wlv[r].push_back(inspan && fabs(vm) <= 1 ? v : NAN);
        }
      }
    });
    concat_rows(r_lp, T.lpids);
    concat_rows(r_z2n, z2n_v);
    concat_rows(r_wr, wr);
    concat_rows(r_wrv, wrv);
    concat_rows(r_wl, wl);
    concat_rows(r_wlv, wlv);
  }
  // selected positions inside the wrap candidate lists
  std::vector<int64_t> lw, lw2;
  for (size_t i = 0; i < wr.size(); ++i)
    if (!std::isnan(wrv[i])) lw.push_back((int64_t)i);
  for (size_t i = 0; i < wl.size(); ++i)
    if (!std::isnan(wlv[i])) lw2.push_back((int64_t)i);
  // span angles (pids over the projection angles)
  int first[3], last[3], cnt[3];
  for (int k = 0; k < 3; ++k) {
    first[k] = -1;
    last[k] = -1;
    cnt[k] = 0;
    for (int p = 0; p < G.Nproj; ++p) {
      const double th = G.proj[p];
      if (th >= k * b - b / 2 && th < k * b + b / 2) {
        if (first[k] < 0) first[k] = p;
        last[k] = p;
        cnt[k]++;
      }
    }
    if (cnt[k] < 2) {
      err = "fewer than two projection angles in a span";
      return false;
    }
  }
  double proj0[3], projl[3];
  for (int k = 0; k < 3; ++k) {
    proj0[k] = G.proj[first[k]];
    projl[k] = G.proj[last[k]] - G.proj[first[k]];
  }
  const double projp = (double)(G.Nproj - 1) / (proj0[2] + projl[2] - proj0[0]);
  auto angle = [&](int k, float z1f) {
    double a;
    if (ref) a = (double)(z1f + (float)(k * b));
    else a = (double)z1f + k * b;
    return (a - proj0[k]) / projl[k] * (cnt[k] - 1) + (proj0[k] - proj0[0]) * projp;
  };
  for (int k = 0; k < 3; ++k) {
    for (size_t i = 0; i < T.lpids.size(); ++i) {
      const int t = T.lpids[i] % Nth;
      T.lp2p1[k].push_back(angle(k, G.thsp[t]));
      T.lp2p2[k].push_back((z2n_v[i] + 1) / 2 * (N - 1));
    }
    // initsadj.py:69 takes z1 at the positions of the selected entries inside
    // the candidate lists (z1 flattened over the whole grid)
    for (int64_t q : lw) T.lp2p1w[k].push_back(angle(k, G.thsp[q % Nth]));
    for (int64_t q : lw2) T.lp2p1w[k].push_back(angle(k, G.thsp[q % Nth]));
    for (int64_t q : lw) T.lp2p2w[k].push_back((wrv[q] + 1) / 2 * (N - 1));
    for (int64_t q : lw2) T.lp2p2w[k].push_back((wlv[q] + 1) / 2 * (N - 1));
  }
  for (int64_t q : lw) T.wids.push_back(wr[q]);
  for (int64_t q : lw2) T.wids.push_back(wl[q]);
  return true;
}

Sizes sizes_of(const Tables& T, bool with_filter) {
  Sizes s;
  const Geo& G = T.G;
  const int64_t nh = G.Nth / 2 + 1;
  s.gl = 10 + (int64_t)G.Nrho * G.Nth;
  int64_t sp = 0;
  for (int k = 0; k < 3; ++k) sp += (int64_t)T.pids[k].size();
  const int64_t nc = (int64_t)T.fcids.size();
  s.fi = 3 + sp + 1 + nc;
  s.ff = 6 * nc + 2 * sp + 2 * G.Nrho * nh;
  const int64_t ac = (int64_t)T.acids.size(), nl = (int64_t)T.lpids.size(), nw = (int64_t)T.wids.size();
  s.ai = 3 + ac + nl + nw + 1;
  s.af = 6 * ac + 6 * nl + 6 * nw + 2 * G.Nrho * nh + (with_filter ? 4 * (int64_t)G.N : 0);
  return s;
}

int check_args(int N0, int Nproj, int Nslices, double cor, const char* filter, bool& with_filter) {
  if (N0 < 2 || Nproj < 2 || Nslices < 1) return lp_internal_set_err(LP_ERR_ARG, "precompute: bad sizes");
  if (!(cor >= 0) || cor > N0) return lp_internal_set_err(LP_ERR_ARG, "precompute: cor out of range");
  const std::string f = filter ? filter : "none";
  static const char* names[] = {"none", "ramp", "shepp-logan", "cosine", "cosine2", "hamming", "hann", "parzen"};
  bool known = false;
  for (const char* n : names)
    if (f == n) known = true;
  if (!known) return lp_internal_set_err(LP_ERR_ARG, "precompute: unknown filter");
  with_filter = f != "none";
  return LP_OK;
}

}  // namespace

extern "C" int lp_precompute_sizes(int N0, int Nproj, int Nslices, double cor, int cubic, const char* filter,
                                   int64_t sizes[5]) {
  bool wf;
  int rc = check_args(N0, Nproj, Nslices, cor, filter, wf);
  if (rc) return rc;
  if (!sizes) return lp_internal_set_err(LP_ERR_ARG, "precompute: null sizes");
  Tables T;
  T.G = make_geo(N0, Nproj, Nslices, cor, cubic);
  std::string err;
  const int nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  if (!build_fwd_coords(T, true, err, nthreads) || !build_adj_coords(T, true, err, nthreads))
    return lp_internal_set_err(LP_ERR_UNSUPPORTED, err.c_str());
  Sizes s = sizes_of(T, wf);
  sizes[0] = s.gl;
  sizes[1] = s.fi;
  sizes[2] = s.ff;
  sizes[3] = s.ai;
  sizes[4] = s.af;
  return LP_OK;
}

template <typename Real>
static int precompute_impl(int N0, int Nproj, int Nslices, double cor, int cubic, const char* filter,
                           int precision, int with_fwd, int nthreads, float* glpars, int32_t* fwdparsi,
                           Real* fwdparamsf, int32_t* adjparsi, Real* adjparamsf) {
  bool wf;
  int rc = check_args(N0, Nproj, Nslices, cor, filter, wf);
  if (rc) return rc;
  if (!glpars || !adjparsi || !adjparamsf || (with_fwd && (!fwdparsi || !fwdparamsf)))
    return lp_internal_set_err(LP_ERR_ARG, "precompute: null output array");
  if (precision != LP_PRECISION_REFERENCE && precision != LP_PRECISION_FP64)
    return lp_internal_set_err(LP_ERR_ARG, "precompute: bad precision");
  const bool ref = precision == LP_PRECISION_REFERENCE;
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  Tables T;
  T.G = make_geo(N0, Nproj, Nslices, cor, cubic);
  const Geo& G = T.G;
  std::string err;
  if ((with_fwd && !build_fwd_coords(T, ref, err, nthreads)) || !build_adj_coords(T, ref, err, nthreads))
    return lp_internal_set_err(LP_ERR_UNSUPPORTED, err.c_str());
  // glpars: [N, N0, Ntheta, Nrho, Nspan, Nproj, Nslices, cor, osangles, cubic] ++ erho
  const float head[10] = {(float)G.N, (float)G.N0, (float)G.Nth, (float)G.Nrho, 3.f, (float)G.Nproj,
                          (float)G.Nslices, (float)G.cor, (float)G.os, (float)(G.cubic ? 1 : 0)};
  memcpy(glpars, head, sizeof(head));
  for (int r = 0; r < G.Nrho; ++r) {
    const float e = ref ? expf_ref(G.rhosp[r]) : (float)exp((double)G.rhosp[r]);
    for (int t = 0; t < G.Nth; ++t) glpars[10 + (size_t)r * G.Nth + t] = e;
  }
  const int nh = G.Nth / 2 + 1;
  auto put_fz = [&](Real* dst, const std::vector<cd>& fz) {
    for (size_t i = 0; i < (size_t)G.Nrho * nh; ++i) {
      dst[2 * i] = (Real)fz[i].real();
      dst[2 * i + 1] = (Real)fz[i].imag();
    }
  };
  if (with_fwd) {
    int64_t o = 0;
    for (int k = 0; k < 3; ++k) fwdparsi[o++] = (int32_t)T.pids[k].size();
    for (int k = 0; k < 3; ++k)
      for (int32_t v : T.pids[k]) fwdparsi[o++] = v;
    fwdparsi[o++] = (int32_t)T.fcids.size();
    for (int32_t v : T.fcids) fwdparsi[o++] = v;
    o = 0;
    for (auto* arr : {T.lp2C1, T.lp2C2, T.p2lp1, T.p2lp2})
      for (int k = 0; k < 3; ++k)
        for (double v : arr[k]) fwdparamsf[o++] = (Real)v;
    put_fz(fwdparamsf + o, kernel_half(G, false, ref, nthreads));
  }
  {
    int64_t o = 0;
    adjparsi[o++] = (int32_t)T.acids.size();
    adjparsi[o++] = (int32_t)T.lpids.size();
    adjparsi[o++] = (int32_t)T.wids.size();
    for (int32_t v : T.acids) adjparsi[o++] = v;
    for (int32_t v : T.lpids) adjparsi[o++] = v;
    for (int32_t v : T.wids) adjparsi[o++] = v;
    adjparsi[o++] = wf ? 1 : 0;
    o = 0;
    for (auto* arr : {T.C2lp1, T.C2lp2, T.lp2p1, T.lp2p2, T.lp2p1w, T.lp2p2w})
      for (int k = 0; k < 3; ++k)
        for (double v : arr[k]) adjparamsf[o++] = (Real)v;
    put_fz(adjparamsf + o, kernel_half(G, true, ref, nthreads));
    o += 2 * (int64_t)G.Nrho * nh;
    if (wf) {
      std::vector<double> fl;
      take_filter(G.N, filter, fl);
      for (int i = 0; i < 4 * G.N; ++i) adjparamsf[o++] = (Real)fl[i];
    }
  }
  return LP_OK;
}

extern "C" int lp_precompute(int N0, int Nproj, int Nslices, double cor, int cubic, const char* filter,
                             int precision, int with_fwd, int nthreads, float* glpars, int32_t* fwdparsi,
                             float* fwdparamsf, int32_t* adjparsi, float* adjparamsf) {
  return precompute_impl(N0, Nproj, Nslices, cor, cubic, filter, precision, with_fwd, nthreads, glpars, fwdparsi,
                         fwdparamsf, adjparsi, adjparamsf);
}

extern "C" int lp_precompute_f64(int N0, int Nproj, int Nslices, double cor, int cubic, const char* filter,
                                 int precision, int with_fwd, int nthreads, float* glpars, int32_t* fwdparsi,
                                 double* fwdparamsf, int32_t* adjparsi, double* adjparamsf) {
  return precompute_impl(N0, Nproj, Nslices, cor, cubic, filter, precision, with_fwd, nthreads, glpars, fwdparsi,
                         fwdparamsf, adjparsi, adjparamsf);
}
