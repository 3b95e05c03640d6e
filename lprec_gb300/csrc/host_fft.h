// Complex FFT in float64 on the host (mixed radix Stockham, any length), used
// by the precompute (convolution kernels) and by the FBP filter setup.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <complex>
#include <vector>

namespace lpgb_host {

typedef std::complex<double> cd;
const double kPi = 3.14159265358979311600;

// forward sign exp(-2 pi i jk/L); run(a, b) leaves the result in a
struct HostFFT {
  int L;
  std::vector<int> radix;
  std::vector<cd> w;  // exp(-2 pi i t / L)
  explicit HostFFT(int L_) : L(L_) {
    int n = L;
    const int fast[] = {4, 2, 3, 5};
    for (int f : fast)
      while (n % f == 0) {
        radix.push_back(f);
        n /= f;
      }
    for (int f = 7; n > 1; f += 2)
      while (n % f == 0) {
        radix.push_back(f);
        n /= f;
      }
    w.resize(L);
    for (int t = 0; t < L; ++t) w[t] = cd(cos(2.0 * kPi * t / L), -sin(2.0 * kPi * t / L));
  }
  void run(cd* a, cd* b) const {  // result in a
    cd* in = a;
    cd* out = b;
    int Ns = 1;
    for (int R : radix) {
      const int Lr = L / R;
      cd v[64];
      std::vector<cd> big;
      cd* vv = v;
      if (R > 64) {
        big.resize(R);
        vv = big.data();
      }
      for (int j = 0; j < Lr; ++j) {
        const int k = j % Ns;
        for (int i = 0; i < R; ++i) {
          cd x = in[j + i * Lr];
          if (Ns > 1 && i > 0) x *= w[(size_t)((int64_t)i * k * (L / (Ns * R)) % L)];
          vv[i] = x;
        }
        const int base = (j - k) * R + k;
        if (R == 2) {
          out[base] = vv[0] + vv[1];
          out[base + Ns] = vv[0] - vv[1];
        } else if (R == 4) {
          cd a0 = vv[0] + vv[2], a1 = vv[0] - vv[2], b0 = vv[1] + vv[3], b1 = vv[1] - vv[3];
          b1 = cd(b1.imag(), -b1.real());
          out[base] = a0 + b0;
          out[base + Ns] = a1 + b1;
          out[base + 2 * Ns] = a0 - b0;
          out[base + 3 * Ns] = a1 - b1;
        } else {
          for (int q = 0; q < R; ++q) {
            cd acc = 0;
            for (int i = 0; i < R; ++i) acc += vv[i] * w[(size_t)((int64_t)i * q % R) * (L / R)];
            out[base + q * Ns] = acc;
          }
        }
      }
      Ns *= R;
      std::swap(in, out);
    }
    if (in != a) memcpy(a, in, sizeof(cd) * L);
  }
};


}  // namespace lpgb_host
