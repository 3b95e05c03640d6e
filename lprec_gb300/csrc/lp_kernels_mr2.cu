// The hot-path kernels on the mixed-radix register FFT (fft_mr.cuh), the longer
// mixed lengths: Ntheta 2064 = 16 * 3 * 43 (an axis 3 pixels off centre at
// N0 = 2048; the prime 43 runs through the output-parallel stage) and Nrho 3072,
// 4032 (the foam data's N = 2016), 4128.
#include "lp_p2.cuh"

namespace lpgb {

using MixedLengths2 = Lengths<2064, 3072, 4032, 4128>;
LP_DEFINE_LENGTH_SET(mr2, MixedLengths2)

}  // namespace lpgb
