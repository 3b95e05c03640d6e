// The hot-path kernels on the mixed-radix register FFT (fft_mr.cuh) for the padded
// sizes of an axis 9 to 16 pixels off centre at N0 = 512 and of an axis up to 8
// pixels off centre at N0 = 1024: N = 544 = 16 * 2 * 17 and 1040 = 16 * 5 * 13
// (Ntheta = N, Nrho = 2N: 1088, 2080).
#include "lp_p2.cuh"

namespace lpgb {

using MixedLengths3 = Lengths<544, 1040, 1088, 2080>;
LP_DEFINE_LENGTH_SET(mr3, MixedLengths3)

}  // namespace lpgb
