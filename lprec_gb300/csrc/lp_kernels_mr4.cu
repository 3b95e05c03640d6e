// The hot-path kernels on the mixed-radix register FFT (fft_mr.cuh) for the padded
// sizes of an axis 9 to 16 pixels off centre at N0 = 1024 and N0 = 2048: N = 1056
// (its Nrho 2112 = 16 * 4 * 3 * 11) and 2080 = 16 * 2 * 5 * 13 (Nrho 4160).
#include "lp_p2.cuh"

namespace lpgb {

using MixedLengths4 = Lengths<2112, 4160>;
LP_DEFINE_LENGTH_SET(mr4, MixedLengths4)

}  // namespace lpgb
