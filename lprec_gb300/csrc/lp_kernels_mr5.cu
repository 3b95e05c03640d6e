// The hot-path kernels on the mixed-radix register FFT (fft_mr.cuh) for the common
// detector widths N0 = 1280 and 2560 (centred axis): Ntheta 1280 = 16 * 16 * 5 and
// 2560, Nrho 2560 and 5120 = 16 * 64 * 5.
#include "lp_p2.cuh"

namespace lpgb {

using MixedLengths5 = Lengths<1280, 2560, 5120>;
LP_DEFINE_LENGTH_SET(mr5, MixedLengths5)

}  // namespace lpgb
