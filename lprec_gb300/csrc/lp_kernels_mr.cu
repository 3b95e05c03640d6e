// The hot-path kernels on the mixed-radix register FFT (fft_mr.cuh) for padded
// sizes that are not powers of two: N = 528 (an off-centre axis at N0 = 512),
// 1008, 1536, 2016 (the reference's foam data) -- Ntheta = N and Nrho = 2N.
// Other sizes run the generic shared-memory kernels of lp_kernels.cu.
#include "lp_p2.cuh"

namespace lpgb {

using MixedLengths = Lengths<528, 1008, 1056, 1536, 2016, 3072, 4032>;
LP_DEFINE_LENGTH_SET(mr, MixedLengths)

}  // namespace lpgb
