// The hot-path kernels on the mixed-radix register FFT (fft_mr.cuh) for padded
// sizes that are not powers of two (Ntheta = N, Nrho = 2N), the shorter lengths:
// Ntheta 528 (an off-centre axis at N0 = 512), 1008, 1536, 2016 (the reference's
// foam data) and Nrho 1056, 2016.  lp_kernels_mr2.cu holds the longer ones (a second
// translation unit, so that the two compile in parallel).  Other sizes run the
// generic shared-memory kernels of lp_kernels.cu.
#include "lp_p2.cuh"

namespace lpgb {

using MixedLengths = Lengths<528, 1008, 1056, 1536, 2016>;
LP_DEFINE_LENGTH_SET(mr, MixedLengths)

}  // namespace lpgb
