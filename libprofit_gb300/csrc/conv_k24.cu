// Single-precision direct convolution kernels with a PSF row stride of 24
// floats compiled in (conv.cuh).
#include "conv.cuh"

namespace pf {

PF_CONV_FIXED_DEF(24)

}  // namespace pf
