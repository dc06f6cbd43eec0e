// FP64 instantiation of the step kernels (built with -fmad=false so that
// every product and sum is rounded as in the serial reference).
#include "gf_kernels_impl.cuh"

template struct GfKernels<double>;
