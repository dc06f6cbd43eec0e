// Mixed-precision instantiation: FP32 element fields and rheology, FP64
// coordinates, temperatures, masses and dt reductions.
#include "gf_kernels_impl.cuh"

template struct GfKernels<float>;
