// Mixed-precision instantiation: FP32 element fields and rheology, FP64
// coordinates, temperatures, masses and dt reductions.  Indices are 32-bit
// here (gf_create rejects mixed models whose arrays would overflow them):
// each memory access of these issue-bound kernels then costs fewer integer
// instructions than with 64-bit indices.
#define GF_IDX int
#include "gf_kernels_impl.cuh"

template struct GfKernels<float>;
