// Library-internal view of a context, for the ensemble driver (gf_batch.cu).
#pragma once

#include "gf_ctx.h"

struct GfMemberView {
    const DevParams *P;
    DevClock *C;
    DevArrays A;
    GfDims d;
    int mode, idt_scale, movegrid, itherm, nmarkers;
    int nloop, nsrate;
    int ifreq_rmasses, ifreq_visc, ifreq_imasses, ifreq_avgsr;
    double z0, rzbo, g;
    cudaStream_t s;
};

extern "C" {
int gf_ctx_view(gf_ctx *c, GfMemberView *v);
unsigned gf_ctx_signature(const gf_ctx *c);
void gf_ctx_advance(gf_ctx *c, unsigned sig); // host bookkeeping after one step
int gf_ctx_take_status(gf_ctx *c);
}
