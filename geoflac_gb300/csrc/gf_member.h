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
    const gf_params *hp; // host parameters of the context
    gf_layout *L;        // host arrays registered with the context
};

extern "C" {
int gf_ctx_view(gf_ctx *c, GfMemberView *v);
unsigned gf_ctx_signature(const gf_ctx *c);
void gf_ctx_advance(gf_ctx *c, unsigned sig); // host bookkeeping after one step
int gf_ctx_take_status(gf_ctx *c);
// the member's stresses or mesh were changed outside its own calls
void gf_ctx_invalidate_forces(gf_ctx *c);
// the device-side part of rsflac.f90:197-236 once the restart files are
// uploaded and marker2elem has run: init_areas, temp0 = temp, heating and
// strain-rate accumulators reset, rmasses, init_visc, dt_mass, dtavg /
// nsrate reset
int gf_ctx_restart_finish(gf_ctx *c);
}
