// ndsph_step.cuh -- the leapfrog corrector's per-particle arithmetic
// (stepND_leapfrog_mhd.f90:185-221), shared by the corrector kernel and by
// the rates sweep of a host-buffer step, which copies each particle's
// corrected state out before the corrector runs.
#pragma once
#include "ndsph_launch.h"

namespace ndsph {

// the corrected state of slot i (stepND_leapfrog_mhd.f90:185-221), read-only:
// the corrector writes it back, a host-buffer step also copies it out before
struct Corrected {
    double x[3], v[3], be[3], al[3], h, en, rho;
};
__device__ __forceinline__ void corrector_values(const FieldPtrs& F, const Side& S, const DevOpts& o, double dt,
                                                 int i, Corrected& c)
{
    const double hdt = 0.5 * dt;
    const int t = S.itype[i];
    c.rho = F.f[RHO][i];
    if (t == NDSPH_ITYPE_BND || t == NDSPH_ITYPE_BNDDUST) {
#pragma unroll
        for (int d = 0; d < 3; d++) {
            c.v[d] = F.f[VIN0 + d][i];
            c.be[d] = F.f[BIN0 + d][i];
            c.al[d] = F.f[ALIN0 + d][i];
        }
        c.rho = F.f[RHOIN][i];
        c.h = F.f[HIN][i];
        c.en = F.f[ENIN][i];
    } else {
        for (int d = 0; d < 3; d++)
            c.v[d] = (F.f[VIN0 + d][i] + hdt * (F.f[F0 + d][i] + F.f[FIN0 + d][i])) / (1.0 + 0.0);
        for (int d = 0; d < 3; d++)
            c.be[d] = (o.imhd != 0) ? F.f[BIN0 + d][i] + hdt * (F.f[DB0 + d][i] + F.f[DBIN0 + d][i])
                                    : F.f[BE0 + d][i];
        c.h = F.f[HIN][i] + hdt * (F.f[DHDT][i] + F.f[DHIN][i]);
        c.en = (o.iener != 0) ? F.f[ENIN][i] + hdt * (F.f[DENDT][i] + F.f[DENIN][i]) : F.f[EN][i];
        for (int d = 0; d < 3; d++)
            c.al[d] = (o.iavlim[d] != 0)
                          ? fmin(F.f[ALIN0 + d][i] + hdt * (F.f[DAL0 + d][i] + F.f[DALIN0 + d][i]), 1.0)
                          : F.f[AL0 + d][i];
    }
    // boundary after the corrector (:221)
#pragma unroll
    for (int d = 0; d < 3; d++) {
        if (d >= o.ndim) { c.x[d] = 0.0; continue; }
        double x = F.f[X0 + d][i];
        if (o.ibound[d] == 3) {
            if (x > o.xmax[d]) x = __dsub_rn(__dadd_rn(o.xmin[d], x), o.xmax[d]);
            else if (x < o.xmin[d]) x = __dsub_rn(o.xmax[d], __dsub_rn(o.xmin[d], x));
        }
        c.x[d] = x;
    }
}

// a host-buffer step in pieces: particle h (host order) = slot i, its rates
// outputs (already in the slab) and corrected state into the staging
__device__ __forceinline__ void step_tail_one(const FieldPtrs& F, const DevOpts& o, double dt, int i, size_t h,
                                              const Side& S, const StepTail& t)
{
    Corrected c;
    corrector_values(F, S, o, dt, i, c);
    const int nd = o.ndim;
    if (t.x) {
#pragma unroll
        for (int d = 0; d < 3; d++)
            if (d < nd) t.x[h * nd + d] = c.x[d];
    }
    if (t.v) for (int d = 0; d < 3; d++) t.v[h * 3 + d] = c.v[d];
    if (t.be) for (int d = 0; d < 3; d++) t.be[h * 3 + d] = c.be[d];
    if (t.al) for (int d = 0; d < 3; d++) t.al[h * 3 + d] = c.al[d];
    if (t.en) t.en[h] = c.en;
    if (t.hh) t.hh[h] = c.h;
    if (t.drhodt) t.drhodt[h] = F.f[DRHODT][i];
    if (t.dhdt) t.dhdt[h] = F.f[DHDT][i];
    if (t.force) for (int d = 0; d < 3; d++) t.force[h * 3 + d] = F.f[F0 + d][i];
    if (t.db) for (int d = 0; d < 3; d++) t.db[h * 3 + d] = F.f[DB0 + d][i];
    if (t.dal) for (int d = 0; d < 3; d++) t.dal[h * 3 + d] = F.f[DAL0 + d][i];
    if (t.curlb) for (int d = 0; d < 3; d++) t.curlb[h * 3 + d] = F.f[CB0 + d][i];
    if (t.gdv) for (int d = 0; d < 3; d++) t.gdv[h * 3 + d] = F.f[GDV0 + d][i];
    if (t.dudt) t.dudt[h] = F.f[DUDT][i];
    if (t.dendt) t.dendt[h] = F.f[DENDT][i];
    if (t.divb) t.divb[h] = F.f[DIVB][i];
    if (t.del2u) t.del2u[h] = F.f[DEL2U][i];
}

}  // namespace ndsph
