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


// ---- per-particle parts of the leapfrog step and of the density / EOS set-up
// (one slot each), shared by the per-kernel step and the fused per-tube step

__device__ __forceinline__ void predictor_one(const FieldPtrs& F, const Side& S, const DevOpts& o, double dt, int i,
                                              int part)
{
    const int t = S.itype[i];
    const bool fixed = (t == NDSPH_ITYPE_BND || t == NDSPH_ITYPE_BNDDUST);
    if (part != 2) {
        double x[3], v[3], f[3];
        for (int d = 0; d < o.ndim; d++) x[d] = F.f[X0 + d][i];
        for (int d = 0; d < 3; d++) { v[d] = F.f[V0 + d][i]; f[d] = F.f[F0 + d][i]; }
        const double h = F.f[HH][i], rho = F.f[RHO][i], dh = F.f[DHDT][i];
        // save (stepND_leapfrog_mhd.f90:70-101)
        for (int d = 0; d < o.ndim; d++) F.f[XIN0 + d][i] = x[d];
        for (int d = 0; d < 3; d++) { F.f[VIN0 + d][i] = v[d]; F.f[FIN0 + d][i] = f[d]; }
        F.f[HIN][i] = h; F.f[RHOIN][i] = rho; F.f[DHIN][i] = dh;
        // a fixed particle moves by its own saved velocity and force; the rest is held
        for (int d = 0; d < o.ndim; d++) F.f[X0 + d][i] = x[d] + dt * v[d] + 0.5 * dt * dt * f[d];
        if (!fixed) {
            for (int d = 0; d < 3; d++) F.f[V0 + d][i] = (v[d] + dt * f[d]) / (1.0 + 0.0);
            F.f[HH][i] = h + dt * dh;
        }
    }
    if (part != 1) {
        double be[3], db[3], al[3], dal[3];
        for (int d = 0; d < 3; d++) {
            be[d] = F.f[BE0 + d][i]; db[d] = F.f[DB0 + d][i]; al[d] = F.f[AL0 + d][i]; dal[d] = F.f[DAL0 + d][i];
        }
        const double en = F.f[EN][i], den = F.f[DENDT][i];
        for (int d = 0; d < 3; d++) {
            F.f[BIN0 + d][i] = be[d]; F.f[ALIN0 + d][i] = al[d]; F.f[DBIN0 + d][i] = db[d]; F.f[DALIN0 + d][i] = dal[d];
        }
        F.f[ENIN][i] = en; F.f[DENIN][i] = den;
        if (fixed) return;
        if (o.imhd != 0)
            for (int d = 0; d < 3; d++) F.f[BE0 + d][i] = be[d] + dt * db[d];
        if (o.iener != 0) F.f[EN][i] = en + dt * den;
        for (int d = 0; d < 3; d++)
            if (o.iavlim[d] != 0) F.f[AL0 + d][i] = fmin(al[d] + dt * dal[d], 1.0);
    }
}
// a fixed particle after the predictor: its position moves by its source's
// saved velocity and force (stepND_leapfrog_mhd.f90:110-116)
__device__ __forceinline__ void predictor_fixed_x_one(const FieldPtrs& F, const Side& S, const DevOpts& o, double dt,
                                                      int i)
{
    const int t = S.itype[i];
    if (t != NDSPH_ITYPE_BND && t != NDSPH_ITYPE_BNDDUST) return;
    const int j = (S.ireal[i] >= 0) ? S.pos_of_id[S.ireal[i]] : i;
    for (int d = 0; d < o.ndim; d++)
        F.f[X0 + d][i] = F.f[XIN0 + d][i] + dt * F.f[VIN0 + d][j] + 0.5 * dt * dt * F.f[FIN0 + d][j];
}

// iterate_density.f90:79-86 (zero gradh.. on non-fixed particles) and
// hhin = hh (:87); h <= 0 check (:99-102)
__device__ __forceinline__ void density_init_one(const FieldPtrs& F, const Side& S, int k, Reduce* red)
{
    if (S.itype[k] != NDSPH_ITYPE_BND) {
        F.f[GRADH][k] = 0.0; F.f[GRADHN][k] = 0.0; F.f[GRADGRADH][k] = 0.0;
        F.f[DRHODT][k] = 0.0; F.f[DHDT][k] = 0.0;
    }
    double h = F.f[HH][k];
    F.f[HNEXT][k] = h;
    F.f[HDEN0][k] = h;
    if (!(h > 2.2250738585072014e-308)) raise_err(red, NDSPH_E_H_NONPOS, S.id[k]);
}

// fixed particles take rho.. from their source after each NR pass
// (iterate_density.f90:312-328)
__device__ __forceinline__ void fixed_density_copy_one(const FieldPtrs& F, const Side& S, int k)
{
    if (S.itype[k] != NDSPH_ITYPE_BND) return;
    int src_id = S.ireal[k];
    if (src_id < 0) return;
    int j = S.pos_of_id[src_id];
    const int fl[7] = {RHO, RHOALT, DRHODT, DHDT, HH, GRADH, GRADHN};
    for (int q = 0; q < 7; q++) F.f[fl[q]][k] = F.f[fl[q]][j];
    // 1/h and the list's h follow the copied h
    const double h = F.f[HH][k];
    S.h1[k] = 1.0 / h;
    float4 xw = S.xs[k];
    xw.w = (float)h;
    S.xs[k] = xw;
}

// conservative2primitive (in-scope part) + equation_of_state eos.f90:40-106
// for slot k; returns the slot's share of stressmax (ratesND_mhd.f90:232-245)
__device__ __forceinline__ double eos_one(const FieldPtrs& F, const Side& S, const DevOpts& o, int k, Reduce* red)
{
    double st = 0.0;
    double rho = F.f[RHO][k];
    F.f[DENS][k] = rho;
    // the FP64 rates sweep reads 1/rho of every neighbour: one division
    // per particle instead of one per pair
    if (o.precision == NDSPH_PREC_FP64) F.f[RHO1][k] = 1.0 / rho;
    double B[3] = {0.0, 0.0, 0.0};
    if (o.imhd >= 11) {
        for (int d = 0; d < 3; d++) B[d] = F.f[BE0 + d][k];
    } else if (o.imhd >= 1 && o.imhd <= 9) {
        for (int d = 0; d < 3; d++) B[d] = F.f[BE0 + d][k] * rho;
    }
    if (o.imhd != 0)
        for (int d = 0; d < 3; d++) F.f[BF0 + d][k] = B[d];
    double uu = F.f[EN][k];
    double pr = F.f[PR][k], cs = F.f[CS][k];
    int it = S.itype[k];
    // the reference stops on a negative thermal energy (eos.f90:66-72)
    if (o.iener != 0 && uu < 0.0) raise_err(red, NDSPH_E_U_NEG, S.id[k]);
    if (o.iener == 0) {
        if (rho > 0.0 && it == NDSPH_ITYPE_GAS) {
            // rho^gamma: FP64 pow in the parity form; in the FP32 form the
            // pressure only enters FP32 pair terms, and FP64 pow costs
            // ~100 FP64 instructions on this part, so powf (~1e-7 relative)
            if (o.precision == NDSPH_PREC_FP32)
                pr = o.polyk * (double)powf((float)rho, (float)o.gamma);
            else
                pr = o.polyk * pow(rho, o.gamma);
            cs = (o.precision == NDSPH_PREC_FP32) ? (double)sqrtf((float)o.gamma * (float)pr / (float)rho)
                                                  : sqrt(o.gamma * pr / rho);
        } else if (it != NDSPH_ITYPE_BND) {
            pr = 0.0;
        }
        if (fabs(o.gamma - 1.0) > 1.e-3 && rho > 0.0) uu = pr / ((o.gamma - 1.0) * rho);
    } else {
        if (rho > 0.0) {
            pr = (o.gamma - 1.0) * uu * rho;
            // FP32 form: c_s only enters FP32 pair terms and timestep bounds;
            // gamma P / rho = gamma (gamma - 1) u without the FP64 divide and
            // square root (~40 FP64 pipe slots per particle on this part)
            cs = (o.precision == NDSPH_PREC_FP32)
                     ? (double)sqrtf((float)(o.gamma * (o.gamma - 1.0)) * (float)uu)
                     : sqrt(o.gamma * pr / rho);
        }
    }
    F.f[UU][k] = uu;
    F.f[PR][k] = pr;
    F.f[CS][k] = cs;
    if (o.imhd != 0 && o.imagforce == 2) {
        double B2 = B[0] * B[0] + B[1] * B[1] + B[2] * B[2];
        st = fmax(0.5 * B2 - pr, 0.0);
    }
    return st;
}

// copy_particle copy_particle.f90:28-80 for fixed particles
// (conservative2primitive.f90:430-441): everything but x and vel
__device__ __forceinline__ void fixed_copy_one(const FieldPtrs& F, const Side& S, int k)
{
    if (S.itype[k] != NDSPH_ITYPE_BND && S.itype[k] != NDSPH_ITYPE_BNDDUST) return;
    int src_id = S.ireal[k];
    if (src_id < 0) return;
    int j = S.pos_of_id[src_id];
    const int fl[] = {PM, RHO, RHOALT, HH, UU, EN, BE0, BE1, BE2, BF0, BF1, BF2, AL0, AL1, AL2, GRADH, GRADHN,
                      GRADGRADH, CS, PR, DENS, F0, F1, F2, DRHODT, DUDT, DENDT, DB0, DB1, DB2, DHDT, DAL0, DAL1,
                      DAL2, DIVB, CB0, CB1, CB2, RHO1};
    for (unsigned q = 0; q < sizeof(fl) / sizeof(fl[0]); q++) F.f[fl[q]][k] = F.f[fl[q]][j];
}

// the leapfrog corrector of slot i (stepND_leapfrog_mhd.f90:185-221) written back
__device__ __forceinline__ void corrector_one(const FieldPtrs& F, const Side& S, const DevOpts& o, double dt, int i,
                                              Reduce* red)
{
    Corrected c;
    corrector_values(F, S, o, dt, i, c);
    const int t = S.itype[i];
    const bool fixed = (t == NDSPH_ITYPE_BND || t == NDSPH_ITYPE_BNDDUST);
    if (!fixed && !(c.h > 0.0)) raise_err(red, NDSPH_E_H_NONPOS, S.id[i]);
    // write back what the step changes
    for (int d = 0; d < 3; d++) F.f[V0 + d][i] = c.v[d];
    if (fixed || o.imhd != 0)
        for (int d = 0; d < 3; d++) F.f[BE0 + d][i] = c.be[d];
    for (int d = 0; d < 3; d++)
        if (fixed || o.iavlim[d] != 0) F.f[AL0 + d][i] = c.al[d];
    if (fixed) F.f[RHO][i] = c.rho;
    F.f[HH][i] = c.h;
    if (fixed || o.iener != 0) F.f[EN][i] = c.en;
#pragma unroll
    for (int d = 0; d < 3; d++)
        if (d < o.ndim && o.ibound[d] == 3) F.f[X0 + d][i] = c.x[d];
}

}  // namespace ndsph
