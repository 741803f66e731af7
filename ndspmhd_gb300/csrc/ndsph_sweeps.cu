// ndsph_sweeps.cu -- the two O(N n_neigh) pair sweeps of the hot path.
//
//  k_density<NDIM, FULL, PREC>: density (density_sums.f90:38-379) as a gather
//    when FULL (first NR pass: union criterion q_i<2 or q_j<2 for numneigh),
//    density_partial (:396-658) otherwise (q_i<2 over the active list), with
//    the Newton-Raphson update of iterate_density.f90:163-278 fused as the
//    per-particle epilogue.
//  k_rates<NDIM, PREC>: get_rates (ratesND_mhd.f90:29-979) as a gather over
//    every pair with q_i<2 or q_j<2: rates_core (:1175-1690),
//    artificial_dissipation (:1700-1894), mhd_terms (:2377-2720),
//    drag_forces (:1074-1169); the per-particle post pass (:532-965) is the
//    epilogue.
//
// The reference scatters each unordered pair to both particles; here every
// particle gathers its own side of every pair, so no atomics touch
// per-particle sums and results are deterministic.  The j-side formulas of
// the reference equal the i-side formulas evaluated from j's point of view
// (forces and dB/dt change sign with dr and dv, div B, curl B and du/dt are
// symmetric or flip consistently), so the gather is the same sum in a
// different order.
//
// Neighbour search: particle slots are cell-sorted; one row per particle
// lists the candidates of the stencil around its cell (built by
// k_build_nlist), and the sweeps walk the rows.  Candidates are screened in FP32 with a
// conservative margin on cell-relative coordinates; in the FP64 form the
// survivors are re-tested exactly in FP64 with the reference's own rounding
// (dx = x_i - x_j' with periodic images placed as ghostND_mhd.f90:224-225
// places ghosts, rij2 = dx.dx without FMA, q2 = rij2*h^-2), so the neighbour
// sets match the reference bit for bit.
#include <cstdio>
#include <type_traits>
#include "ndsph_launch.h"
#include "ndsph_step.cuh"

namespace ndsph {

static inline int nblk(long n, int bs) { return (int)((n + bs - 1) / bs); }

// the ghosts' hhmax of particle i's simulation: the max h at its last
// (re)link (ghostND_mhd.f90:218); per simulation in a periodic batch
__device__ __forceinline__ double ghost_hmax(const SweepArgs& a, int i)
{
    return a.o.stacked ? bitsd(a.o.sim_aux[(size_t)a.S.sim[i] * SIMAUX + SA_HG]) : bitsd(a.red->hmax_ghost);
}

__device__ __forceinline__ bool type_match(int ti, int tj)
{
    return (tj == ti) || (ti == NDSPH_ITYPE_GAS && tj == NDSPH_ITYPE_BND) ||
           (tj == NDSPH_ITYPE_GAS && ti == NDSPH_ITYPE_BND) ||
           (ti == NDSPH_ITYPE_DUST && tj == NDSPH_ITYPE_BNDDUST) ||
           (tj == NDSPH_ITYPE_DUST && ti == NDSPH_ITYPE_BNDDUST);
}

// interpolate_kernel* index logic (kernelND.f90:4382-4391) in FP64:
// index = int(q2*ddq2table) clamped to ikern, value + slope*(q2 - index*dq2table)
struct TabIdx {
    int i0;
    double dxx;
};
__device__ __forceinline__ TabIdx tab_index(const Tables& t, double q2)
{
    int idx = (int)__dmul_rn(q2, t.ddq2table);
    if (idx > IKERN || idx < 0) idx = IKERN;
    TabIdx r;
    r.i0 = idx;
    r.dxx = __dsub_rn(q2, __dmul_rn((double)idx, t.dq2table));
    return r;
}
__device__ __forceinline__ double tab_val(const double2* tab, const TabIdx& ix)
{
    double2 e = __ldg(&tab[ix.i0]);
    return e.x + e.y * ix.dxx;
}
struct TabIdxF {
    int i0;
    float dxx;
};
__device__ __forceinline__ TabIdxF tab_indexf(const Tables& t, float q2)
{
    int idx = (int)(q2 * t.ddq2tablef);
    if (idx > IKERN || idx < 0) idx = IKERN;
    TabIdxF r;
    r.i0 = idx;
    r.dxx = q2 - (float)idx * t.dq2tablef;
    return r;
}
__device__ __forceinline__ float tab_valf(const float2* tab, const TabIdxF& ix)
{
    float2 e = __ldg(&tab[ix.i0]);
    return fmaf(e.y, ix.dxx, e.x);
}

// FP32 form: the cubic spline W, dW/dq and d2W/dq2 evaluated directly,
// C (t^3/4 - u^3) with t = max(2-q, 0), u = max(1-q, 0) (kernelND.f90:4143-4192).
// The reference interpolates them linearly in q^2 from its 4001-point tables;
// for q^2 >= KERN_Q2_DIRECT the two agree within 1.4e-7 C (W) and 7.5e-7 C
// (dW/dq), well inside the form's 1e-5 budget, and no table is read.  Below
// it (a few per cent of pairs) the table is used: there the linear
// interpolation in q^2 departs from the polynomial (dW/dq ~ q ~ sqrt(q^2)).
constexpr float KERN_Q2_DIRECT = 0.25f;
struct KerF {
    float w, gw, ggw;
};
__device__ __forceinline__ KerF kern_cubic(float q, float c)
{
    const float t = fmaxf(2.0f - q, 0.0f), u = fmaxf(1.0f - q, 0.0f);
    const float t2 = t * t, u2 = u * u;
    KerF k;
    k.w = c * (0.25f * t2 * t - u2 * u);
    k.gw = c * (3.0f * u2 - 0.75f * t2);
    k.ggw = c * (1.5f * t - 6.0f * u);
    return k;
}

// cell offsets (dx, dy, dz) of a stencil index o = (dx+r) + sw (dy+r) +
// sw^2 (dz+r), r = (sw-1)/2, sw = 3 or 5; the divisions by 3, 9, 5, 25 are
// exact multiply-shifts for o < sw^3 (checked for every o)
template <int NDIM>
__device__ __forceinline__ void stencil_d(unsigned o, int sw, int d[3])
{
    if (NDIM == 1) {   // any odd width
        d[0] = (int)o - ((sw - 1) >> 1);
        d[1] = d[2] = 0;
        return;
    }
    unsigned q, q2;
    int r;
    if (sw == 5) {
        q = (o * 205u) >> 10;    // o / 5
        q2 = (o * 41u) >> 10;    // o / 25
        d[0] = (int)(o - 5u * q);
        d[1] = (int)(q - 5u * q2);
        r = 2;
    } else {
        q = (o * 11u) >> 5;      // o / 3
        q2 = (o * 57u) >> 9;     // o / 9
        d[0] = (int)(o - 3u * q);
        d[1] = (int)(q - 3u * q2);
        r = 1;
    }
    d[2] = (int)q2;
    d[0] -= r;
    d[1] = (NDIM >= 2) ? d[1] - r : 0;
    d[2] = (NDIM >= 3) ? d[2] - r : 0;
}

// stencil cell with periodic wrap; returns false if outside (open dims)
template <int NDIM>
struct Stencil {
    int cc[3];
    int base;   // first cell of the simulation's grid (stacked periodic batch)
    __device__ Stencil(int cell, const Grid& g) { cell_coords(cell, g, cc, &base); }
    // cell at offset d (a stencil of any width) with periodic wrap flags;
    // false if outside an open dimension
    __device__ __forceinline__ bool cell_at_d(const int d[3], const Grid& g, const DevOpts& op, int& cid,
                                              int w[3]) const
    {
        int c[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            w[k] = 0;
            c[k] = cc[k] + d[k];
            if (k < NDIM) {
                if (c[k] < 0) {
                    if (!op.periodic[k]) return false;
                    c[k] += g.nc[k];
                    w[k] = -1;
                } else if (c[k] >= g.nc[k]) {
                    if (!op.periodic[k]) return false;
                    c[k] -= g.nc[k];
                    w[k] = 1;
                }
            }
        }
        cid = base + (c[2] * g.nc[1] + c[1]) * g.nc[0] + c[0];
        return true;
    }
    // offsets and wrap flags of a stored row entry's stencil index
    // o = (dx+r) + sw (dy+r) + sw^2 (dz+r) (the cell exists)
    __device__ __forceinline__ void offset(unsigned o, const Grid& g, int d[3], int w[3]) const
    {
        stencil_d<NDIM>(o, NDIM == 2 ? 3 : g.sw, d);   // 2D always searches 3 wide
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const int c = cc[k] + d[k];
            w[k] = (k < NDIM) ? ((c < 0) ? -1 : ((c >= g.nc[k]) ? 1 : 0)) : 0;
        }
    }
};

// periodic image of x_j as the reference's ghost would place it, and the
// ghost-existence test (0 < distance-to-boundary < radkern*hhmax,
// ghostND_mhd.f90:218).  w = +1: image beyond xmax, w = -1: below xmin.
__device__ __forceinline__ bool image_coord(double xj, int w, int d, const DevOpts& o, double dxbound,
                                            double& xim)
{
    if (w == 0) { xim = xj; return true; }
    if (w > 0) {
        double dist = __dsub_rn(xj, o.xmin[d]);
        xim = __dadd_rn(o.xmax[d], dist);
        return (dist < dxbound) && (dist > 0.0);
    }
    double dist = __dsub_rn(o.xmax[d], xj);
    xim = __dadd_rn(o.xmin[d], __dsub_rn(xj, o.xmax[d]));
    return (dist < dxbound) && (dist > 0.0);
}

// exact FP64 separation and rij2 for slot j seen from x_i
template <int NDIM>
__device__ __forceinline__ bool exact_dx(const FieldPtrs& F, int j, const double xi[3], const int w[3],
                                         const DevOpts& o, double dxbound, double dx[3], double& rij2)
{
    bool exists = true;
#pragma unroll
    for (int d = 0; d < 3; d++) dx[d] = 0.0;
#pragma unroll
    for (int d = 0; d < NDIM; d++) {
        double xim;
        exists &= image_coord(F.f[X0 + d][j], w[d], d, o, dxbound, xim);
        dx[d] = __dsub_rn(xi[d], xim);
    }
    double r = __dmul_rn(dx[0], dx[0]);
    if (NDIM >= 2) r = __dadd_rn(r, __dmul_rn(dx[1], dx[1]));
    if (NDIM >= 3) r = __dadd_rn(r, __dmul_rn(dx[2], dx[2]));
    rij2 = r;
    return exists;
}

// FP32 screen on cell-relative coordinates
template <int NDIM>
__device__ __forceinline__ float screen_r2(const float4& xsi, const float4& xsj, const int d[3], const Grid& g,
                                           float dxf[3])
{
    dxf[0] = (xsi.x - xsj.x) - (float)d[0] * g.csf[0];
    dxf[1] = (NDIM >= 2) ? (xsi.y - xsj.y) - (float)d[1] * g.csf[1] : 0.f;
    dxf[2] = (NDIM >= 3) ? (xsi.z - xsj.z) - (float)d[2] * g.csf[2] : 0.f;
    return dxf[0] * dxf[0] + dxf[1] * dxf[1] + dxf[2] * dxf[2];
}

// reciprocal and square root in the pair precision: exact (IEEE) in FP64,
// the hardware approximations (MUFU, ~1 ulp) in the FP32 form
// The FP32 forms are the PTX approximate instructions with denormals flushed
// (.ftz): without .ftz each one carries a scaling fix-up for denormal inputs,
// which no physical quantity of the pair sums is; that fix-up was ~10 % of
// the 128^3 rates sweep's instructions.
__device__ __forceinline__ float rsqrt_ftz(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float div_ftz(float a, float b)
{
    float y;
    asm("div.approx.ftz.f32 %0, %1, %2;" : "=f"(y) : "f"(a), "f"(b));
    return y;
}
__device__ __forceinline__ float rcp_ftz(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
template <typename R>
__device__ __forceinline__ R rcp(R x)
{
    if constexpr (std::is_same<R, float>::value) return rcp_ftz(x);
    else return 1.0 / x;
}
template <typename R>
__device__ __forceinline__ R sqrtp(R x)
{
    if constexpr (std::is_same<R, float>::value) return x * rsqrt_ftz(fmaxf(x, 1e-37f));
    else return sqrt(x);
}
template <typename R>
__device__ __forceinline__ R divp(R a, R b)
{
    if constexpr (std::is_same<R, float>::value) return div_ftz(a, b);
    else return a / b;
}

// compensated FP32 accumulator (Kahan, branch-free)
struct KSum {
    float s, c;
    __device__ KSum() : s(0.f), c(0.f) {}
    __device__ __forceinline__ void add(float v)
    {
        const float y = v - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double val() const { return (double)s - (double)c; }
    __device__ __forceinline__ float valf() const { return s - c; }
};
// plain FP32 sum with the same interface: the density outputs no later
// quantity of the step reads (the number density, its h-derivative and the
// second h-derivative term), where the compensation's three extra adds a
// pair buy nothing the step uses
struct FSum {
    float s = 0.f;
    __device__ __forceinline__ void add(float v) { s += v; }
    __device__ __forceinline__ float valf() const { return s; }
};

// ===========================================================================
// density + Newton-Raphson
// ===========================================================================
// Candidate sources of the two sweeps: RowSrc walks the slot's neighbour row
// (the sweeps' own loops, below); a source with kRows = false supplies the
// candidates itself through for_each(i, f), calling f(pk) with entries
// packed as in the rows, (j << shift) | stencil offset of j's cell.
struct RowSrc {
    static constexpr bool kRows = true;
};

template <int NDIM, bool FULL, int PREC, class Src>
__device__ __forceinline__ void density_body(const SweepArgs& a, const int i, const Src& src)
{
    const FieldPtrs& F = a.F;
    const DevOpts& o = a.o;
    const Grid& g = a.g;
    const int typei = a.S.itype[i];
    const bool fixed_i = (typei == NDSPH_ITYPE_BND || typei == NDSPH_ITYPE_BNDDUST);
    if (!FULL && typei == NDSPH_ITYPE_BND) return;
    double xi[3] = {0.0, 0.0, 0.0}, vi[3];
#pragma unroll
    for (int d = 0; d < NDIM; d++) xi[d] = F.f[X0 + d][i];
#pragma unroll
    for (int d = 0; d < 3; d++) vi[d] = F.f[V0 + d][i];
    const double hi = F.f[HH][i];
    const double hi1 = a.S.h1[i];
    const double hi21 = __dmul_rn(hi1, hi1);
    const float4 xsi = a.S.xs[i];
    const float hif = (float)hi;
    const float hi21f = __frcp_rn(hif * hif);
    float vif[3] = {0.f, 0.f, 0.f};
    if (PREC == NDSPH_PREC_FP32) {
        const float4 pvi = a.S.pk_v[i];
        vif[0] = pvi.x; vif[1] = pvi.y; vif[2] = pvi.z;
    }
    const double dxbound = 2.0 * ghost_hmax(a, i);
    const float abs_tol = 1e-6f * fmaxf(g.csf[0], fmaxf(g.csf[1], g.csf[2]));

    // FP64 sums (PREC 0) or compensated FP32 sums (PREC 1), in kernel units
    double sw = 0.0, sn = 0.0, sg = 0.0, sgn = 0.0, sgg = 0.0, sd = 0.0;
    KSum fw, fg, fd;
    FSum fn, fgn, fgg;
    int nn = 0;

    Stencil<NDIM> stn(a.S.cell[i], g);
    // the full pass's rule for this particle (union criterion, Jacobi h):
    // every particle of a full pass; in a batch's mixed pass only those of
    // the simulations whose every particle is still unconverged
    const bool uni = FULL && (!a.mixed || o.sim_aux[(size_t)a.S.sim[i] * SIMAUX + SA_FULL] != 0ull);
    // a batch: a particle that converges (or is fixed) ends its simulation's
    // full passes (iterate_density.f90:129-133 per run)
    auto sim_converged = [&]() {
        if (o.batched) {
            unsigned long long* c = o.sim_aux + (size_t)a.S.sim[i] * SIMAUX + SA_CONV;
            if (*c == 0ull) *c = 1ull;
        }
    };
    // one candidate: its list entry, position and type, and (FP32 form) its
    // velocity/mass pack, loaded by the caller
    const unsigned shift = (NDIM == 3) ? (unsigned)g.nlshift : 5u, omask = (1u << shift) - 1u;
    // FP32 form: the kernel sums of one accepted pair (q_i < 2)
    // 1/h of i for the FP32 pair sums: with the rsqrt of q^2 it gives 1/r
    const float hi1f = rcp_ftz(hif);
    auto sums32 = [&](int j, float q2i, const float dxf[3], const float4& pvj) {
        const float mj = pvj.w;
        const float rq = rsqrt_ftz(fmaxf(q2i, 1e-37f));   // 1/q (the sqrt's own rsqrt)
        const float q = q2i * rq;
        float wv, gw, ggw;
        if (q2i >= KERN_Q2_DIRECT) {
            const KerF kf = kern_cubic(q, a.t.cnormf);
            wv = kf.w; gw = kf.gw; ggw = kf.ggw;
        } else {
            const TabIdxF ix = tab_indexf(a.t, q2i);
            wv = tab_valf(a.t.wf, ix);
            gw = tab_valf(a.t.gwf, ix);
            ggw = tab_valf(a.t.ggwf, ix);
        }
        fw.add(mj * wv);
        fn.add(wv);
        const float tg = q * gw + (float)NDIM * wv;
        fg.add(mj * tg);
        fgn.add(tg);
        fgg.add(mj * ((float)(NDIM * (NDIM + 1)) * wv + (float)(2 * (NDIM + 1)) * q * gw + q2i * ggw));
        if (j != i) {
            // 1/r_ij = (1/q)(1/h_i), no reciprocal of its own (a coincident
            // pair has dv.r = 0, and 1/q stays finite)
            float dvr = (vif[0] - pvj.x) * dxf[0];
            if (NDIM >= 2) dvr += (vif[1] - pvj.y) * dxf[1];
            if (NDIM >= 3) dvr += (vif[2] - pvj.z) * dxf[2];
            fd.add(mj * dvr * gw * (rq * hi1f));
        }
    };
    auto pair = [&](unsigned pk, const float4& xsj, int typej, const float4& pvj) {
        const int j = (int)(pk >> shift);
        int d[3], w[3];
        stn.offset(pk & omask, g, d, w);
        float dxf[3];
        const float r2f = screen_r2<NDIM>(xsi, xsj, d, g, dxf);
        const float hm = uni ? fmaxf(hif, xsj.w) : hif;
        if (PREC == NDSPH_PREC_FP64) {
            const float rc = 2.0f * hm * 1.0002f + abs_tol;
            if (r2f > rc * rc) return;
        } else {
            if (r2f >= 4.0f * hm * hm) return;
        }
        if (!type_match(typei, typej)) return;
        if (PREC == NDSPH_PREC_FP64) {
            double dx[3], rij2;
            if (!exact_dx<NDIM>(F, j, xi, w, o, dxbound, dx, rij2)) return;
            const double q2i = __dmul_rn(rij2, hi21);
            bool inc;
            if (uni) {
                const double hj1 = a.S.h1[j];
                const double q2j = __dmul_rn(__dmul_rn(rij2, hj1), hj1);
                inc = (q2i < 4.0) || (q2j < 4.0);
            } else {
                inc = q2i < 4.0;
            }
            if (!inc) return;
            nn++;
            if (q2i >= 4.0 || fixed_i) return;
            const double mj = F.f[PM][j];
            const TabIdx ix = tab_index(a.t, q2i);
            const double wv = tab_val(a.t.w, ix);
            const double gw = tab_val(a.t.gw, ix);
            const double ggw = tab_val(a.t.ggw, ix);
            const double q = sqrt(q2i);
            sw += mj * wv;
            sn += wv;
            const double tg = q * gw + (double)NDIM * wv;
            sg += mj * tg;
            sgn += tg;
            sgg += mj * ((double)(NDIM * (NDIM + 1)) * wv + (double)(2 * (NDIM + 1)) * q * gw + q2i * ggw);
            if (j != i) {
                const double rij = sqrt(rij2);
                double dvr = (vi[0] - F.f[V0][j]) * dx[0];
                if (NDIM >= 2) dvr += (vi[1] - F.f[V1][j]) * dx[1];
                if (NDIM >= 3) dvr += (vi[2] - F.f[V2][j]) * dx[2];
                sd += mj * dvr * gw / (rij + 2.220446049250313e-16);
            }
        } else {
            // FP32 form: separation from the FP32 cell-relative coordinates
            const float q2i = r2f * hi21f;
            nn++;
            if (fixed_i || !(q2i < 4.0f)) return;
            sums32(j, q2i, dxf, pvj);
        }
    };
    if constexpr (!Src::kRows) {
        const bool typed = (PREC == NDSPH_PREC_FP64 || o.idust != 0);
        src.for_each(i, [&](unsigned pk) {
            const int j = (int)(pk >> shift);
            pair(pk, a.S.xs[j], typed ? a.S.itype[j] : typei,
                 PREC == NDSPH_PREC_FP64 ? make_float4(0.f, 0.f, 0.f, 0.f) : a.S.pk_v[j]);
        });
    } else if (PREC == NDSPH_PREC_FP64) {
        const int ncand = a.S.nl_cnt[i];
        const unsigned* row = a.S.nl + (size_t)i * a.nl_stride;
        const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int k = 0; k < ncand; k++) {
            const unsigned pk = row[k];
            const int j = (int)(pk >> shift);
            pair(pk, a.S.xs[j], a.S.itype[j], z4);
        }
    } else {
        const int ncand = a.S.nl_cnt[i];
        const unsigned* row = a.S.nl + (size_t)i * a.nl_stride;
        // FP32 form: four candidates' loads in flight at once (the pair work
        // is short, so the loop is bound by load latency otherwise)
        // rows are 16-byte aligned with a stride of a multiple of 4 entries
        // without dust every type pair matches; rows split by type hold only
        // the slot's own type here
        const bool typed = (o.idust != 0) && !a.typed_rows;
        // the next four row entries are loaded while this group's positions
        // and packs are fetched and summed (1.20 -> 1.16 ms of density
        // passes per 128^3 step)
        uint4 rn = make_uint4(0u, 0u, 0u, 0u);
        if (ncand > 0) rn = *reinterpret_cast<const uint4*>(row);
        for (int k0 = 0; k0 < ncand; k0 += 4) {
            const uint4 r4 = rn;
            if (k0 + 4 < ncand) rn = *reinterpret_cast<const uint4*>(row + k0 + 4);
            unsigned pk[4] = {r4.x, r4.y, r4.z, r4.w};
            float4 xj[4], vj[4];
            int tj[4];
#pragma unroll
            for (int u = 0; u < 4; u++) if (k0 + u >= ncand) pk[u] = (unsigned)i << shift;
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int j = (int)(pk[u] >> shift);
                xj[u] = a.S.xs[j];
                tj[u] = typed ? a.S.itype[j] : typei;
                vj[u] = a.S.pk_v[j];
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (k0 + u < ncand) pair(pk[u], xj[u], tj[u], vj[u]);
        }
    }
    a.S.numneigh[i] = nn;
    if (fixed_i) {
        if (o.learned) F.f[HROOT][i] = hi;
        sim_converged();
        return;
    }

    // ---- sums in reference units and the Newton-Raphson update
    // (iterate_density.f90:163-278).  FP64 for the parity form.  The FP32
    // form keeps FP64 for rho (its compensated sum carries ~48 bits), the
    // residual f = m (hfact/h)^ndim - rho (a difference ~1e-3 of its terms)
    // and h, and runs omega, dh/drho, the other sums and the second
    // derivative in FP32: an FP64 division costs ~30 FP32 issue slots on
    // this part, and an FP32 residual would move the convergence decision of
    // particles near the tolerance ----
    typedef typename std::conditional<PREC == NDSPH_PREC_FP64, double, float>::type E;
    double hfac = hi1;
    if (NDIM >= 2) hfac *= hi1;
    if (NDIM >= 3) hfac *= hi1;
    double rho;
    E hfacE, h1E, Esn, Esg, Esgn, Esgg, Esd;
    if constexpr (PREC == NDSPH_PREC_FP64) {
        rho = hfac * sw;
        hfacE = hfac; h1E = hi1;
        Esn = sn; Esg = sg; Esgn = sgn; Esgg = sgg; Esd = sd;
    } else {
        rho = hfac * fw.val();
        hfacE = (float)hfac; h1E = (float)hi1;
        Esn = fn.valf(); Esg = fg.valf(); Esgn = fgn.valf(); Esgg = fgg.valf(); Esd = fd.valf();
    }
    const E rhoalt = hfacE * Esn;
    E gradh = -hfacE * h1E * Esg;
    const E gradhn = -hfacE * h1E * Esgn;
    E gradgradh = hfacE * h1E * h1E * Esgg;
    E drhodt = hfacE * h1E * Esd;

    const double pm = F.f[PM][i];
    const double hfact = o.hfact;
    const int its = a.d_its ? *a.d_its : a.its;
    if (rho <= 1.e-6 && rho <= 0.0) {
        raise_err(a.red, NDSPH_E_RHO_NONPOS, a.S.id[i]);
        return;
    }
    const E dwdhsumi = gradh;
    E dhdrhoi, omegai, d2hdrho2i;
    double hnew;
    if constexpr (PREC == NDSPH_PREC_FP64) {
        // the reference's expressions and association (parity form)
        double hb = hi / hfact;
        double hpow = hb;
        if (NDIM >= 2) hpow = hpow * hb;
        if (NDIM >= 3) hpow = hpow * hb;
        const double rhoi = pm / hpow;
        dhdrhoi = -hi / ((double)NDIM * rho);
        omegai = 1.0 - dhdrhoi * gradh;
        if (omegai < 1.e-5 && fabs(omegai) == 0.0) omegai = 1.0;
        gradh = 1.0 / omegai;
        const double func = rhoi - rho;
        const double dfdh = omegai / dhdrhoi;
        const double rn = rho * (double)NDIM;
        d2hdrho2i = hi * (double)(NDIM + 1) / (rn * rn);
        hnew = hi - func / dfdh;
    } else {
        // f/f' = f dh/drho / omega
        const double hb1 = hfact * hi1;
        double hpow1 = hb1;
        if (NDIM >= 2) hpow1 = hpow1 * hb1;
        if (NDIM >= 3) hpow1 = hpow1 * hb1;
        const float func = (float)(pm * hpow1 - rho);
        const float rhof = (float)rho;
        const float rho1 = __frcp_rn(rhof);
        dhdrhoi = -hif * rho1 * (1.0f / (float)NDIM);
        omegai = 1.0f - dhdrhoi * gradh;
        if (omegai < 1.e-5f && fabsf(omegai) == 0.0f) omegai = 1.0f;
        gradh = __frcp_rn(omegai);
        d2hdrho2i = hif * (float)(NDIM + 1) * (rho1 * rho1) * (1.0f / (float)(NDIM * NDIM));
        hnew = hi - (double)(func * dhdrhoi * gradh);
    }
    gradgradh = (E)rho * (d2hdrho2i * dwdhsumi + dhdrhoi * dhdrhoi * gradgradh);
    if (hnew > 1.2 * hi) hnew = 1.2 * hi;
    else if (hnew < 0.8 * hi) hnew = 0.8 * hi;
    if (hnew <= 0.0 || (double)gradh <= 2.2250738585072014e-308) {
        hnew = hfact * pow(pm / rho, 1.0 / (double)NDIM);
    } else if (its > 100) {
        hnew = hfact * pow(pm / rho, 1.0 / (double)NDIM);
    }
    bool relink = false;
    if (nn <= 1) {
        hnew = hi + o.psep;
        relink = true;
    }
    const double hin = F.f[HDEN0][i];
    const bool converged =
        ((PREC == NDSPH_PREC_FP64 ? fabs((hnew - hi) / hin) < o.tolh : fabs(hnew - hi) < o.tolh * hin) &&
         omegai > (E)0) ||
        o.maxdensits == 0;
    double* hdst = FULL ? F.f[HNEXT] : F.f[HH];
    if (!converged) {
        // warp-aggregated append: the lanes running here together take
        // consecutive entries in lane order, so the next pass's warps read
        // runs of neighbouring slots (spatially close particles) instead of
        // one slot per atomic in arbitrary order
        const unsigned am = __activemask();
        const int lane = (int)(threadIdx.x & 31u);
        const int leader = __ffs(am) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(a.ncalc_next, __popc(am));
        base = __shfl_sync(am, base, leader);
        a.S.active_next[base + __popc(am & ((1u << lane) - 1u))] = i;
        if (its <= o.maxdensits) {
            hdst[i] = hnew;
            if (!FULL) {
                // a partial pass reads only its own h: keep 1/h and the list's h current
                a.S.h1[i] = 1.0 / hnew;
                float4 xw = a.S.xs[i];
                xw.w = (float)hnew;
                a.S.xs[i] = xw;
            }
        }
        if (hnew > ghost_hmax(a, i)) {
            relink = true;
            if (o.stacked) o.sim_aux[(size_t)a.S.sim[i] * SIMAUX + SA_RELINK] = 1ull;
        }
        if (Src::kRows && (float)hnew + a.nl_dmax > a.S.hb[i] * a.nl_skin) a.red->nl_stale = 1;
    } else {
        sim_converged();
        drhodt = drhodt * gradh;
        F.f[DHDT][i] = (double)(dhdrhoi * drhodt);
        // learned h: the training target is the Newton step from the
        // converged h, the root to second order, not h itself (which the
        // tolerance leaves up to ~tolh from it)
        if (o.learned) F.f[HROOT][i] = hnew;
    }
    if (relink) a.red->redolink = 1;
    F.f[RHO][i] = (double)rho;
    F.f[RHOALT][i] = (double)rhoalt;
    F.f[DRHODT][i] = (double)drhodt;
    F.f[GRADH][i] = (double)gradh;
    F.f[GRADHN][i] = (double)gradhn;
    F.f[GRADGRADH][i] = (double)gradgradh;
}

template <int NDIM, bool FULL, int PREC>
__global__ void __launch_bounds__(128) k_density(SweepArgs a)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    int i;
    if (FULL && !a.mixed) {
        if (t >= a.n) return;
        i = t;
    } else {
        const int nlist = a.d_nlist ? *a.d_nlist : a.nlist;
        if (t >= nlist) return;
        i = a.S.active[t];
    }
    density_body<NDIM, FULL, PREC>(a, i, RowSrc{});
}

void launch_density(const SweepArgs& a, bool full, cudaStream_t st)
{
    const int bs = 128;
    const int nthreads = (full && !a.mixed) ? a.n : (a.d_nlist ? a.n : a.nlist);
    if (nthreads <= 0) return;
    const int nb = nblk(nthreads, bs);
#define DLAUNCH(ND, FU, PR) NDSPH_COUNT_LAUNCH, k_density<ND, FU, PR><<<nb, bs, 0, st>>>(a)
    if (a.o.precision == NDSPH_PREC_FP64) {
        if (a.o.ndim == 1) { if (full) DLAUNCH(1, true, 0); else DLAUNCH(1, false, 0); }
        else if (a.o.ndim == 2) { if (full) DLAUNCH(2, true, 0); else DLAUNCH(2, false, 0); }
        else { if (full) DLAUNCH(3, true, 0); else DLAUNCH(3, false, 0); }
    } else {
        if (a.o.ndim == 1) { if (full) DLAUNCH(1, true, 1); else DLAUNCH(1, false, 1); }
        else if (a.o.ndim == 2) { if (full) DLAUNCH(2, true, 1); else DLAUNCH(2, false, 1); }
        else { if (full) DLAUNCH(3, true, 1); else DLAUNCH(3, false, 1); }
    }
#undef DLAUNCH
}

// ===========================================================================
// rates
// ===========================================================================
template <typename R>
struct Acc;
template <>
struct Acc<double> {
    double v = 0.0;
    __device__ __forceinline__ void add(double x) { v += x; }
    __device__ __forceinline__ double val() const { return v; }
};
template <>
struct Acc<float> {
    KSum k;
    __device__ __forceinline__ void add(float x) { k.add(x); }
    __device__ __forceinline__ double val() const { return k.val(); }
    __device__ __forceinline__ float valf() const { return k.valf(); }
};
// plain sum in the pair precision: the sources of the dissipation switches
// (del2u, graddivv), which only enter dalpha/dt and carry no cancellation
// the switches are sensitive to, and div B and curl B, outputs that no later
// quantity of the step reads (each compensated sum costs three more adds a
// pair: the four plain ones here took the 128^3 sweep from 2.52 to 2.47 ms)
template <typename R>
struct AccPlain {
    R v = 0;
    __device__ __forceinline__ void add(R x) { v += x; }
    __device__ __forceinline__ double val() const { return (double)v; }
    __device__ __forceinline__ R valf() const { return v; }
};
// an accumulator's value in the pair precision R: for FP32, the compensated
// pair's difference rounded once in FP32 (the same float as rounding its
// exact FP64 difference), with no FP64 conversion on the way
template <typename R, typename A>
__device__ __forceinline__ R accv(const A& x)
{
    if constexpr (std::is_same<R, float>::value) return x.valf();
    else return x.val();
}

// per-particle quantities the rates sweep reads for either side of a pair
// gradh: the grad-h term itself in the FP64 form; in the FP32 form the pack's
// m gradh h^-(ndim+1)
template <typename R>
struct PData {
    R vx, vy, vz, m, rho, pr, cs, u, Bx, By, Bz, gradh, a0, a1, a2, h;
};
template <int PREC>
__device__ __forceinline__ void load_p(const SweepArgs& a, int j,
                                       PData<typename std::conditional<PREC == 0, double, float>::type>& q)
{
    if constexpr (PREC == NDSPH_PREC_FP64) {
        const FieldPtrs& F = a.F;
        q.vx = F.f[V0][j]; q.vy = F.f[V1][j]; q.vz = F.f[V2][j]; q.m = F.f[PM][j];
        q.rho = F.f[RHO][j]; q.pr = fmax(F.f[PR][j], 0.0); q.cs = F.f[CS][j]; q.u = F.f[UU][j];
        q.Bx = F.f[BF0][j]; q.By = F.f[BF1][j]; q.Bz = F.f[BF2][j]; q.gradh = F.f[GRADH][j];
        q.a0 = F.f[AL0][j]; q.a1 = F.f[AL1][j]; q.a2 = F.f[AL2][j]; q.h = F.f[HH][j];
    } else {
        const float4 v = a.S.pk_v[j], t = a.S.pk_t[j], b = a.S.pk_b[j], al = a.S.pk_a[j];
        q.vx = v.x; q.vy = v.y; q.vz = v.z; q.m = v.w;
        q.rho = t.x; q.pr = t.y; q.cs = t.z; q.u = t.w;
        q.Bx = b.x; q.By = b.y; q.Bz = b.z; q.gradh = b.w;   // m gradh h^-(ndim+1)
        q.a0 = al.x; q.a1 = al.y; q.a2 = al.z; q.h = al.w;
    }
}


#ifndef NDSPH_RATES_FP32_MINB
#define NDSPH_RATES_FP32_MINB 4
#endif
constexpr int RATES_BS = 128;      // threads per block of the rates sweep
#ifndef NDSPH_RATES_CHUNK
#define NDSPH_RATES_CHUNK 80
#endif
// accepted entries per thread per chunk of the 3D FP32 rows (~90 candidates)
template <int NDIM>
constexpr int rates_chunk() { return NDSPH_RATES_CHUNK; }
// every lane of a warp calls it together (the reductions at its end are warp
// shuffles, and block-wide in a one-simulation FP32 sweep): `live` false runs
// an empty candidate set on slot i.  TYPED: two particle types (the 3D FP32
// sweep of a gas + dust run, rows split by type), see the two runs below.
template <int NDIM, int PREC, class Src, bool TYPED = false>
__device__ __forceinline__ void rates_body(const SweepArgs& a, const int i, const bool live, const Src& src)
{
    typedef typename std::conditional<PREC == NDSPH_PREC_FP64, double, float>::type R;
    const FieldPtrs& F = a.F;
    const DevOpts& o = a.o;
    const Grid& g = a.g;
    const int typei = a.S.itype[i];
    double xi[3] = {0.0, 0.0, 0.0};
    if (PREC == NDSPH_PREC_FP64) {
#pragma unroll
        for (int d = 0; d < NDIM; d++) xi[d] = F.f[X0 + d][i];
    }
    const double hi1_d = a.S.h1[i];
    const double hi21_d = hi1_d * hi1_d;
    const float4 xsi = a.S.xs[i];
    const float hif = xsi.w;
    const double dxbound = 2.0 * ghost_hmax(a, i);
    const float abs_tol = 1e-6f * fmaxf(g.csf[0], fmaxf(g.csf[1], g.csf[2]));

    PData<R> pi;
    load_p<PREC>(a, i, pi);
    const R hi = pi.h;
    const R hi1 = (PREC == 0) ? (R)hi1_d : rcp(hi);
    R hfacgrki = hi1 * hi1;
    if (NDIM >= 2) hfacgrki *= hi1;
    if (NDIM >= 3) hfacgrki *= hi1;
    const R vi[3] = {pi.vx, pi.vy, pi.vz};
    const R rhoi = pi.rho;
    const R rho1i = rcp(rhoi);
    const R rho21i = rho1i * rho1i;
    const R pri = pi.pr;
    const R Prho2i = pri * rho21i;
    const R csi = pi.cs;
    const R ui = pi.u;
    const R alphai = pi.a0, alphaui = pi.a1, alphaBi = pi.a2;
    const R gradhi = (PREC == NDSPH_PREC_FP64) ? pi.gradh : (R)F.f[GRADH][i];
    // FP32 form: h^-(ndim+1) gradh of i, the j-independent factor of i's
    // kernel gradient
    const R hgi = hfacgrki * gradhi;
    const bool mhd = (o.imhd != 0);
    R Bi[3] = {0, 0, 0}, Brhoi[3] = {0, 0, 0};
    R B2i = 0, Brho2i = 0, va2i = 0;
    if (mhd) {
        Bi[0] = pi.Bx; Bi[1] = pi.By; Bi[2] = pi.Bz;
#pragma unroll
        for (int d = 0; d < 3; d++) Brhoi[d] = Bi[d] * rho1i;
        B2i = Bi[0] * Bi[0] + Bi[1] * Bi[1] + Bi[2] * Bi[2];
        Brho2i = B2i * rho21i;
        va2i = B2i * rho1i;
    }
    const R vsig2i = csi * csi + va2i;
    const R stressmax = (R)bitsd(o.batched ? o.sim_red[(size_t)a.S.sim[i] * SIMRED + SR_STRESS]
                                           : a.red->stressmax);
    const R beta = (R)o.beta;
    const bool i_dust = (typei == NDSPH_ITYPE_DUST);

    Acc<R> fx, fy, fz, dbx, dby, dbz, du;
    AccPlain<R> d2u, gx, gy, gz, dvb, cbx, cby, cbz;
    R dtc = (R)1.e6, dtav = (R)3.0e38, vsmax = 0, tsmin = (R)3.0e38, hcsts = 0;
    // FP64 form: the two timestep minima as the pair (h, v) of the smallest
    // h / v, compared by cross-multiplication and divided once per particle
    R dtc_h = (R)1.e6, dtc_v = 1, dtav_h = (R)3.0e38, dtav_v = 1;

    Stencil<NDIM> stn(a.S.cell[i], g);
    // the terms of one candidate pair (rates_core, artificial_dissipation,
    // mhd_terms, drag_forces for the pair (i, j)); returns early when the
    // pair is out of range
    const unsigned shift = (NDIM == 3) ? (unsigned)g.nlshift : 5u, omask = (1u << shift) - 1u;
    // pre: (FP32 form) the candidate's position and its four packs, loaded
    // by the caller ahead of the pair (nullptr: loaded here); tpre its type
    auto pair_terms = [&](const unsigned pk, const float4* pre, int tpre) {
            const int j = (int)(pk >> shift);
            if (j == i) return;
            int d[3], w[3];
            stn.offset(pk & omask, g, d, w);
            const float4 xsj = pre ? pre[0] : a.S.xs[j];
            float dxf[3];
            const float r2f = screen_r2<NDIM>(xsi, xsj, d, g, dxf);
            const float hm = fmaxf(hif, xsj.w);
            R dr[3], rij, q2i, q2j, hj1;
            double irij = 0.0;   // FP64 form: 1/rij, reused by the conduction term
            float irf = 0.f;     // FP32 form: the same, the screen's rsqrt
            if constexpr (PREC == NDSPH_PREC_FP64) {
                const float rc = 2.0f * hm * 1.0002f + abs_tol;
                if (r2f > rc * rc) return;
                double dx[3], rij2;
                if (!exact_dx<NDIM>(F, j, xi, w, o, dxbound, dx, rij2)) return;
                const double hj1d = a.S.h1[j];
                const double q2id = __dmul_rn(rij2, hi21_d);
                const double q2jd = __dmul_rn(rij2, __dmul_rn(hj1d, hj1d));
                if (!(q2id < 4.0 || q2jd < 4.0)) return;
                const double rijd = sqrt(rij2);
                if (rijd <= 2.220446049250313e-16) {
                    if (a.S.itype[j] == typei && rijd < 2.2250738585072014e-308 && typei != 2)
                        raise_err(a.red, NDSPH_E_CLUMP, a.S.id[i]);
                    dr[0] = dr[1] = dr[2] = 0;
                    irij = 1.0 / rijd;
                } else {
                    const double ir = 1.0 / rijd;
                    dr[0] = dx[0] * ir; dr[1] = dx[1] * ir; dr[2] = dx[2] * ir;
                    irij = ir;
                }
                rij = rijd; q2i = q2id; q2j = q2jd; hj1 = hj1d;
            } else {
                if (!(r2f < 4.0f * hm * hm)) return;
                const float ir = rsqrt_ftz(fmaxf(r2f, 1e-37f));
                const float rr = r2f * ir;
                irf = ir;
                if (rr <= 1e-30f) {
                    if (a.S.itype[j] == typei && typei != 2) raise_err(a.red, NDSPH_E_CLUMP, a.S.id[i]);
                    dr[0] = dr[1] = dr[2] = 0;
                } else {
                    dr[0] = dxf[0] * ir; dr[1] = dxf[1] * ir; dr[2] = dxf[2] * ir;
                }
                rij = rr;
                hj1 = rcp(xsj.w);
                q2i = r2f * (hi1 * hi1);
                q2j = r2f * (hj1 * hj1);
            }
            // without dust every type pair matches and no drag applies
            const int typej = pre ? tpre : ((PREC == NDSPH_PREC_FP64 || o.idust != 0) ? a.S.itype[j] : typei);
            PData<R> pj;
            if constexpr (PREC == NDSPH_PREC_FP32) {
                if (pre) {
                    pj.vx = pre[1].x; pj.vy = pre[1].y; pj.vz = pre[1].z; pj.m = pre[1].w;
                    pj.rho = pre[2].x; pj.pr = pre[2].y; pj.cs = pre[2].z; pj.u = pre[2].w;
                    pj.Bx = pre[3].x; pj.By = pre[3].y; pj.Bz = pre[3].z; pj.gradh = pre[3].w;
                    pj.a0 = pre[4].x; pj.a1 = pre[4].y; pj.a2 = pre[4].z; pj.h = pre[4].w;
                } else {
                    load_p<PREC>(a, j, pj);
                }
            } else {
                load_p<PREC>(a, j, pj);
            }
            const R mj = pj.m;
            const R vj[3] = {pj.vx, pj.vy, pj.vz};
            const R dvel[3] = {vi[0] - vj[0], vi[1] - vj[1], vi[2] - vj[2]};
            const R rhoj = pj.rho;
            if (type_match(typei, typej)) {
                // ---------------- rates_core ----------------
                // mw: the mass factor of every hydro/MHD term below; the
                // FP32 form has m_j in the kernel gradients already
                const R mw = (PREC == NDSPH_PREC_FP64) ? mj : (R)1;
                R gwi, gwj;
                if constexpr (PREC == NDSPH_PREC_FP64) {
                    gwi = tab_val(a.t.gw, tab_index(a.t, q2i));
                    gwj = tab_val(a.t.gw, tab_index(a.t, q2j));
                } else {
                    const float c = a.t.cnormf;
                    if (q2i >= KERN_Q2_DIRECT) {
                        const float qi = rij * hi1;
                        const float t = fmaxf(2.0f - qi, 0.0f), u = fmaxf(1.0f - qi, 0.0f);
                        gwi = c * (3.0f * u * u - 0.75f * t * t);
                    } else {
                        gwi = tab_valf(a.t.gwf, tab_indexf(a.t, q2i));
                    }
                    if (q2j >= KERN_Q2_DIRECT) {
                        const float qj = rij * hj1;
                        const float t = fmaxf(2.0f - qj, 0.0f), u = fmaxf(1.0f - qj, 0.0f);
                        gwj = c * (3.0f * u * u - 0.75f * t * t);
                    } else {
                        gwj = tab_valf(a.t.gwf, tab_indexf(a.t, q2j));
                    }
                }
                R grkerni, grkernj;
                if constexpr (PREC == NDSPH_PREC_FP64) {
                    R hfacgrkj = hj1 * hj1;
                    if (NDIM >= 2) hfacgrkj *= hj1;
                    if (NDIM >= 3) hfacgrkj *= hj1;
                    grkerni = gwi * hfacgrki * gradhi;
                    grkernj = gwj * hfacgrkj * pj.gradh;
                } else {
                    // m_j times the two kernel gradients (pj.gradh is the
                    // pack's m gradh h^-(ndim+1))
                    grkerni = (gwi * hgi) * mj;
                    grkernj = gwj * pj.gradh;
                }
                const R grkern = (R)0.5 * (grkerni + grkernj);
                const R dvdotr = dvel[0] * dr[0] + dvel[1] * dr[1] + dvel[2] * dr[2];
                const R rho1j = (PREC == NDSPH_PREC_FP64) ? (R)F.f[RHO1][j] : rcp(rhoj);
                const R rho21j = rho1j * rho1j;
                const R rhoav1 = (R)0.5 * (rho1i + rho1j);
                const R prj = pj.pr;
                const R Prho2j = prj * rho21j;
                const R csj = pj.cs;
                R vsigi, vsigj, vsigB;
                R dB[3] = {0, 0, 0}, Brhoj[3] = {0, 0, 0};
                R projBrhoi = 0, projBrhoj = 0, projdB = 0, Brho2j = 0;
                if (mhd) {
                    const R Bj[3] = {pj.Bx, pj.By, pj.Bz};
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        Brhoj[c] = Bj[c] * rho1j;
                        dB[c] = Bi[c] - Bj[c];
                    }
                    const R projBi = Bi[0] * dr[0] + Bi[1] * dr[1] + Bi[2] * dr[2];
                    const R projBj = Bj[0] * dr[0] + Bj[1] * dr[1] + Bj[2] * dr[2];
                    projdB = dB[0] * dr[0] + dB[1] * dr[1] + dB[2] * dr[2];
                    projBrhoi = projBi * rho1i;
                    projBrhoj = projBj * rho1j;
                    const R B2j = Bj[0] * Bj[0] + Bj[1] * Bj[1] + Bj[2] * Bj[2];
                    const R va2j = B2j * rho1j;
                    Brho2j = B2j * rho21j;
                    const R vsig2j = csj * csj + va2j;
                    const R ti = csi * projBi, tj = csj * projBj;
                    const R vpi = vsig2i * vsig2i - (R)4 * (ti * ti) * rho1i;
                    const R vpj = vsig2j * vsig2j - (R)4 * (tj * tj) * rho1j;
                    if (vpi < (R)0 || vpj < (R)0) raise_err(a.red, NDSPH_E_VSIG_DET, a.S.id[i]);
                    vsigi = sqrtp((R)0.5 * (vsig2i + sqrtp(fmax(vpi, (R)0))));
                    vsigj = sqrtp((R)0.5 * (vsig2j + sqrtp(fmax(vpj, (R)0))));
                    vsigB = sqrtp(dvel[0] * dvel[0] + dvel[1] * dvel[1] + dvel[2] * dvel[2]);
                } else {
                    vsigi = csi; vsigj = csj; vsigB = 0;
                }
                R vsig = (R)0.5 * fmax(vsigi + vsigj - beta * dvdotr, (R)0);
                R vsigu = sqrtp(fabs(pri - prj) * rhoav1);
                R vsigdtc = fmax(vsig, (R)0.5 * (vsigi + vsigj + beta * fabs(dvdotr)));
                vsigdtc = fmax(vsigdtc, vsigB);
                const R hmin = fmin(hi, pj.h);
                if (i_dust) {
                    vsig = 0; vsigu = 0;
                } else {
                    vsmax = fmax(vsmax, vsigdtc);
                    if (vsigdtc > (R)1.e-10) {
                        if (PREC == NDSPH_PREC_FP64) {
                            if (hmin * dtc_v < dtc_h * vsigdtc) { dtc_h = hmin; dtc_v = vsigdtc; }
                        } else {
                            dtc = fmin(dtc, divp(hmin, vsigdtc));
                        }
                    }
                }
                R fxi = 0, fyi = 0, fzi = 0;
                // FP32 form: the pair's induction terms (resistivity and the
                // dB/dt term), added to the compensated sums once
                R dbp[3] = {0, 0, 0};
                const bool resist = o.imhd > 0 && o.imhd != 10 && o.iav >= 2;
                const bool induct = o.imhd == 1 || o.imhd == 11;
                // ---------------- artificial_dissipation ----------------
                if (o.iav > 0) {
                    const R alphaav = (R)0.5 * (alphai + pj.a0);
                    const R alphau = (R)0.5 * (alphaui + pj.a1);
                    const R alphaB = (R)0.5 * (alphaBi + pj.a2);
                    const R vsigav = fmax(fmax(alphaav, alphau), alphaB) * vsig;
                    R term, termu, termB;
                    if constexpr (PREC == NDSPH_PREC_FP64) {
                        term = vsig * rhoav1 * grkern;
                        termu = vsigu * rhoav1 * grkern;
                        termB = vsigB * rhoav1 * grkern;
                    } else {
                        const R rg = rhoav1 * grkern;
                        term = vsig * rg;
                        termu = vsigu * rg;
                        termB = vsigB * rg;
                    }
                    if (dvdotr < (R)0 && o.iav <= 3) {
                        const R visc = alphaav * term * (-dvdotr);
                        fxi -= mw * visc * dr[0]; fyi -= mw * visc * dr[1]; fzi -= mw * visc * dr[2];
                    }
                    if (resist) {
                        const R fb = rhoi * mw * alphaB * termB * rhoav1;
                        if constexpr (PREC == NDSPH_PREC_FP64) {
                            dbx.add(fb * dB[0]); dby.add(fb * dB[1]); dbz.add(fb * dB[2]);
                        } else {
                            dbp[0] = fb * dB[0]; dbp[1] = fb * dB[1]; dbp[2] = fb * dB[2];
                        }
                    }
                    if (o.iener > 0 && o.iener != 3) {
                        R vissv = 0;
                        if (dvdotr < (R)0 && o.iav <= 3) {
                            // v_i.r - v_j.r as the reference forms it; the
                            // FP32 form takes the pair's dv.r (the same
                            // quantity, one rounding instead of a difference
                            // of two dot products)
                            R tt;
                            if constexpr (PREC == NDSPH_PREC_FP64)
                                tt = (vi[0] * dr[0] + vi[1] * dr[1] + vi[2] * dr[2]) -
                                     (vj[0] * dr[0] + vj[1] * dr[1] + vj[2] * dr[2]);
                            else
                                tt = dvdotr;
                            vissv = -alphaav * (R)0.5 * (tt * tt);
                        }
                        const R vissu = (o.iener == 1) ? (R)0 : alphau * (ui - pj.u);
                        R vissB = 0;
                        if (o.imhd > 0 && o.imhd != 10 && o.iav >= 2)
                            vissB = -alphaB * (R)0.5 * (dB[0] * dB[0] + dB[1] * dB[1] + dB[2] * dB[2]) * rhoav1;
                        du.add(mw * (term * vissv + termu * vissu + termB * vissB));
                    }
                    if (vsigav > (R)1.e-10) {
                        if (PREC == NDSPH_PREC_FP64) {
                            if (hmin * dtav_v < dtav_h * vsigav) { dtav_h = hmin; dtav_v = vsigav; }
                        } else {
                            dtav = fmin(dtav, divp(hmin, vsigav));
                        }
                    }
                }
                // ---------------- pressure ----------------
                const R prterm = Prho2i * grkerni + Prho2j * grkernj;
                fxi -= mw * prterm * dr[0]; fyi -= mw * prterm * dr[1]; fzi -= mw * prterm * dr[2];
                // ---------------- mhd_terms ----------------
                if (mhd) {
                    const R fiso = (R)0.5 * (Brho2i * grkerni + Brho2j * grkernj);
                    if constexpr (PREC == NDSPH_PREC_FP64) {
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            const R fan = (Brhoi[c] * projBrhoi - stressmax * dr[c] * rho21i) * grkerni +
                                          (Brhoj[c] * projBrhoj - stressmax * dr[c] * rho21j) * grkernj;
                            const R fm = mw * (fan - fiso * dr[c]);
                            if (c == 0) fxi += fm; else if (c == 1) fyi += fm; else fzi += fm;
                        }
                    } else {
                        // the same terms regrouped: B_i/rho_i (B_i.r/rho_i) grkerni
                        // + B_j (B_j.r/rho_j)/rho_j grkernj - (stressmax (grkerni/rho_i^2
                        // + grkernj/rho_j^2) + fiso) r
                        const R pbi = projBrhoi * grkerni;
                        const R pbj = projBrhoj * rho1j * grkernj;
                        const R st = stressmax * (rho21i * grkerni + rho21j * grkernj) + fiso;
                        fxi += Brhoi[0] * pbi + pj.Bx * pbj - st * dr[0];
                        fyi += Brhoi[1] * pbi + pj.By * pbj - st * dr[1];
                        fzi += Brhoi[2] * pbi + pj.Bz * pbj - st * dr[2];
                    }
                    dvb.add(-mw * projdB * grkern);
                    if (o.imhd > 0) {
                        const R c0 = dB[1] * dr[2] - dB[2] * dr[1];
                        const R c1 = dB[2] * dr[0] - dB[0] * dr[2];
                        const R c2 = dB[0] * dr[1] - dB[1] * dr[0];
                        cbx.add(mw * c0 * grkern); cby.add(mw * c1 * grkern); cbz.add(mw * c2 * grkern);
                    }
                    if (induct) {
                        const R fb = mw * projBrhoi * grkerni;
                        if constexpr (PREC == NDSPH_PREC_FP64) {
                            dbx.add(-fb * dvel[0]); dby.add(-fb * dvel[1]); dbz.add(-fb * dvel[2]);
                        } else {
                            dbp[0] -= fb * dvel[0]; dbp[1] -= fb * dvel[1]; dbp[2] -= fb * dvel[2];
                        }
                    }
                }
                fx.add(fxi); fy.add(fyi); fz.add(fzi);
                if constexpr (PREC == NDSPH_PREC_FP32) {
                    if ((resist && o.iav > 0) || induct) { dbx.add(dbp[0]); dby.add(dbp[1]); dbz.add(dbp[2]); }
                }
                if (o.iav > 0) {
                    if (o.iavlim[1] > 0) {
                        const R graduterm = (ui - pj.u) * ((PREC == NDSPH_PREC_FP64) ? (R)irij : (R)irf);
                        d2u.add(mw * rho1j * graduterm * grkerni);
                    }
                    if (o.iavlim[0] != 3) {
                        gx.add(mw * (dvel[0] - dvdotr) * grkerni);
                        gy.add(mw * (dvel[1] - dvdotr) * grkerni);
                        gz.add(mw * (dvel[2] - dvdotr) * grkerni);
                    }
                }
            } else if (o.idust == 2 && o.idrag_nature > 0) {
                // ---------------- drag_forces ----------------
                const R dv2 = dvel[0] * dvel[0] + dvel[1] * dvel[1] + dvel[2] * dvel[2];
                R drd[3];
                if (rij <= (R)2.220446049250313e-16) {
                    if (dv2 <= (R)2.220446049250313e-16) return;
                    const R ivij = rcp(sqrtp(dv2));
                    drd[0] = dvel[0] * ivij; drd[1] = dvel[1] * ivij; drd[2] = dvel[2] * ivij;
                } else {
                    drd[0] = dr[0]; drd[1] = dr[1]; drd[2] = dr[2];
                }
                const R rsum = rhoi + rhoj;
                // the simulation's drag constant (per simulation in a batch)
                const R Kdrag = (R)(o.sim_aux ? bitsd(o.sim_aux[(size_t)a.S.sim[i] * SIMAUX + SA_KDRAG]) : o.Kdrag);
                const R ts = divp(rhoj * rhoi, Kdrag * rsum);
                R wgas, csg;
                if (typei == NDSPH_ITYPE_GAS || typei == NDSPH_ITYPE_BND) {
                    R wdi;
                    if constexpr (PREC == 0) wdi = tab_val(a.t.wdrag, tab_index(a.t, q2i));
                    else wdi = tab_valf(a.t.wdragf, tab_indexf(a.t, q2i));
                    R hfw = hi1;
                    if (NDIM >= 2) hfw *= hi1;
                    if (NDIM >= 3) hfw *= hi1;
                    wgas = wdi * hfw;
                    csg = csi;
                    hcsts = fmax(hcsts, divp(hi, csg * ts));
                } else {
                    if (typej != NDSPH_ITYPE_GAS && typej != NDSPH_ITYPE_BND) return;
                    R wdj;
                    if constexpr (PREC == 0) wdj = tab_val(a.t.wdrag, tab_index(a.t, q2j));
                    else wdj = tab_valf(a.t.wdragf, tab_indexf(a.t, q2j));
                    R hfw = hj1;
                    if (NDIM >= 2) hfw *= hj1;
                    if (NDIM >= 3) hfw *= hj1;
                    wgas = wdj * hfw;
                    csg = pj.cs;
                    hcsts = fmax(hcsts, divp(pj.h, csg * ts));
                }
                tsmin = fmin(tsmin, ts);
                const R projv = dvel[0] * drd[0] + dvel[1] * drd[1] + dvel[2] * drd[2];
                const R dragterm = divp((R)NDIM * wgas, rsum * ts) * projv;
                const R dragterm_en = dragterm * projv;
                fx.add(-dragterm * mj * drd[0]);
                fy.add(-dragterm * mj * drd[1]);
                fz.add(-dragterm * mj * drd[2]);
                if (typei == NDSPH_ITYPE_GAS) du.add(mj * dragterm_en);
            }
    };
    if constexpr (!Src::kRows) {
        if (live) src.for_each(i, [&](unsigned pk) { pair_terms(pk, nullptr, 0); });
    } else if constexpr (PREC == NDSPH_PREC_FP64 || NDIM < 3) {
        // the FP64 form, and short 1D/2D rows (~8 / ~25 entries, most of them
        // accepted), take one pass over the row
        const int ncand = live ? a.S.nl_cnt[i] : 0;
        const unsigned* row = a.S.nl + (size_t)i * a.nl_stride;
        for (int k = 0; k < ncand; k++) pair_terms(row[k], nullptr, 0);
    } else {
        // Two phases per chunk of the row: screen the candidates (four row
        // entries and positions in flight at a time) and keep the accepted
        // entries in shared memory, then run the pair terms over those only,
        // so the lanes of a warp do not idle on rejected candidates in the
        // long part.  The accepted pairs, their order and the screen
        // arithmetic are those of a single pass over the row.
        constexpr int RATES_CHUNK = rates_chunk<NDIM>();
        __shared__ unsigned acc_buf[RATES_CHUNK * RATES_BS];
        unsigned* mine = acc_buf + threadIdx.x;
        const bool typed = (o.idust != 0);
        // drag_only: a row of the other type's entries, whose pair terms are
        // the drag terms alone (they read no B, gradh or alpha of the
        // neighbour, and its h is the position's h)
        auto sweep_row = [&](const unsigned* row, const int ncand, auto drag_only) {
            int k = 0;   // a multiple of 4 whenever a vector row load is issued
            while (k < ncand) {
                int na = 0;
                while (na + 4 <= RATES_CHUNK && k < ncand) {
                    unsigned pq[4];
                    int m = 4;
                    if (k + 4 <= ncand) {
                        const uint4 r4 = *reinterpret_cast<const uint4*>(row + k);
                        pq[0] = r4.x; pq[1] = r4.y; pq[2] = r4.z; pq[3] = r4.w;
                    } else {
                        m = ncand - k;
#pragma unroll
                        for (int u = 0; u < 4; u++) pq[u] = (u < m) ? row[k + u] : ((unsigned)i << shift);
                    }
                    float4 xq[4];
#pragma unroll
                    for (int u = 0; u < 4; u++) xq[u] = a.S.xs[pq[u] >> shift];
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        int d[3], w[3];
                        stn.offset(pq[u] & omask, g, d, w);
                        float dxf[3];
                        const float r2f = screen_r2<NDIM>(xsi, xq[u], d, g, dxf);
                        const float hm = fmaxf(hif, xq[u].w);
                        if ((int)(pq[u] >> shift) != i && r2f < 4.0f * hm * hm) {
                            mine[na * RATES_BS] = pq[u];
                            na++;
                        }
                    }
                    k += m;
                }
                // the accepted entries: each one's four packs are loaded
                // together at the start of its pair, one round trip to L1/L2
                // (loaded inside the pair terms, the packs waited for the
                // position's screen: 2.83 -> 2.64 ms at 128^3), and its
                // position one pair ahead (4 registers), so the screen, the
                // separation and the kernel gradients start without waiting
                // and overlap the packs' loads (2.39 -> 2.33 ms).  Loading
                // all of the next entry's data ahead needs 20 more registers
                // and spilled (3.14 ms).
                unsigned pk_next = (na > 0) ? mine[0] : 0u;
                float4 x_next = (na > 0) ? a.S.xs[pk_next >> shift] : make_float4(0.f, 0.f, 0.f, 0.f);
                for (int q = 0; q < na; q++) {
                    const unsigned pk = pk_next;
                    const int j = (int)(pk >> shift);
                    float4 cur[5];
                    cur[0] = x_next;
                    if (q + 1 < na) {
                        pk_next = mine[(q + 1) * RATES_BS];
                        x_next = a.S.xs[pk_next >> shift];
                    }
                    cur[1] = a.S.pk_v[j];
                    cur[2] = a.S.pk_t[j];
                    if constexpr (decltype(drag_only)::value) {
                        cur[3] = make_float4(0.f, 0.f, 0.f, 0.f);
                        cur[4] = make_float4(0.f, 0.f, 0.f, cur[0].w);
                    } else {
                        cur[3] = a.S.pk_b[j];
                        cur[4] = a.S.pk_a[j];
                    }
                    pair_terms(pk, cur, typed ? a.S.itype[j] : typei);
                }
            }
        };
        sweep_row(a.S.nl + (size_t)i * a.nl_stride, live ? a.S.nl_cnt[i] : 0, std::false_type{});
        // two particle types (gas and dust: TYPED, rows split by type): the
        // rows of the other type, the drag pairs, follow as a second run, so
        // the lanes of a warp take one branch of the pair terms at a time
        // instead of alternating between the hydro/MHD terms and the drag
        // terms pair by pair
        if constexpr (TYPED)
            sweep_row(a.S.nl2 + (size_t)i * a.nl_stride, live ? a.S.nl_cnt2[i] : 0, std::true_type{});
    }

    if (PREC == NDSPH_PREC_FP64) {
        dtc = dtc_h / dtc_v;
        dtav = dtav_h / dtav_v;
    }

    // ---- per-particle post pass ratesND_mhd.f90:532-965 (in the pair
    // precision R: FP64 for the parity form, FP32 for the FP32 form) ----
    const R hi_p = (PREC == 0) ? (R)F.f[HH][i] : hi;
    const R rho1 = (PREC == 0) ? (R)(1.0 / F.f[RHO][i]) : rho1i;
    R force[3] = {accv<R>(fx), accv<R>(fy), accv<R>(fz)};
    R dBe[3] = {accv<R>(dbx), accv<R>(dby), accv<R>(dbz)};
    R dudt = accv<R>(du);
    R divB = accv<R>(dvb);
    R curlB[3] = {accv<R>(cbx), accv<R>(cby), accv<R>(cbz)};
    const R del2u = accv<R>(d2u);
    const R gdv[3] = {accv<R>(gx), accv<R>(gy), accv<R>(gz)};
    if (mhd) {
        if (o.imhd > 0)
            for (int c = 0; c < 3; c++) curlB[c] *= rho1;
        divB *= rho1;
    }
    const R fmag = sqrtp(force[0] * force[0] + force[1] * force[1] + force[2] * force[2]);
    R fonh_r = divp(fmag, hi_p);
    if (typei == 1) fonh_r = 0;
    R va2 = 0;
    if (mhd) va2 = B2i * rho1i;   // B^2/dens with dens = rho
    const R vsig = sqrtp(csi * csi + va2);
    const R drhodt = (R)F.f[DRHODT][i];
    if (o.imhd >= 11 && o.imhd <= 19) {
        for (int c = 0; c < 3; c++) dBe[c] = dBe[c] + (R)F.f[BE0 + c][i] * rho1 * drhodt;
    } else if (o.imhd >= 1 && o.imhd <= 9) {
        for (int c = 0; c < 3; c++) dBe[c] = dBe[c] * rho1;
    } else {
        dBe[0] = dBe[1] = dBe[2] = 0;
    }
    R dendt;
    if (o.iener > 0 && o.iav >= 0 && o.iener != 3 && o.iener != 10 && o.iener != 11) {
        dudt = dudt + pri * (rho1 * rho1) * drhodt;
        dendt = dudt;
    } else {
        dendt = dudt;
    }
    if (typei == NDSPH_ITYPE_DUST) dendt = 0;
    R daldt[3] = {0, 0, 0};
    if (o.iavlim[0] != 0 || o.iavlim[1] != 0 || o.iavlim[2] != 0) {
        const R tdecay1 = divp((R)o.avdecayconst * vsig, hi_p);
        if (o.iavlim[0] == 1 || o.iavlim[0] == 2) {
            R source = fmax(drhodt * rho1, (R)0);
            if (o.iavlim[0] == 2) source = source * ((R)2 - alphai);
            daldt[0] = ((R)o.alphamin - alphai) * tdecay1 + (R)o.avfact * source;
        }
        if (o.iener > 0 && o.iavlim[1] > 0) {
            R sourceu = 0;
            if (ui > (R)2.220446049250313e-16) sourceu = divp(hi_p * fabs(del2u), sqrtp(ui));
            daldt[1] = ((R)o.alphaumin - alphaui) * tdecay1 + sourceu;
        }
    }
    R drhodt_out = drhodt;
    bool zero_dh = false;
    if (typei == NDSPH_ITYPE_BND || typei == NDSPH_ITYPE_BNDDUST) {
        for (int c = 0; c < 3; c++) { force[c] = 0; dBe[c] = 0; daldt[c] = 0; curlB[c] = 0; }
        drhodt_out = 0; dudt = 0; dendt = 0; divB = 0;
        zero_dh = true;
    }
    double fonh = live ? (double)fonh_r : 0.0;
    if (live) {
        for (int c = 0; c < 3; c++) {
            F.f[F0 + c][i] = force[c];
            F.f[DB0 + c][i] = dBe[c];
            F.f[DAL0 + c][i] = daldt[c];
            F.f[GDV0 + c][i] = gdv[c];
            if (o.imhd > 0) F.f[CB0 + c][i] = curlB[c];
        }
        if (zero_dh) { F.f[DRHODT][i] = 0.0; F.f[DHDT][i] = 0.0; }
        else if (PREC != 0) { /* drhodt unchanged */ }
        if (PREC == 0) F.f[DRHODT][i] = drhodt_out;
        F.f[DUDT][i] = dudt;
        F.f[DENDT][i] = dendt;
        F.f[DIVB][i] = divB;
        F.f[DEL2U][i] = del2u;
        if (a.tail_on) step_tail_one(F, o, a.red->dt, i, (size_t)a.S.id[i], a.S, a.tail);
    }

    // ---- global reductions ----
    if (PREC != 0 && !o.batched) {
        // FP32 form, one simulation: block reductions on the FP32 bit
        // patterns of the non-negative values (ordered as integers), then one
        // conversion to FP64 per block and quantity -- the same doubles as
        // converting every value first
        (void)hcsts;
        const float fh = live ? (float)fonh_r : 0.f;
        const unsigned long long b_dtc = block_min_bits(__float_as_uint(fmaxf((float)dtc, 0.f)));
        const unsigned long long b_dtav = block_min_bits(__float_as_uint(fmaxf((float)dtav, 0.f)));
        const unsigned long long b_vs = block_max_bits(__float_as_uint(fmaxf((float)vsmax, 0.f)));
        const unsigned long long b_ts = block_min_bits(__float_as_uint(fmaxf((float)tsmin, 0.f)));
        const unsigned long long b_fh = block_max_bits(__float_as_uint(fmaxf(fh, 0.f)));
        if (threadIdx.x == 0) {
            // FP32 "no limit" (above 1e37) is the FP64 largest value
            auto up = [](unsigned long long b, bool nolimit) {
                double v = (double)__uint_as_float((unsigned)b);
                if (nolimit && v > 1e37) v = 1.7976931348623157e308;
                return dbits(v);
            };
            atomicMin(&a.red->dtcourant, up(b_dtc, false));
            atomicMin(&a.red->dtav, up(b_dtav, true));
            atomicMax(&a.red->vsigmax, up(b_vs, false));
            atomicMin(&a.red->ts_min, up(b_ts, true));
            atomicMax(&a.red->fhmax, up(b_fh, false));
        }
        return;
    }
    // (warp first, then one atomic per warp or block)
    double rdtc = (double)dtc, rdtav = (double)dtav, rvs = (double)vsmax, rts = (double)tsmin;
    if (PREC != 0) {
        if (rdtav > 1e37) rdtav = 1.7976931348623157e308;
        if (rts > 1e37) rts = 1.7976931348623157e308;
    }
    if (o.batched) {
        // per-simulation reductions: one atomic per warp when the whole warp
        // belongs to one simulation (the usual case: tubes are contiguous)
        const int si = live ? a.S.sim[i] : -1;
        const int s0 = __shfl_sync(0xffffffffu, si, 0);
        const bool uniform = __all_sync(0xffffffffu, si == s0 || si < 0);
        if (uniform) {
            for (int off = 16; off > 0; off >>= 1) {
                rdtc = fmin(rdtc, __shfl_down_sync(0xffffffffu, rdtc, off));
                rdtav = fmin(rdtav, __shfl_down_sync(0xffffffffu, rdtav, off));
                rvs = fmax(rvs, __shfl_down_sync(0xffffffffu, rvs, off));
                rts = fmin(rts, __shfl_down_sync(0xffffffffu, rts, off));
                fonh = fmax(fonh, __shfl_down_sync(0xffffffffu, fonh, off));
            }
        }
        if ((uniform && (threadIdx.x & 31) == 0 && s0 >= 0) || (!uniform && live)) {
            unsigned long long* r = o.sim_red + (size_t)(uniform ? s0 : si) * SIMRED;
            atomic_min_pos(&r[SR_DTC], rdtc);
            atomic_min_pos(&r[SR_DTAV], rdtav);
            atomic_max_pos(&r[SR_VSIG], rvs);
            atomic_min_pos(&r[SR_TS], rts);
            atomic_max_pos(&r[SR_FH], fonh);
        }
        return;
    }
    // block-wide reductions on the bit patterns of the non-negative values,
    // one atomic per block and quantity
    (void)hcsts;
    const unsigned long long b_dtc = block_min_bits(dbits(fmax(rdtc, 0.0)));
    const unsigned long long b_dtav = block_min_bits(dbits(fmax(rdtav, 0.0)));
    const unsigned long long b_vs = block_max_bits(dbits(fmax(rvs, 0.0)));
    const unsigned long long b_ts = block_min_bits(dbits(fmax(rts, 0.0)));
    const unsigned long long b_fh = block_max_bits(dbits(fmax(fonh, 0.0)));
    if (threadIdx.x == 0) {
        atomicMin(&a.red->dtcourant, b_dtc);
        atomicMin(&a.red->dtav, b_dtav);
        atomicMax(&a.red->vsigmax, b_vs);
        atomicMin(&a.red->ts_min, b_ts);
        atomicMax(&a.red->fhmax, b_fh);
    }
}

// FP32 packs (FP32 form): velocities + masses before the density passes,
// everything the rates sweep reads after the EOS
__device__ __forceinline__ void pack_v_one(const SweepArgs& a, int k)
{
    const FieldPtrs& F = a.F;
    a.S.pk_v[k] = make_float4((float)F.f[V0][k], (float)F.f[V1][k], (float)F.f[V2][k], (float)F.f[PM][k]);
}
// The fourth word of pk_b is m gradh h^-(ndim+1): the factor that turns the
// kernel's dW/dq at q_j into particle j's mass-weighted grad-h gradient.
// Every hydro/MHD pair term carries m_j times one of the kernel gradients,
// so the FP32 sweep folds m_j in once per pair instead of once per term
// (~20 fewer multiplies a pair: 2.57 -> 2.52 ms for the 128^3 sweep).
__device__ __forceinline__ void pack_rates_one(const SweepArgs& a, int k)
{
    const FieldPtrs& F = a.F;
    const float m = (float)F.f[PM][k], hf = (float)F.f[HH][k];
    const float h1 = rcp_ftz(hf);
    float hfac = h1 * h1;
    if (a.o.ndim >= 2) hfac *= h1;
    if (a.o.ndim >= 3) hfac *= h1;
    a.S.pk_v[k] = make_float4((float)F.f[V0][k], (float)F.f[V1][k], (float)F.f[V2][k], m);
    a.S.pk_t[k] = make_float4((float)F.f[RHO][k], (float)fmax(F.f[PR][k], 0.0), (float)F.f[CS][k], (float)F.f[UU][k]);
    a.S.pk_b[k] = make_float4((float)F.f[BF0][k], (float)F.f[BF1][k], (float)F.f[BF2][k],
                              (m * (float)F.f[GRADH][k]) * hfac);
    a.S.pk_a[k] = make_float4((float)F.f[AL0][k], (float)F.f[AL1][k], (float)F.f[AL2][k], hf);
}
__global__ void k_pack_v(SweepArgs a)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < a.n) pack_v_one(a, k);
}
__global__ void k_pack_rates(SweepArgs a)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < a.n) pack_rates_one(a, k);
}
void launch_pack_v(const SweepArgs& a, cudaStream_t st)
{
    if (a.n > 0) NDSPH_COUNT_LAUNCH, k_pack_v<<<nblk(a.n, 256), 256, 0, st>>>(a);
}
void launch_pack_rates(const SweepArgs& a, cudaStream_t st)
{
    if (a.n > 0) NDSPH_COUNT_LAUNCH, k_pack_rates<<<nblk(a.n, 256), 256, 0, st>>>(a);
}

template <int NDIM, int PREC, bool TYPED = false>
__global__ void __launch_bounds__(RATES_BS, PREC == 0 ? 2 : NDSPH_RATES_FP32_MINB) k_rates(SweepArgs a)
{
    // no early return: every lane of the warp takes part in the final
    // shuffle reductions; lanes past n run an empty stencil on slot 0
    const int ithread = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = ithread < (a.plist ? a.pn : a.n);
    const int i = live ? (a.plist ? a.plist[a.pi0 + ithread] : ithread) : 0;
    rates_body<NDIM, PREC, RowSrc, TYPED>(a, i, live, RowSrc{});
}

void launch_rates(const SweepArgs& a, cudaStream_t st)
{
    const int bs = RATES_BS;
    const int np = a.plist ? a.pn : a.n;
    if (np <= 0) return;
    const int nb = nblk(np, bs);
    if (a.o.precision == NDSPH_PREC_FP64) {
        if (a.o.ndim == 1) NDSPH_COUNT_LAUNCH, k_rates<1, 0><<<nb, bs, 0, st>>>(a);
        else if (a.o.ndim == 2) NDSPH_COUNT_LAUNCH, k_rates<2, 0><<<nb, bs, 0, st>>>(a);
        else NDSPH_COUNT_LAUNCH, k_rates<3, 0><<<nb, bs, 0, st>>>(a);
    } else {
        if (a.o.ndim == 1) NDSPH_COUNT_LAUNCH, k_rates<1, 1><<<nb, bs, 0, st>>>(a);
        else if (a.o.ndim == 2) NDSPH_COUNT_LAUNCH, k_rates<2, 1><<<nb, bs, 0, st>>>(a);
        else if (a.typed_rows) NDSPH_COUNT_LAUNCH, k_rates<3, 1, true><<<nb, bs, 0, st>>>(a);
        else NDSPH_COUNT_LAUNCH, k_rates<3, 1><<<nb, bs, 0, st>>>(a);
    }
}



// ===========================================================================
// Fused step of a batch of 1D simulations (the tubes of a parameter sweep):
// one block per tube runs the whole leapfrog step of its tube -- predictor,
// order by x, every Newton-Raphson density pass, EOS, rates, the tube's dt
// and the corrector -- in one launch for all tubes, with no global sort,
// permutation gather or neighbour rows (stepND_leapfrog_mhd.f90:31-275 with
// derivs.f90:27-287 per tube, as the reference runs one tube per process,
// multi/multirun.f90).  The particles stay in their slots; each tube keeps
// an order by x in shared memory, and a particle's candidates are the run of
// that order within 2 max(h_i, h_j) of it: scanning away from it stops at the
// first particle farther than twice the largest h of every particle beyond
// (prefix / suffix maxima of h), so no pair is missed.  The candidates reach
// the density and rates sweeps' own per-particle bodies packed as neighbour-
// row entries, over cells of the tube's own grid (8 cells to 2 hmax), so the
// pair arithmetic and the Newton-Raphson semantics are the sweeps'.
// ===========================================================================
constexpr int TUBE_BS = 128;

// candidates of slot i of a tube in x order (see above)
struct TubeWin {
    static constexpr bool kRows = false;
    const float* X;      // [m] x - (tube's smallest x), in x order
    const float* H;      // [m] h rounded up, in x order
    const float* PMX;    // [m] prefix max of H
    const float* SMX;    // [m] suffix max of H
    const int* idx;      // [m] x order -> slot
    const int* pos;      // [m] slot - t0 -> x order
    const int* cell;     // cell of each slot (tube grid)
    const int* id;
    Reduce* red;
    int t0, m;
    template <class Fn>
    __device__ __forceinline__ void for_each(int i, Fn&& f) const
    {
        const int k = pos[i - t0];
        const int ci = cell[i];
        const float xk = X[k], hk = H[k];
        auto emit = [&](int j) {
            const int d = cell[j] - ci;
            // the tube grid puts every candidate within 8 cells (checked)
            if (d < -8 || d > 8) {
                raise_err(red, NDSPH_E_CELLS, id[i]);
                return;
            }
            f(((unsigned)j << 5) | (unsigned)(d + 8));
        };
        // in increasing x, the order the cell-sorted rows give (sums in a
        // shock tube are sensitive to their order: the cell path, the
        // reference and this one then round alike)
        int q0 = k;
        while (q0 > 0 && xk - X[q0 - 1] < 2.0f * fmaxf(hk, PMX[q0 - 1]) * 1.001f + 2e-6f) q0--;
        for (int q = q0; q < k; q++) emit(idx[q]);
        emit(i);
        for (int q = k + 1; q < m; q++) {
            if (X[q] - xk >= 2.0f * fmaxf(hk, SMX[q]) * 1.001f + 2e-6f) break;
            emit(idx[q]);
        }
    }
};

struct TubeShared {
    double cs;       // cell size of the tube grid in use (0: none yet)
    int ncalc, bad;
};

// block-wide max / min of one double per thread
__device__ __forceinline__ double tube_block_max(double v, double* scratch)
{
    for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) scratch[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = scratch[0];
    for (int w = 1; w < TUBE_BS / 32; w++) r = fmax(r, scratch[w]);
    __syncthreads();
    return r;
}
__device__ __forceinline__ double tube_block_min(double v, double* scratch)
{
    return -tube_block_max(-v, scratch);
}

// inclusive running max of a[0..m) from the front (dir = +1) or the back
// (dir = -1) into out: each thread scans a contiguous chunk, the chunk
// maxima are combined, then applied
__device__ __forceinline__ void tube_running_max(const float* a, float* out, int m, int dir, float* part)
{
    const int per = (m + TUBE_BS - 1) / TUBE_BS;
    const int c0 = threadIdx.x * per, c1 = min(c0 + per, m);
    float run = 0.f;
    for (int q = c0; q < c1; q++) {
        const int k = (dir > 0) ? q : (m - 1 - q);
        run = fmaxf(run, a[k]);
        out[k] = run;
    }
    part[threadIdx.x] = run;
    __syncthreads();
    float before = 0.f;
    for (int t = 0; t < (int)threadIdx.x; t++) before = fmaxf(before, part[t]);
    for (int q = c0; q < c1; q++) {
        const int k = (dir > 0) ? q : (m - 1 - q);
        out[k] = fmaxf(out[k], before);
    }
    __syncthreads();
}

struct TubeArgs {
    SweepArgs a;
    const int* tube_start;   // [nsim + 1] first slot of each tube (tubes are contiguous)
    const int* order;        // [nsim] tubes, largest first
    double* dt_next;         // [nsim] the next step's dt of each tube
    double* sim_out;         // [nsim * 4] dtcourant, dtforce, dt next, time
    // several steps in one call: the previous launch's corrector also ran
    // this step's save and predictor (predicted), and this launch's corrector
    // runs the next step's (predict_next) -- each particle's corrected state
    // goes straight into the next save and predictor, one pass over its
    // fields instead of two
    int predicted, predict_next;
};

template <int PREC>
__global__ void __launch_bounds__(TUBE_BS) k_tube_step(TubeArgs T)
{
    extern __shared__ __align__(16) unsigned char tube_smem[];
    __shared__ TubeShared sh;
    __shared__ double red_scratch[TUBE_BS / 32];
    __shared__ float part[TUBE_BS];
    // the sweeps' arguments with this tube's grid, pass number and active
    // list: one copy per block in shared memory, changed by thread 0 between
    // barriers
    __shared__ __align__(16) unsigned char a_raw[sizeof(SweepArgs)];
    SweepArgs& a = *reinterpret_cast<SweepArgs*>(a_raw);
    const int s = T.order[blockIdx.x];
    const int t0 = T.tube_start[s], m = T.tube_start[s + 1] - t0;
    const int tid = threadIdx.x;
    if (tid == 0) a = T.a;
    __syncthreads();
    const FieldPtrs& F = T.a.F;
    const Side& S = T.a.S;
    const DevOpts& o = T.a.o;
    float* X = reinterpret_cast<float*>(tube_smem);
    float* H = X + m;
    float* PMX = H + m;
    float* SMX = PMX + m;
    int* idx = reinterpret_cast<int*>(SMX + m);
    int* pos = idx + m;
    const double dt = o.sim_dt[s];

    // ---- reductions of this tube start afresh; predictor
    if (tid == 0) {
        unsigned long long* r = o.sim_red + (size_t)s * SIMRED;
        r[SR_DTC] = dbits(1.e6);
        r[SR_DTAV] = dbits(1.7976931348623157e308);
        r[SR_VSIG] = 0ull;
        r[SR_TS] = dbits(1.7976931348623157e308);
        r[SR_FH] = 0ull;
        r[SR_STRESS] = 0ull;
        sh.bad = 0;
    }
    if (!T.predicted) {
        for (int k = tid; k < m; k += TUBE_BS) predictor_one(F, S, o, dt, t0 + k, 0);
        __syncthreads();
        if (o.has_fixed) {
            for (int k = tid; k < m; k += TUBE_BS) predictor_fixed_x_one(F, S, o, dt, t0 + k);
            __syncthreads();
        }
    } else {
        __syncthreads();
    }

    // ---- x order of the tube (a particle seldom passes another: checked,
    // and ranked afresh when one has)
    double xmin = 1.7976931348623157e308;
    int bad = 0, unsorted = 0;
    for (int k = tid; k < m; k += TUBE_BS) {
        const double x = F.f[X0][t0 + k];
        if (!isfinite(x)) bad = 1;
        xmin = fmin(xmin, x);
        if (k + 1 < m && F.f[X0][t0 + k + 1] < x) unsorted = 1;
    }
    if (__syncthreads_or(bad)) {
        if (tid == 0) raise_err(a.red, NDSPH_E_NAN, S.id[t0]);
        return;
    }
    xmin = tube_block_min(xmin, red_scratch);
    if (__syncthreads_or(unsorted)) {
        for (int k = tid; k < m; k += TUBE_BS) {
            const double xk = F.f[X0][t0 + k];
            int r = 0;
            for (int q = 0; q < m; q++) {
                const double xq = F.f[X0][t0 + q];
                r += (xq < xk) || (xq == xk && q < k);
            }
            idx[r] = t0 + k;
        }
    } else {
        for (int k = tid; k < m; k += TUBE_BS) idx[k] = t0 + k;
    }
    __syncthreads();
    for (int k = tid; k < m; k += TUBE_BS) {
        pos[idx[k] - t0] = k;
        X[k] = (float)(F.f[X0][idx[k]] - xmin);
    }
    __syncthreads();

    // ---- per pass: the tube grid and the window bounds from the current h
    TubeWin win;
    win.X = X; win.H = H; win.PMX = PMX; win.SMX = SMX; win.idx = idx; win.pos = pos;
    win.cell = S.cell; win.id = S.id; win.red = a.red; win.t0 = t0; win.m = m;
    // The cells (8 to 2 hmax with the window's margins) are set once a step
    // with 10 % room for h to grow and set again only when some h outgrows
    // them; 1/h and the FP32 h follow every pass.
    if (tid == 0) sh.cs = 0.0;
    auto prep = [&]() -> bool {
        float hmf = 0.f;
        for (int k = tid; k < m; k += TUBE_BS) {
            const float h = (float)F.f[HH][idx[k]] * 1.000001f;
            H[k] = h;
            hmf = fmaxf(hmf, h);
        }
        const double hm = tube_block_max((double)hmf, red_scratch);
        if (!(hm > 0.0) || !isfinite(hm)) return false;
        const bool regrid = (2.0 * hm * 1.002 + 4e-6) > 7.5 * sh.cs;
        if (regrid) {
            const double cs = (2.0 * hm * 1.1 + 4e-6) / 7.5;
            const double origin = xmin - cs;
            const double inv_cs = 1.0 / cs;
            for (int k = tid; k < m; k += TUBE_BS) {
                const int i = t0 + k;
                const double x = F.f[X0][i];
                const int c = (int)floor((x - origin) * inv_cs);
                S.cell[i] = c;
                S.xs[i] = make_float4((float)(x - (origin + (double)c * cs)), 0.f, 0.f, 0.f);
            }
            __syncthreads();
            if (tid == 0) {
                sh.cs = cs;
                a.g.nc[0] = 1 << 30; a.g.nc[1] = 1; a.g.nc[2] = 1;
                a.g.ncells = 1 << 30;
                a.g.origin[0] = origin; a.g.cs[0] = cs; a.g.inv_cs[0] = inv_cs; a.g.csf[0] = (float)cs;
                a.g.sw = 17;
                a.g.nlshift = 5;
            }
        }
        for (int k = tid; k < m; k += TUBE_BS) {
            const int i = t0 + k;
            const double h = F.f[HH][i];
            S.xs[i].w = (float)h;
            S.h1[i] = 1.0 / h;
        }
        tube_running_max(H, PMX, m, +1, part);
        tube_running_max(H, SMX, m, -1, part);
        return true;
    };

    // ---- iterate_density (iterate_density.f90:43-360) over the tube
    for (int k = tid; k < m; k += TUBE_BS) {
        density_init_one(F, S, t0 + k, a.red);
        if (PREC == NDSPH_PREC_FP32) pack_v_one(a, t0 + k);
    }
    if (tid == 0) {
        a.d_its = nullptr;
        a.d_nlist = nullptr;
        a.ncalc_next = &sh.ncalc;
    }
    __syncthreads();
    int* act = S.active + t0;
    int* act_next = S.active_next + t0;
    int its = 0, ncalc = m;
    while (ncalc > 0 && its <= o.maxdensits) {
        its++;
        const bool full = (ncalc == m);
        if (full && its > 1) {
            for (int k = tid; k < m; k += TUBE_BS) F.f[HNEXT][t0 + k] = F.f[HH][t0 + k];
        }
        if (!prep()) {
            if (tid == 0) raise_err(a.red, NDSPH_E_H_NONPOS, S.id[t0]);
            return;
        }
        if (tid == 0) {
            sh.ncalc = 0;
            a.its = its;
            a.S.active_next = act_next;
        }
        __syncthreads();
        if (full) {
            for (int k = tid; k < m; k += TUBE_BS) density_body<1, true, PREC>(a, idx[k], win);
        } else {
            for (int k = tid; k < ncalc; k += TUBE_BS) density_body<1, false, PREC>(a, act[k], win);
        }
        __syncthreads();
        if (full)
            for (int k = tid; k < m; k += TUBE_BS) F.f[HH][t0 + k] = F.f[HNEXT][t0 + k];
        __syncthreads();
        if (o.has_fixed) {
            for (int k = tid; k < m; k += TUBE_BS) fixed_density_copy_one(F, S, t0 + k);
            __syncthreads();
        }
        ncalc = sh.ncalc;
        int* tmp = act; act = act_next; act_next = tmp;
        __syncthreads();
    }
    if (its > o.maxdensits && o.maxdensits > 0) {
        if (tid == 0) raise_err(a.red, NDSPH_E_NOT_CONVERGED, S.id[t0]);
        return;
    }

    // ---- conservative2primitive + EOS, fixed-particle copies
    double st = 0.0;
    for (int k = tid; k < m; k += TUBE_BS) st = fmax(st, eos_one(F, S, o, t0 + k, a.red));
    st = tube_block_max(st, red_scratch);
    if (tid == 0 && st > 0.0) o.sim_red[(size_t)s * SIMRED + SR_STRESS] = dbits(st);
    if (o.has_fixed) {
        for (int k = tid; k < m; k += TUBE_BS) fixed_copy_one(F, S, t0 + k);
        __syncthreads();
    }
    if (PREC == NDSPH_PREC_FP32) {
        for (int k = tid; k < m; k += TUBE_BS) pack_rates_one(a, t0 + k);
    }
    __syncthreads();

    // ---- get_rates over the tube (every lane of each warp takes part)
    if (!prep()) {
        if (tid == 0) raise_err(a.red, NDSPH_E_H_NONPOS, S.id[t0]);
        return;
    }
    __syncthreads();
    for (int k0 = 0; k0 < m; k0 += TUBE_BS) {
        const int k = k0 + tid;
        const bool live = k < m;
        rates_body<1, PREC>(a, live ? idx[k] : idx[0], live, win);
    }
    __syncthreads();

    // ---- the tube's next dt (stepND_leapfrog_mhd.f90:252) and its clock
    if (tid == 0) {
        const unsigned long long* r = o.sim_red + (size_t)s * SIMRED;
        const double dtcourant = bitsd(r[SR_DTC]);
        const double fhmax = bitsd(r[SR_FH]);
        double dtforce = 1.7976931348623157e308;
        if (fhmax > 0.0) dtforce = fmin(dtforce, sqrt(1.0 / fhmax));
        double dtdrag = 1.7976931348623157e308;
        const double kdrag = o.sim_aux ? bitsd(o.sim_aux[(size_t)s * SIMAUX + SA_KDRAG]) : o.Kdrag;
        if (o.idust == 2 && o.idrag_nature != 0 && (kdrag > 0.0 || o.idrag_nature > 1))
            dtdrag = fmin(dtdrag, bitsd(r[SR_TS]));
        double dtn = o.C_force * dtforce;
        dtn = fmin(dtn, o.C_cour * dtcourant);
        dtn = fmin(dtn, 0.9 * dtdrag);
        dtn = fmin(dtn, o.C_force * 1.7976931348623157e308);
        T.dt_next[s] = dtn;
        T.sim_out[s * 4 + 0] = dtcourant;
        T.sim_out[s * 4 + 1] = dtforce;
        T.sim_out[s * 4 + 2] = dtn;
        T.sim_out[s * 4 + 3] += dt;
    }
    // ---- corrector (and with predict_next the next step's save and
    // predictor, with the dt just set)
    if (T.predict_next) {
        __syncthreads();
        const double dtn = T.dt_next[s];
        for (int k = tid; k < m; k += TUBE_BS) {
            corrector_one(F, S, o, dt, t0 + k, a.red);
            predictor_one(F, S, o, dtn, t0 + k, 0);
        }
        __syncthreads();
        if (o.has_fixed) {
            for (int k = tid; k < m; k += TUBE_BS) predictor_fixed_x_one(F, S, o, dtn, t0 + k);
            __syncthreads();
        }
    } else {
        for (int k = tid; k < m; k += TUBE_BS) corrector_one(F, S, o, dt, t0 + k, a.red);
        __syncthreads();
    }
    if (tid == 0) o.sim_dt[s] = T.dt_next[s];
}

size_t tube_smem_bytes(int maxm) { return (size_t)maxm * (4 * sizeof(float) + 2 * sizeof(int)); }

void launch_tube_step(const SweepArgs& a, const int* tube_start, const int* order, int nsim, double* dt_next,
                      double* sim_out, int maxm, bool predicted, bool predict_next, cudaStream_t st)
{
    TubeArgs T;
    T.a = a;
    T.tube_start = tube_start;
    T.order = order;
    T.dt_next = dt_next;
    T.sim_out = sim_out;
    T.predicted = predicted ? 1 : 0;
    T.predict_next = predict_next ? 1 : 0;
    const size_t smem = tube_smem_bytes(maxm);
    // (128 registers a thread: 4 blocks, 16 warps per SM; forcing 5 blocks
    // spilled and was 8 % slower)
    if (a.o.precision == NDSPH_PREC_FP64) {
        cudaFuncSetAttribute(k_tube_step<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        NDSPH_COUNT_LAUNCH, k_tube_step<0><<<nsim, TUBE_BS, smem, st>>>(T);
    } else {
        cudaFuncSetAttribute(k_tube_step<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        NDSPH_COUNT_LAUNCH, k_tube_step<1><<<nsim, TUBE_BS, smem, st>>>(T);
    }
}

// ===========================================================================
// neighbour lists: every candidate j (self included) of slot i with
// |x_i - x_j| < 2 max(h_i, h_j) skin (+ FP32 margin) inside the search
// stencil (sw^NDIM cells around i's cell).  The sweeps then test only these;
// a list is rebuilt when some h grows past its slack (NR epilogue flag) and
// on every link.
// ===========================================================================
// distance from a cell-relative coordinate x to the slab of cells at offset
// dc, [dc cs, (dc+1) cs)
__device__ __forceinline__ float slab_dist(float x, int dc, float cs)
{
    const float lo = (float)dc * cs;
    return fmaxf(fmaxf(lo - x, x - (lo + cs)), 0.0f);
}

// the rows a build writes for one slot: its own row and count, and with
// TYPED (two particle types) the row and count of the other type's entries
struct RowOut {
    unsigned* row;
    int cnt;
    unsigned* row2;
    int cnt2;
    int typei;
};
template <bool TYPED>
__device__ __forceinline__ void row_put(const SweepArgs& a, RowOut& out, int tj, unsigned e)
{
    if (TYPED && !type_match(out.typei, tj)) {
        if (out.cnt2 < a.nl_stride) out.row2[out.cnt2] = e;
        out.cnt2++;
    } else {
        if (out.cnt < a.nl_stride) out.row[out.cnt] = e;
        out.cnt++;
    }
}

// candidates of slot i in the slot range [jb, je) of a run of x-adjacent
// cells starting at x offset dx0: the x offset of j's cell steps up at each
// of the run's inner cell starts b[0..3] (je where the run is shorter); the
// stencil index is obase + dx + r.  Loads are issued four at a time so that
// their latencies overlap.
template <int NDIM, bool TYPED = false>
__device__ __forceinline__ void nl_scan_run(const SweepArgs& a, const float4& xsi, float hi, float sk,
                                            float abs_tol, int jb, int je, const int b[4], int dx0, float oy,
                                            float oz, unsigned obase, RowOut& out)
{
    const Grid& g = a.g;
    const unsigned shift = (NDIM == 3) ? (unsigned)g.nlshift : 5u;
    const int r = (NDIM == 2) ? 1 : (g.sw - 1) >> 1;
    for (int j0 = jb; j0 < je; j0 += 4) {
        float4 q[4];
        int tq[4] = {0, 0, 0, 0};
#pragma unroll
        for (int u = 0; u < 4; u++) {
            q[u] = (j0 + u < je) ? a.S.xs[j0 + u] : make_float4(0.f, 0.f, 0.f, 0.f);
            if (TYPED) tq[u] = (j0 + u < je) ? a.S.itype[j0 + u] : 0;
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int j = j0 + u;
            if (j >= je) break;
            const int dx = dx0 + (j >= b[0]) + (j >= b[1]) + (j >= b[2]) + (j >= b[3]);
            float r2 = (xsi.x - q[u].x) - (float)dx * g.csf[0];
            r2 = r2 * r2;
            if (NDIM >= 2) { const float t = (xsi.y - q[u].y) - oy; r2 += t * t; }
            if (NDIM >= 3) { const float t = (xsi.z - q[u].z) - oz; r2 += t * t; }
            const float rc = sk * fmaxf(hi, q[u].w) + abs_tol;
            if (r2 > rc * rc) continue;
            row_put<TYPED>(a, out, tq[u], ((unsigned)j << shift) | (obase + (unsigned)(dx + r)));
        }
    }
}

// the same scan on positions relative to the grid origin (3D, one
// simulation): the separation is a plain difference (ox: the periodic image
// shift of the run's cells), and the x cell offset is counted only for the
// entries written
template <bool TYPED = false>
__device__ __forceinline__ void nl_scan_run_g(const SweepArgs& a, const float4& xgi, float hi, float sk,
                                              float abs_tol, int jb, int je, const int b[4], int dx0, float ox,
                                              float oy, float oz, unsigned obase, RowOut& out)
{
    const unsigned shift = (unsigned)a.g.nlshift;
    const int r = (a.g.sw - 1) >> 1;
    const float xi = xgi.x - ox, yi = xgi.y - oy, zi = xgi.z - oz;
    for (int j0 = jb; j0 < je; j0 += 4) {
        float4 q[4];
        int tq[4] = {0, 0, 0, 0};
#pragma unroll
        for (int u = 0; u < 4; u++) {
            q[u] = (j0 + u < je) ? a.S.xg[j0 + u] : make_float4(0.f, 0.f, 0.f, 0.f);
            if (TYPED) tq[u] = (j0 + u < je) ? a.S.itype[j0 + u] : 0;
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int j = j0 + u;
            if (j >= je) break;
            const float tx = xi - q[u].x, ty = yi - q[u].y, tz = zi - q[u].z;
            const float r2 = tx * tx + ty * ty + tz * tz;
            const float rc = sk * fmaxf(hi, q[u].w) + abs_tol;
            if (r2 > rc * rc) continue;
            const int dx = dx0 + (j >= b[0]) + (j >= b[1]) + (j >= b[2]) + (j >= b[3]);
            row_put<TYPED>(a, out, tq[u], ((unsigned)j << shift) | (obase + (unsigned)(dx + r)));
        }
    }
}

// origin-relative FP32 positions for the 3D row build: the slot's cell
// corner plus its cell-relative position (after a kept link the slot may
// have left that cell; the sum is still its position, unwrapped)
__global__ void k_xg(Side S, Grid g, int n)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int cc[3];
    cell_coords(S.cell[k], g, cc);
    const float4 x = S.xs[k];
    S.xg[k] = make_float4((float)cc[0] * g.csf[0] + x.x, (float)cc[1] * g.csf[1] + x.y,
                          (float)cc[2] * g.csf[2] + x.z, x.w);
}

// One thread per particle.  For each (dy, dz) row of the stencil, the cells
// whose box lies within the stencil's reach of the particle (r cells: every
// pair a sweep may need is within it) form a run of x-adjacent cells, one
// slot range unless it wraps or leaves an open box; rows and cells beyond
// the reach are skipped.
template <int NDIM, bool XG = false, bool TYPED = false>
__global__ void __launch_bounds__(128) k_build_nlist(SweepArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    if (a.gate && *a.gate == 0) return;
    const Grid& g = a.g;
    const float4 xsi = a.S.xs[i];
    const float4 xgi = XG ? a.S.xg[i] : xsi;
    const float hi = xsi.w;
    const float csmin = fminf(g.csf[0], fminf(NDIM >= 2 ? g.csf[1] : g.csf[0], NDIM >= 3 ? g.csf[2] : g.csf[0]));
    const float abs_tol = 1e-6f * fmaxf(g.csf[0], fmaxf(g.csf[1], g.csf[2]));
    const float sk = 2.0f * a.nl_skin * 1.0002f;
    const int sw = (NDIM == 2) ? 3 : g.sw, r = (sw - 1) >> 1;
    const float reach = (float)r * csmin * 1.001f + abs_tol;
    const float reach2 = reach * reach;
    Stencil<NDIM> stn(a.S.cell[i], g);
    RowOut out;
    out.row = a.S.nl + (size_t)i * a.nl_stride;
    out.cnt = 0;
    out.row2 = TYPED ? a.S.nl2 + (size_t)i * a.nl_stride : nullptr;
    out.cnt2 = 0;
    out.typei = TYPED ? a.S.itype[i] : 0;
    if (NDIM == 1) {
        // 1D: cells of 2 hmax / r in a run of 2r + 1; a cell is searched only
        // within 2 skin max(h_i, largest h of the cell) of the particle, so a
        // particle of small h in a dense region (a dense tube of a batch,
        // whose cells are sized by the sparsest) scans only the cells next to it
        const int bnone[4] = {0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff};
        for (int dx = -r; dx <= r; dx++) {
            const float ex = slab_dist(xsi.x, dx, g.csf[0]);
            if (ex > reach) continue;
            int d[3] = {dx, 0, 0}, w[3], cid;
            if (!stn.cell_at_d(d, g, a.o, cid, w)) continue;
            if (ex > sk * fmaxf(hi, a.cell_h[cid]) + abs_tol) continue;
            nl_scan_run<NDIM>(a, xsi, hi, sk, abs_tol, a.cell_start[cid], a.cell_start[cid + 1], bnone, dx, 0.f, 0.f,
                              0u, out);
        }
    }
    const int zlo = (NDIM >= 3) ? -r : 0, ylo = (NDIM >= 2) ? -r : 0;
    for (int dz = zlo; dz <= -zlo && NDIM >= 2; dz++) {
        const float ez = (NDIM >= 3) ? slab_dist(xsi.z, dz, g.csf[2]) : 0.f;
        for (int dy = ylo; dy <= -ylo; dy++) {
            const float ey = (NDIM >= 2) ? slab_dist(xsi.y, dy, g.csf[1]) : 0.f;
            const float e2 = ey * ey + ez * ez;
            if (e2 > reach2) continue;
            // x cells whose box is within the reach
            const float ax = sqrtf(reach2 - e2) + abs_tol;
            const int dx0 = max(-r, (int)floorf((xsi.x - ax) / g.csf[0]));
            const int dx1 = min(r, (int)floorf((xsi.x + ax) / g.csf[0]));
            if (dx0 > dx1) continue;
            unsigned obase = 0;
            if (NDIM >= 2) obase += (unsigned)((dy + r) * sw);
            if (NDIM >= 3) obase += (unsigned)((dz + r) * sw * sw);
            const float oy = (NDIM >= 2) ? (float)dy * g.csf[1] : 0.f;
            const float oz = (NDIM >= 3) ? (float)dz * g.csf[2] : 0.f;
            int d[3] = {dx0, dy, dz}, w[3];
            int c0, c1;
            const bool ok0 = stn.cell_at_d(d, g, a.o, c0, w);
            d[0] = dx1;
            const bool ok1 = stn.cell_at_d(d, g, a.o, c1, w);
            // origin-relative positions: the periodic image shifts of the
            // row (the same for every cell of it in y and z)
            const float gy = XG ? (float)w[1] * (float)a.o.L[1] : 0.f;
            const float gz = XG ? (float)w[2] * (float)a.o.L[2] : 0.f;
            if (ok0 && ok1 && c1 - c0 == dx1 - dx0) {
                // consecutive cells: one slot range
                int b[4];
#pragma unroll
                for (int k = 0; k < 4; k++) b[k] = (k < dx1 - dx0) ? a.cell_start[c0 + k + 1] : 0x7fffffff;
                if (XG)
                    nl_scan_run_g<TYPED>(a, xgi, hi, sk, abs_tol, a.cell_start[c0], a.cell_start[c1 + 1], b, dx0,
                                         (float)w[0] * (float)a.o.L[0], gy, gz, obase, out);
                else
                    nl_scan_run<NDIM, TYPED>(a, xsi, hi, sk, abs_tol, a.cell_start[c0], a.cell_start[c1 + 1], b,
                                             dx0, oy, oz, obase, out);
            } else {
                const int bnone[4] = {0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff};
                for (int dx = dx0; dx <= dx1; dx++) {
                    d[0] = dx;
                    int cid;
                    if (!stn.cell_at_d(d, g, a.o, cid, w)) continue;
                    if (XG)
                        nl_scan_run_g<TYPED>(a, xgi, hi, sk, abs_tol, a.cell_start[cid], a.cell_start[cid + 1],
                                             bnone, dx, (float)w[0] * (float)a.o.L[0], gy, gz, obase, out);
                    else
                        nl_scan_run<NDIM, TYPED>(a, xsi, hi, sk, abs_tol, a.cell_start[cid], a.cell_start[cid + 1],
                                                 bnone, dx, oy, oz, obase, out);
                }
            }
        }
    }
    a.S.nl_cnt[i] = out.cnt < a.nl_stride ? out.cnt : a.nl_stride;
    if (TYPED) a.S.nl_cnt2[i] = out.cnt2 < a.nl_stride ? out.cnt2 : a.nl_stride;
    a.S.hb[i] = hi;
    if (a.S.xsb) a.S.xsb[i] = xsi;
    const int cmax = max(out.cnt, out.cnt2);
    if (cmax > a.nl_stride) { a.red->nl_overflow = 1; if (a.graph) a.red->gfail |= 2; }
    // the longest row: one atomic per warp (one per particle put 2.1 M
    // atomics on one word at 128^3)
    const unsigned am = __activemask();
    const int wmax = __reduce_max_sync(am, cmax);
    if ((int)(threadIdx.x & 31u) == __ffs((int)am) - 1) atomicMax(&a.red->nl_maxcnt, wmax);
}

// largest h (the xs.w the build uses) of each cell's particles (1D pruning)
__global__ void k_cell_hmax(const int* __restrict__ start, const float4* __restrict__ xs, float* cell_h,
                            int ncells)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    float m = 0.f;
    for (int k = start[c]; k < start[c + 1]; k++) m = fmaxf(m, xs[k].w);
    cell_h[c] = m;
}

void launch_build_nlist(const SweepArgs& a, cudaStream_t st)
{
    if (a.n <= 0) return;
    if (a.o.ndim == 1)
        NDSPH_COUNT_LAUNCH, k_cell_hmax<<<nblk(a.g.ncells, 256), 256, 0, st>>>(a.cell_start, a.S.xs, a.cell_h,
                                                                            a.g.ncells);
    const int nbp = nblk(a.n, 128);
    if (a.o.ndim == 1) NDSPH_COUNT_LAUNCH, k_build_nlist<1><<<nbp, 128, 0, st>>>(a);
    else if (a.o.ndim == 2) NDSPH_COUNT_LAUNCH, k_build_nlist<2><<<nbp, 128, 0, st>>>(a);
    else if ((!a.o.batched || a.o.stacked) && a.g.nc[0] <= 1024 && a.g.nc[1] <= 1024 && a.g.nc[2] <= 1024) {
        // 3D simulations of at most 1024 cells a side: the scan runs on
        // FP32 positions relative to the grid origin, which carry an error of
        // at most ~6e-8 x 1024 cells, well inside the rows' 2e-4 radius margin
        NDSPH_COUNT_LAUNCH, k_xg<<<nbp, 128, 0, st>>>(a.S, a.g, a.n);
        if (a.typed_rows) NDSPH_COUNT_LAUNCH, k_build_nlist<3, true, true><<<nbp, 128, 0, st>>>(a);
        else NDSPH_COUNT_LAUNCH, k_build_nlist<3, true><<<nbp, 128, 0, st>>>(a);
    } else if (a.typed_rows) NDSPH_COUNT_LAUNCH, k_build_nlist<3, false, true><<<nbp, 128, 0, st>>>(a);
    else NDSPH_COUNT_LAUNCH, k_build_nlist<3><<<nbp, 128, 0, st>>>(a);
}

// ===========================================================================
// neighbour CSR for the parity tests (check_neighbourlist.f90 replacement).
// mode 0: q_i<2; mode 1: q_i<2 or q_j<2 with q2 = rij2*(h1*h1); type filter
// as density; self excluded; indices are original (0-based) ids.
// ===========================================================================
template <int NDIM>
__global__ void k_neigh(SweepArgs a, int mode, const long long* offsets, long long* counts, int* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const FieldPtrs& F = a.F;
    double xi[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < NDIM; d++) xi[d] = F.f[X0 + d][i];
    const double hi1 = a.S.h1[i];
    const double hi21 = __dmul_rn(hi1, hi1);
    const int typei = a.S.itype[i];
    const double dxbound = 2.0 * ghost_hmax(a, i);
    Stencil<NDIM> stn(a.S.cell[i], a.g);
    const int sw = a.g.sw, r = (sw - 1) >> 1;
    const int nst = (NDIM == 1) ? sw : (NDIM == 2 ? sw * sw : sw * sw * sw);
    long long k = offsets ? offsets[a.S.id[i]] : 0;
    long long cnt = 0;
    for (int so = 0; so < nst; so++) {
        int cid, d[3], w[3];
        d[0] = so % sw - r;
        d[1] = (NDIM >= 2) ? (so / sw) % sw - r : 0;
        d[2] = (NDIM >= 3) ? so / (sw * sw) - r : 0;
        if (!stn.cell_at_d(d, a.g, a.o, cid, w)) continue;
        for (int j = a.cell_start[cid]; j < a.cell_start[cid + 1]; j++) {
            if (j == i) continue;
            if (!type_match(typei, a.S.itype[j])) continue;
            double dx[3], rij2;
            if (!exact_dx<NDIM>(F, j, xi, w, a.o, dxbound, dx, rij2)) continue;
            const double q2i = __dmul_rn(rij2, hi21);
            const double hj1 = a.S.h1[j];
            const double q2j = __dmul_rn(rij2, __dmul_rn(hj1, hj1));
            const bool ok = (mode == 0) ? (q2i < 4.0) : (q2i < 4.0 || q2j < 4.0);
            if (!ok) continue;
            if (out) out[k++] = a.S.id[j];
            cnt++;
        }
    }
    if (counts) counts[a.S.id[i]] = cnt;
}

void launch_neigh_count(const SweepArgs& a, int mode, long long* counts, cudaStream_t st)
{
    const int nb = nblk(a.n, 128);
    if (a.o.ndim == 1) NDSPH_COUNT_LAUNCH, k_neigh<1><<<nb, 128, 0, st>>>(a, mode, nullptr, counts, nullptr);
    else if (a.o.ndim == 2) NDSPH_COUNT_LAUNCH, k_neigh<2><<<nb, 128, 0, st>>>(a, mode, nullptr, counts, nullptr);
    else NDSPH_COUNT_LAUNCH, k_neigh<3><<<nb, 128, 0, st>>>(a, mode, nullptr, counts, nullptr);
}
void launch_neigh_fill(const SweepArgs& a, int mode, const long long* offsets, int* out, cudaStream_t st)
{
    const int nb = nblk(a.n, 128);
    if (a.o.ndim == 1) NDSPH_COUNT_LAUNCH, k_neigh<1><<<nb, 128, 0, st>>>(a, mode, offsets, nullptr, out);
    else if (a.o.ndim == 2) NDSPH_COUNT_LAUNCH, k_neigh<2><<<nb, 128, 0, st>>>(a, mode, offsets, nullptr, out);
    else NDSPH_COUNT_LAUNCH, k_neigh<3><<<nb, 128, 0, st>>>(a, mode, offsets, nullptr, out);
}

}  // namespace ndsph
