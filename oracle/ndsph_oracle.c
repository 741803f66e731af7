/*
 * ndsph_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement (plain C, FP64, single thread) of the NDSPMHD per-step hot
 * path, used as the parity oracle by tests/, by __graft_entry__.smoke() and
 * as the timed CPU baseline of bench.py.  It is never linked into, loaded by
 * or called from the product library (ndspmhd_gb300/csrc).
 *
 * It follows the reference's own data structures on purpose: explicit ghost
 * particles for periodic boundaries (ghostND_mhd.f90), the head/next cell link
 * list (linkND.f90), the half-stencil symmetric pair loops (density_sums.f90,
 * ratesND_mhd.f90) and the partial full-stencil gather (density_partial), so
 * that it reproduces the reference's pair decisions and iteration semantics
 * literally.  Each routine cites the reference file:line it restates.
 *
 * Parity status: the reference cannot be built in this project's containers
 * (no Fortran compiler; SPLASH modules missing), so this restatement is pinned
 * by analytic invariants (kernel normalisation, lattice density, pairwise
 * momentum conservation, brute-force neighbour sets) -- see tests/.
 *
 * Build: oracle/Makefile (-O2 -ffp-contract=off so x86 and aarch64 give the
 * same bits).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

#include "../include/ndsph.h"

#define IKERN 4000
#define MAXNDIM 3

/* ------------------------------------------------------------------------- */
/* kernel tables: kernelND.f90:34-58, setkerntable :127-157,                  */
/* cubic spline (default case) :4143-4192, normalisation :4279-4289,          */
/* double-hump drag kernel 41 :1659-1697                                      */
/* ------------------------------------------------------------------------- */
typedef struct {
    double wij[IKERN + 1], grwij[IKERN + 1], grgrwij[IKERN + 1];
    double wijdrag[IKERN + 1], grwijdrag[IKERN + 1], grgrwijdrag[IKERN + 1];
    double dq2table, ddq2table, radkern, radkern2;
} orc_kernels;

static double powi_f(double x, int n)
{
    /* gfortran expands x**n for small integer n as repeated products */
    switch (n) {
    case 1: return x;
    case 2: return x * x;
    case 3: return (x * x) * x;
    default: { double r = 1.0; for (int i = 0; i < n; i++) r *= x; return r; }
    }
}

static void orc_setkern_tables(orc_kernels* K, int ndim)
{
    const double pi = 3.141592653589;           /* kernelND.f90:39 (truncated) */
    K->radkern = 2.0;
    K->radkern2 = K->radkern * K->radkern;
    K->dq2table = K->radkern * K->radkern / (double)IKERN;
    double cnormk = 0.0;
    switch (ndim) {
    case 1: cnormk = 0.66666666666; break;
    case 2: cnormk = 10. / (7. * pi); break;
    case 3: cnormk = 1. / pi; break;
    }
    for (int i = 0; i <= IKERN; i++) {
        double q2 = i * K->dq2table;
        double q = sqrt(q2);
        double w, g, gg;
        if (q < 1.0) {
            w = 1. - 1.5 * q2 + 0.75 * q * q2;
            g = -3. * q + 2.25 * q2;
            gg = -3. + 4.5 * q;
        } else if (q >= 1.0 && q <= 2.0) {
            double t = 2. - q;
            w = 0.25 * powi_f(t, 3);
            g = -0.75 * powi_f(t, 2);
            gg = 1.5 * t;
        } else {
            w = 0.0; g = 0.0; gg = 0.0;
        }
        K->wij[i] = cnormk * w;
        K->grwij[i] = cnormk * g;
        K->grgrwij[i] = cnormk * gg;
    }
    /* drag kernel 41 (double hump M4, Fulk & Quinn 1996) */
    double cd = 0.0;
    switch (ndim) {
    case 1: cd = 2.0; break;
    case 2: cd = 70. / (31. * pi); break;
    case 3: cd = 10. / (9. * pi); break;
    }
    for (int i = 0; i <= IKERN; i++) {
        double q2 = i * K->dq2table;
        double q = sqrt(q2);
        double q4 = q2 * q2;
        double w, g, gg;
        if (q < 1.0) {
            w = q2 - 1.5 * q4 + 0.75 * q4 * q;
            g = 2. * q - 6. * q2 * q + 3.75 * q4;
            gg = 2. - 18. * q2 + 15. * q2 * q;
        } else if (q >= 1.0 && q <= 2.0) {
            double t = 2. - q;
            w = 0.25 * q2 * powi_f(t, 3);
            g = 0.5 * q * powi_f(t, 3) - 0.75 * q2 * powi_f(t, 2);
            gg = 0.5 * powi_f(t, 3) - 3. * q * powi_f(t, 2) + 1.5 * q2 * t;
        } else {
            w = 0.0; g = 0.0; gg = 0.0;
        }
        K->wijdrag[i] = cd * w;
        K->grwijdrag[i] = cd * g;
        K->grgrwijdrag[i] = cd * gg;
    }
    K->ddq2table = 1. / K->dq2table;
}

/* index/slope logic shared by every interpolate_* (kernelND.f90:4367-4393) */
static inline void kidx(const orc_kernels* K, double q2, int* index, int* index1, double* dxx)
{
    int idx = (int)(q2 * K->ddq2table);
    int idx1 = idx + 1;
    if (idx > IKERN || idx < 0) idx = IKERN;
    if (idx1 > IKERN || idx1 < 0) idx1 = IKERN;
    *index = idx;
    *index1 = idx1;
    *dxx = q2 - idx * K->dq2table;
}

static inline double klerp(const orc_kernels* K, const double* t, int i0, int i1, double dxx)
{
    double slope = (t[i1] - t[i0]) * K->ddq2table;
    return t[i0] + slope * dxx;
}

/* interpolate_kernels_dens kernelND.f90:4599-4638 (walt/gradwalt tables equal
 * wij/grwij because ikernelalt = ikernel, initialiseND_mhd.f90:180-187)       */
static inline void interp_dens(const orc_kernels* K, double q2, double* w, double* gw,
                               double* ggw, double* walt, double* gwalt)
{
    int i0, i1; double dxx;
    kidx(K, q2, &i0, &i1, &dxx);
    *w = klerp(K, K->wij, i0, i1, dxx);
    *gw = klerp(K, K->grwij, i0, i1, dxx);
    *ggw = klerp(K, K->grgrwij, i0, i1, dxx);
    *walt = klerp(K, K->wij, i0, i1, dxx);
    *gwalt = klerp(K, K->grwij, i0, i1, dxx);
}

/* interpolate_kernels kernelND.f90:4426-4469 */
static inline void interp_rates(const orc_kernels* K, double q2, double* w, double* gw,
                                double* gwalt, double* ggwalt)
{
    int i0, i1; double dxx;
    kidx(K, q2, &i0, &i1, &dxx);
    *w = klerp(K, K->wij, i0, i1, dxx);
    *gw = klerp(K, K->grwij, i0, i1, dxx);
    *gwalt = klerp(K, K->grwij, i0, i1, dxx);
    *ggwalt = klerp(K, K->grgrwij, i0, i1, dxx);
}

/* interpolate_kerneldrag kernelND.f90:4398-4421 */
static inline double interp_drag(const orc_kernels* K, double q2)
{
    int i0, i1; double dxx;
    kidx(K, q2, &i0, &i1, &dxx);
    return klerp(K, K->wijdrag, i0, i1, dxx);
}

/* ------------------------------------------------------------------------- */
/* simulation state: the part/rates/hterms/linklist/bound modules             */
/* (variablesND.f90:44-217) with room for ghosts                             */
/* ------------------------------------------------------------------------- */
typedef struct {
    ndsph_opts o;
    orc_kernels K;
    int ndim, npart, ntotal, cap;
    double avfact;
    /* part */
    double *x, *vel, *Bevol, *Bfield, *en, *uu, *hh, *pmass, *rho, *rhoalt, *dens, *pr,
        *spsound, *alpha, *psi;
    int *itype, *ireal;
    /* hterms / rates */
    double *gradh, *gradhn, *gradsoft, *gradgradh, *drhodt, *dhdt;
    double *force, *dBevoldt, *dudt, *dendt, *daldt, *divB, *curlB, *del2u, *graddivv;
    /* linklist */
    int *ll, *iamincell, *numneigh, *ifirstincell;
    int ncells, ncellsx[MAXNDIM];
    double dxcell;
    /* bound / timestep */
    double hhmax;
    double dtcourant, dtforce, dtav, dtdrag, dtvisc, vsigmax, stressmax;
    double dt, time;
    int nsteps, itsdensity, ncalctotal, nrelink;
    /* step save arrays (part_in) */
    double *xin, *velin, *Bevolin, *hhin, *enin, *alphain;
    double *forcein, *dBevoldtin, *dhdtin, *dendtin, *daldtin;
    /* scratch */
    int *listneigh;
    int err;
    char msg[256];
} orc_sim;

#define NCALLOC(ptr, n) do { (ptr) = calloc((size_t)(n), sizeof(*(ptr))); } while (0)

static void sim_alloc(orc_sim* s, int cap)
{
    int nd = s->ndim;
    /* grow all per-particle arrays to cap, keeping contents */
#define GROW(ptr, stride) do { void* p_ = realloc((ptr), (size_t)cap * (stride) * sizeof(*(ptr))); \
        if (cap > s->cap) memset((char*)p_ + (size_t)s->cap * (stride) * sizeof(*(ptr)), 0, \
                                 (size_t)(cap - s->cap) * (stride) * sizeof(*(ptr))); (ptr) = p_; } while (0)
    GROW(s->x, nd); GROW(s->vel, 3); GROW(s->Bevol, 3); GROW(s->Bfield, 3);
    GROW(s->en, 1); GROW(s->uu, 1); GROW(s->hh, 1); GROW(s->pmass, 1); GROW(s->rho, 1);
    GROW(s->rhoalt, 1); GROW(s->dens, 1); GROW(s->pr, 1); GROW(s->spsound, 1);
    GROW(s->alpha, 3); GROW(s->psi, 1); GROW(s->itype, 1); GROW(s->ireal, 1);
    GROW(s->gradh, 1); GROW(s->gradhn, 1); GROW(s->gradsoft, 1); GROW(s->gradgradh, 1);
    GROW(s->drhodt, 1); GROW(s->dhdt, 1); GROW(s->force, 3); GROW(s->dBevoldt, 3);
    GROW(s->dudt, 1); GROW(s->dendt, 1); GROW(s->daldt, 3); GROW(s->divB, 1);
    GROW(s->curlB, 3); GROW(s->del2u, 1); GROW(s->graddivv, 3);
    GROW(s->ll, 1); GROW(s->iamincell, 1); GROW(s->numneigh, 1); GROW(s->listneigh, 1);
#undef GROW
    s->cap = cap;
}

/* makeghost ghostND_mhd.f90:363-420 + copy_particle copy_particle.f90:28-80  */
static void copy_particle(orc_sim* s, int i, int j)
{
    s->pmass[i] = s->pmass[j]; s->rho[i] = s->rho[j]; s->rhoalt[i] = s->rhoalt[j];
    s->hh[i] = s->hh[j]; s->uu[i] = s->uu[j]; s->en[i] = s->en[j];
    for (int d = 0; d < 3; d++) {
        s->Bevol[i * 3 + d] = s->Bevol[j * 3 + d];
        s->Bfield[i * 3 + d] = s->Bfield[j * 3 + d];
        s->alpha[i * 3 + d] = s->alpha[j * 3 + d];
        s->force[i * 3 + d] = s->force[j * 3 + d];
        s->dBevoldt[i * 3 + d] = s->dBevoldt[j * 3 + d];
        s->daldt[i * 3 + d] = s->daldt[j * 3 + d];
        s->curlB[i * 3 + d] = s->curlB[j * 3 + d];
    }
    s->psi[i] = s->psi[j]; s->gradh[i] = s->gradh[j]; s->gradhn[i] = s->gradhn[j];
    s->gradsoft[i] = s->gradsoft[j]; s->gradgradh[i] = s->gradgradh[j];
    s->spsound[i] = s->spsound[j]; s->pr[i] = s->pr[j]; s->dens[i] = s->dens[j];
    if (s->itype[i] != NDSPH_ITYPE_BND && s->itype[i] != NDSPH_ITYPE_BNDDUST &&
        s->itype[i] != 11 && s->itype[j] == NDSPH_ITYPE_GAS)
        s->itype[i] = s->itype[j];
    s->drhodt[i] = s->drhodt[j]; s->dudt[i] = s->dudt[j]; s->dendt[i] = s->dendt[j];
    s->dhdt[i] = s->dhdt[j]; s->divB[i] = s->divB[j];
}

static void makeghost(orc_sim* s, int jpart, const double* xg, const double* vg)
{
    int ip = s->ntotal;
    if (ip >= s->cap) sim_alloc(s, s->cap + s->cap / 2 + 16);
    s->ntotal = ip + 1;
    for (int d = 0; d < s->ndim; d++) s->x[ip * s->ndim + d] = xg[d];
    s->itype[ip] = s->itype[jpart];   /* set again after the loop (:330) */
    copy_particle(s, ip, jpart);
    for (int d = 0; d < 3; d++) s->vel[ip * 3 + d] = vg[d];
    s->ireal[ip] = jpart;
}

/* set_ghost_particles ghostND_mhd.f90:33-361, periodic branches only
 * (xnew = xperbound + dxshift, :224-225; edges :250-300; corners :300-330)    */
static void set_ghost_particles(orc_sim* s)
{
    int nd = s->ndim;
    s->ntotal = s->npart;
    double hmax = s->hh[0];
    for (int i = 1; i < s->npart; i++) if (s->hh[i] > hmax) hmax = s->hh[i];
    s->hhmax = hmax;
    double dxbound[MAXNDIM];
    for (int d = 0; d < nd; d++) dxbound[d] = s->K.radkern * s->hhmax;
    int imakeghost[MAXNDIM][2];
    double xnew[MAXNDIM][2];
    memset(imakeghost, 0, sizeof imakeghost);
    for (int jpart = 0; jpart < s->npart; jpart++) {
        for (int idimen = 0; idimen < nd; idimen++) {
            if (s->o.ibound[idimen] <= 1) { imakeghost[idimen][0] = imakeghost[idimen][1] = 0; continue; }
            for (int imaxmin = 0; imaxmin < 2; imaxmin++) {
                double xpart[MAXNDIM], vpart[3];
                for (int d = 0; d < nd; d++) xpart[d] = s->x[jpart * nd + d];
                for (int d = 0; d < 3; d++) vpart[d] = s->vel[jpart * 3 + d];
                double xbound, xperbound, dx;
                if (imaxmin == 0) {           /* max */
                    xbound = s->o.xmax[idimen]; xperbound = s->o.xmin[idimen];
                    dx = s->o.xmax[idimen] - s->x[jpart * nd + idimen];
                } else {                      /* min */
                    xbound = s->o.xmin[idimen]; xperbound = s->o.xmax[idimen];
                    dx = s->x[jpart * nd + idimen] - s->o.xmin[idimen];
                }
                imakeghost[idimen][imaxmin] = (dx < dxbound[idimen]) && (dx > 0);
                if (!imakeghost[idimen][imaxmin]) continue;
                double dxshift = s->x[jpart * nd + idimen] - xbound;
                xnew[idimen][imaxmin] = xperbound + dxshift;     /* periodic */
                xpart[idimen] = xnew[idimen][imaxmin];
                makeghost(s, jpart, xpart, vpart);
                if (idimen > 0) {
                    for (int idp = 0; idp < idimen; idp++) {
                        for (int imp = 0; imp < 2; imp++) {
                            if (!imakeghost[idp][imp]) continue;
                            xpart[idp] = xnew[idp][imp];
                            makeghost(s, jpart, xpart, vpart);
                            if (idp >= 1) {
                                int idpp = idp - 1;
                                for (int impp = 0; impp < 2; impp++) {
                                    if (!imakeghost[idpp][impp]) continue;
                                    xpart[idpp] = xnew[idpp][impp];
                                    makeghost(s, jpart, xpart, vpart);
                                    xpart[idpp] = s->x[jpart * nd + idpp];
                                }
                            }
                            xpart[idp] = s->x[jpart * nd + idp];
                        }
                    }
                }
            }
        }
    }
    for (int i = s->npart; i < s->ntotal; i++) s->itype[i] = s->itype[s->ireal[i]];
}

/* set_linklist linkND.f90:45-161 */
static int set_linklist(orc_sim* s)
{
    int nd = s->ndim;
    int allle1 = 1;
    for (int d = 0; d < nd; d++) if (s->o.ibound[d] > 1) allle1 = 0;
    if (allle1) {
        double hmax = s->hh[0];
        for (int i = 1; i < s->npart; i++) if (s->hh[i] > hmax) hmax = s->hh[i];
        s->hhmax = hmax;
    }
    s->dxcell = s->K.radkern * s->hhmax;
    if (s->dxcell <= 0) { s->err = NDSPH_E_H_NONPOS; snprintf(s->msg, sizeof s->msg, "link: max h <= 0"); return s->err; }
    double xminp[MAXNDIM], xmaxp[MAXNDIM];
    for (int d = 0; d < nd; d++) {
        double mn = s->x[d], mx = s->x[d];
        for (int i = 1; i < s->ntotal; i++) {
            double v = s->x[i * nd + d];
            if (v < mn) mn = v;
            if (v > mx) mx = v;
        }
        xminp[d] = mn - 0.00001;
        xmaxp[d] = mx + 0.00001;
        xminp[d] = xminp[d] - s->dxcell - 0.00001;
        xmaxp[d] = xmaxp[d] + s->dxcell + 0.00001;
        s->ncellsx[d] = (int)((xmaxp[d] - xminp[d]) / s->dxcell) + 1;
        if (s->ncellsx[d] == 0) { s->err = NDSPH_E_CELLS; return s->err; }
    }
    long nc = 1;
    for (int d = 0; d < nd; d++) nc *= s->ncellsx[d];
    if (nc > 400000000L) { s->err = NDSPH_E_CELLS; snprintf(s->msg, sizeof s->msg, "link: too many cells"); return s->err; }
    s->ncells = (int)nc;
    free(s->ifirstincell);
    s->ifirstincell = malloc(sizeof(int) * (size_t)nc);
    for (long c = 0; c < nc; c++) s->ifirstincell[c] = -1;
    for (int i = 0; i < s->ntotal; i++) {
        s->ll[i] = -1;
        int icx[MAXNDIM];
        for (int d = 0; d < nd; d++) {
            icx[d] = (int)((s->x[i * nd + d] - xminp[d]) / s->dxcell) + 1;
            if (icx[d] < 0 || icx[d] > s->ncellsx[d]) {
                s->err = NDSPH_E_CELLS; snprintf(s->msg, sizeof s->msg, "link: particle crossed boundary %d", i);
                return s->err;
            }
        }
        int icell = icx[0];
        if (nd >= 2) icell += (icx[1] - 1) * s->ncellsx[0];
        if (nd >= 3) icell += (icx[2] - 1) * s->ncellsx[0] * s->ncellsx[1];
        icell -= 1;                                   /* to 0-based */
        s->ll[i] = s->ifirstincell[icell];
        s->ifirstincell[icell] = i;
        s->iamincell[i] = icell;
    }
    return 0;
}

/* get_neighbour_list get_neighbour_lists.f90:37-165 (half stencil) */
static int get_neighbour_list(orc_sim* s, int icell, int* list)
{
    if (s->ifirstincell[icell] < 0) return 0;
    int nc[14], n = 0, nx = s->ncellsx[0];
    nc[n++] = icell; nc[n++] = icell + 1;
    if (s->ndim >= 2) { nc[n++] = icell + nx - 1; nc[n++] = icell + nx; nc[n++] = icell + nx + 1; }
    if (s->ndim >= 3) {
        int nxy = s->ncellsx[0] * s->ncellsx[1];
        nc[n++] = icell + nxy - 1; nc[n++] = icell + nxy; nc[n++] = icell + nxy + 1;
        nc[n++] = icell + nxy + nx - 1; nc[n++] = icell + nxy + nx; nc[n++] = icell + nxy + nx + 1;
        nc[n++] = icell + nxy - nx - 1; nc[n++] = icell + nxy - nx; nc[n++] = icell + nxy - nx + 1;
    }
    int j = 0;
    for (int k = 0; k < n; k++) {
        if (nc[k] >= s->ncells) { s->err = NDSPH_E_CELLS; return 0; }
        for (int ip = s->ifirstincell[nc[k]]; ip >= 0; ip = s->ll[ip]) list[j++] = ip;
    }
    return j;
}

/* get_neighbour_list_partial get_neighbour_lists.f90:176-316 (full stencil) */
static int get_neighbour_list_partial(orc_sim* s, int icell, int* list)
{
    if (s->ifirstincell[icell] < 0) return 0;
    int nc[27], n = 0, nx = s->ncellsx[0];
    nc[n++] = icell - 1; nc[n++] = icell; nc[n++] = icell + 1;
    if (s->ndim >= 2) {
        nc[n++] = icell + nx - 1; nc[n++] = icell + nx; nc[n++] = icell + nx + 1;
        nc[n++] = icell - nx - 1; nc[n++] = icell - nx; nc[n++] = icell - nx + 1;
        if (s->ndim >= 3) {
            int nxy = s->ncellsx[0] * s->ncellsx[1];
            int base[3] = {nxy, 0, -nxy};
            (void)base;
            nc[n++] = icell + nxy + nx - 1; nc[n++] = icell + nxy + nx; nc[n++] = icell + nxy + nx + 1;
            nc[n++] = icell + nxy - 1; nc[n++] = icell + nxy; nc[n++] = icell + nxy + 1;
            nc[n++] = icell + nxy - nx - 1; nc[n++] = icell + nxy - nx; nc[n++] = icell + nxy - nx + 1;
            nc[n++] = icell - nxy + nx - 1; nc[n++] = icell - nxy + nx; nc[n++] = icell - nxy + nx + 1;
            nc[n++] = icell - nxy - 1; nc[n++] = icell - nxy; nc[n++] = icell - nxy + 1;
            nc[n++] = icell - nxy - nx - 1; nc[n++] = icell - nxy - nx; nc[n++] = icell - nxy - nx + 1;
        }
    }
    int j = 0;
    for (int k = 0; k < n; k++) {
        if (nc[k] >= s->ncells || nc[k] < 0) { s->err = NDSPH_E_CELLS; return 0; }
        for (int ip = s->ifirstincell[nc[k]]; ip >= 0; ip = s->ll[ip]) list[j++] = ip;
    }
    return j;
}

static inline int type_match(int ti, int tj)
{
    /* density_sums.f90:168-172, ratesND_mhd.f90:437-440 */
    return (tj == ti) || (ti == NDSPH_ITYPE_GAS && tj == NDSPH_ITYPE_BND) ||
           (tj == NDSPH_ITYPE_GAS && ti == NDSPH_ITYPE_BND) ||
           (ti == NDSPH_ITYPE_DUST && tj == NDSPH_ITYPE_BNDDUST) ||
           (tj == NDSPH_ITYPE_DUST && ti == NDSPH_ITYPE_BNDDUST);
}

static inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

static inline double dotn(const double* a, const double* b, int n)
{
    double r = a[0] * b[0];
    for (int d = 1; d < n; d++) r = r + a[d] * b[d];
    return r;
}

/* density density_sums.f90:38-379 (in-scope branches: ikernav=3, igravity=0,
 * imhd /= 5, iprterm=0, no one-fluid dust).  Symmetric half-stencil pairs with
 * the union criterion and its Fortran precedence (:189-190).                   */
static void density_full(orc_sim* s, double* densn)
{
    const int nd = s->ndim, np = s->npart, nt = s->ntotal;
    const orc_kernels* K = &s->K;
    for (int i = 0; i < np; i++) {
        if (s->itype[i] != NDSPH_ITYPE_BND && s->itype[i] != NDSPH_ITYPE_BNDDUST) {
            s->rho[i] = 0.; s->drhodt[i] = 0.; densn[i] = 0.;
            s->gradh[i] = 0.; s->gradhn[i] = 0.; s->gradsoft[i] = 0.; s->gradgradh[i] = 0.;
        }
    }
    for (int i = 0; i < s->cap; i++) s->numneigh[i] = 0;
    double* h1 = malloc(sizeof(double) * (size_t)nt);
    for (int i = 0; i < nt; i++) h1[i] = 1. / s->hh[i];
    double dr[3] = {0, 0, 0};
    for (int icell = 0; icell < s->ncells; icell++) {
        int nneigh = get_neighbour_list(s, icell, s->listneigh);
        int idone = -1;
        for (int i = s->ifirstincell[icell]; i >= 0; i = s->ll[i]) {
            idone++;
            double pmassi = s->pmass[i];
            const double* xi = &s->x[i * nd];
            const double* veli = &s->vel[i * 3];
            double hi = s->hh[i], hi1 = h1[i];
            double hfacwabi = powi_f(hi1, nd);
            double hi21 = hi1 * hi1;
            int itypei = s->itype[i];
            for (int n = idone; n < nneigh; n++) {
                int j = s->listneigh[n];
                int itypej = s->itype[j];
                if (!type_match(itypei, itypej)) continue;
                double dx[MAXNDIM];
                for (int d = 0; d < nd; d++) dx[d] = xi[d] - s->x[j * nd + d];
                double hj1 = h1[j];
                double rij2 = dotn(dx, dx, nd);
                double q2i = rij2 * hi21;
                double q2j = rij2 * hj1 * hj1;
                if ((q2i < K->radkern2) || ((q2j < K->radkern2) && (i < np || j < np))) {
                    if (i < np) s->numneigh[i]++;
                    if (j < np && j != i) s->numneigh[j]++;
                    double rij = sqrt(rij2);
                    for (int d = 0; d < nd; d++) dr[d] = dx[d] / (rij + DBL_EPSILON);
                    double hfacwabj = powi_f(hj1, nd);
                    double weight = (j == i) ? 0.5 : 1.0;
                    double pmassj = s->pmass[j];
                    double wabi, grkerni, grgrkerni, wabalti, grkernalti;
                    double wabj, grkernj, grgrkernj, wabaltj, grkernaltj;
                    interp_dens(K, q2i, &wabi, &grkerni, &grgrkerni, &wabalti, &grkernalti);
                    interp_dens(K, q2j, &wabj, &grkernj, &grgrkernj, &wabaltj, &grkernaltj);
                    wabi = wabi * hfacwabi;
                    wabalti = wabalti * hfacwabi;
                    grkerni = grkerni * hfacwabi * hi1;
                    grgrkerni = grgrkerni * hfacwabi * hi1 * hi1;
                    grkernalti = grkernalti * hfacwabi * hi1;
                    wabj = wabj * hfacwabj;
                    wabaltj = wabaltj * hfacwabj;
                    grkernj = grkernj * hfacwabj * hj1;
                    grgrkernj = grgrkernj * hfacwabj * hj1 * hj1;
                    grkernaltj = grkernaltj * hfacwabj * hj1;
                    double dwdhi = -rij * grkerni * hi1 - nd * wabi * hi1;
                    double dwdhj = -rij * grkernj * hj1 - nd * wabj * hj1;
                    double dwaltdhi = -rij * grkernalti * hi1 - nd * wabalti * hi1;
                    double dwaltdhj = -rij * grkernaltj * hj1 - nd * wabaltj * hj1;
                    double dwdhdhi = (nd * (nd + 1)) * wabi * (hi1 * hi1) + 2. * (nd + 1) * rij * (hi1 * hi1) * grkerni
                                   + (rij * rij) * (hi1 * hi1) * grgrkerni;
                    double dwdhdhj = (nd * (nd + 1)) * wabj * (hj1 * hj1) + 2. * (nd + 1) * rij * (hj1 * hj1) * grkernj
                                   + (rij * rij) * (hj1 * hj1) * grgrkernj;
                    if (itypei != NDSPH_ITYPE_BND) {
                        s->rho[i] += pmassj * wabi * weight;
                        densn[i] += wabalti * weight;
                    }
                    if (itypej != NDSPH_ITYPE_BND) {
                        s->rho[j] += pmassi * wabj * weight;
                        densn[j] += wabaltj * weight;
                    }
                    if (i != j) {
                        double dvel[3];
                        for (int d = 0; d < 3; d++) dvel[d] = veli[d] - s->vel[j * 3 + d];
                        double dvdotr = dot3(dvel, dr);
                        s->drhodt[i] += pmassj * dvdotr * grkerni;
                        s->drhodt[j] += pmassi * dvdotr * grkernj;
                    }
                    if (itypei != NDSPH_ITYPE_BND) {
                        s->gradh[i] += weight * pmassj * dwdhi;
                        s->gradhn[i] += weight * dwaltdhi;
                        s->gradgradh[i] += weight * pmassj * dwdhdhi;
                    }
                    if (itypej != NDSPH_ITYPE_BND) {
                        s->gradh[j] += weight * pmassi * dwdhj;
                        s->gradhn[j] += weight * dwaltdhj;
                        s->gradgradh[j] += weight * pmassi * dwdhdhj;
                    }
                }
            }
            (void)hi;
        }
    }
    free(h1);
}

/* density_partial density_sums.f90:396-658 (gather over the full stencil,
 * q_i < 2 only, for the particles in ipartlist)                               */
static void density_partial(orc_sim* s, double* densn, int nlist, const int* ipartlist)
{
    const int nd = s->ndim;
    const orc_kernels* K = &s->K;
    double dr[3] = {0, 0, 0};
    for (int ip = 0; ip < nlist; ip++) {
        int i = ipartlist[ip];
        s->rho[i] = 0.; s->drhodt[i] = 0.; densn[i] = 0.; s->gradh[i] = 0.; s->gradhn[i] = 0.;
        s->gradsoft[i] = 0.; s->gradgradh[i] = 0.; s->numneigh[i] = 0;
    }
    int icellprev = -1, nneigh = 0;
    for (int ip = 0; ip < nlist; ip++) {
        int i = ipartlist[ip];
        int icell = s->iamincell[i];
        if (icell != icellprev) nneigh = get_neighbour_list_partial(s, icell, s->listneigh);
        icellprev = icell;
        double hi = s->hh[i];
        double hi1 = 1. / hi;
        double hi21 = hi1 * hi1;
        double hfacwabi = powi_f(hi1, nd);
        double hfacgrkerni = hfacwabi * hi1;
        const double* xi = &s->x[i * nd];
        const double* veli = &s->vel[i * 3];
        int itypei = s->itype[i];
        if (itypei == NDSPH_ITYPE_BND) continue;
        for (int n = 0; n < nneigh; n++) {
            int j = s->listneigh[n];
            if (s->itype[j] != itypei && s->itype[j] != NDSPH_ITYPE_BND) continue;
            double dx[MAXNDIM];
            for (int d = 0; d < nd; d++) dx[d] = xi[d] - s->x[j * nd + d];
            double rij2 = dotn(dx, dx, nd);
            double q2i = rij2 * hi21;
            if (q2i < K->radkern2) {
                double rij = sqrt(rij2);
                for (int d = 0; d < nd; d++) dr[d] = dx[d] / (rij + DBL_EPSILON);
                s->numneigh[i]++;
                double pmassj = s->pmass[j];
                double wabi, grkerni, grgrkerni, wabalti, grkernalti;
                interp_dens(K, q2i, &wabi, &grkerni, &grgrkerni, &wabalti, &grkernalti);
                wabi = wabi * hfacwabi;
                wabalti = wabalti * hfacwabi;
                grkerni = grkerni * hfacgrkerni;
                grgrkerni = grgrkerni * hfacwabi * hi1 * hi1;
                grkernalti = grkernalti * hfacgrkerni;
                double dwdhi = -rij * grkerni * hi1 - nd * wabi * hi1;
                double dwaltdhi = -rij * grkernalti * hi1 - nd * wabalti * hi1;
                double dwdhdhi = (nd * (nd + 1)) * wabi * (hi1 * hi1) + 2. * (nd + 1) * rij * (hi1 * hi1) * grkerni
                               + (rij * rij) * (hi1 * hi1) * grgrkerni;
                s->rho[i] += pmassj * wabi;
                densn[i] += wabalti;
                if (i != j) {
                    double dvel[3];
                    for (int d = 0; d < 3; d++) dvel[d] = veli[d] - s->vel[j * 3 + d];
                    double dvdotr = dot3(dvel, dr);
                    s->drhodt[i] += pmassj * dvdotr * grkerni;
                }
                s->gradh[i] += pmassj * dwdhi;
                s->gradhn[i] += dwaltdhi;
                s->gradgradh[i] += pmassj * dwdhdhi;
            }
        }
    }
}

static void copy_density_to_ghosts(orc_sim* s)
{
    /* iterate_density.f90:312-344 */
    int any1 = 0, anygt1 = 0;
    for (int d = 0; d < s->ndim; d++) { if (s->o.ibound[d] == 1) any1 = 1; if (s->o.ibound[d] > 1) anygt1 = 1; }
    if (any1) {
        for (int i = 0; i < s->npart; i++) {
            if (s->itype[i] == NDSPH_ITYPE_BND) {
                int j = s->ireal[i];
                if (j >= 0) {
                    s->rho[i] = s->rho[j]; s->rhoalt[i] = s->rhoalt[j]; s->drhodt[i] = s->drhodt[j];
                    s->dhdt[i] = s->dhdt[j]; s->hh[i] = s->hh[j]; s->gradh[i] = s->gradh[j];
                    s->gradhn[i] = s->gradhn[j]; s->gradsoft[i] = s->gradsoft[j];
                }
            }
        }
    }
    if (anygt1) {
        for (int i = s->npart; i < s->ntotal; i++) {
            int j = s->ireal[i];
            if (j >= 0) {
                s->rho[i] = s->rho[j]; s->rhoalt[i] = s->rhoalt[j]; s->drhodt[i] = s->drhodt[j];
                s->dhdt[i] = s->dhdt[j]; s->hh[i] = s->hh[j]; s->gradh[i] = s->gradh[j];
                s->gradhn[i] = s->gradhn[j]; s->gradsoft[i] = s->gradsoft[j];
            }
        }
    }
}

static int any_ibound_gt1(const orc_sim* s)
{
    for (int d = 0; d < s->ndim; d++) if (s->o.ibound[d] > 1) return 1;
    return 0;
}

/* iterate_density iterate_density.f90:43-360 (usenumdens = .false.,
 * ibiascorrection = 0, h_min = 0, rhomin = 0)                                 */
static int iterate_density(orc_sim* s)
{
    const int nd = s->ndim, np = s->npart;
    const double hfact = s->o.hfact, tolh = s->o.tolh;
    const int itsmax = s->o.maxdensits;
    const double h_min = 0.0, rhomin = 0.0;
    double dndim = 1.0 / nd;
    int* redolist = malloc(sizeof(int) * (size_t)(np > 0 ? np : 1));
    int* redoprev = malloc(sizeof(int) * (size_t)(np > 0 ? np : 1));
    double* hhin = malloc(sizeof(double) * (size_t)(np > 0 ? np : 1));
    s->itsdensity = 0;
    s->ncalctotal = 0;
    s->nrelink = 0;
    int ncalc = np;
    int redolink = 0;
    for (int i = 0; i < s->cap; i++) {
        if (s->itype[i] != NDSPH_ITYPE_BND) {
            s->gradh[i] = 0.; s->gradhn[i] = 0.; s->gradsoft[i] = 0.; s->gradgradh[i] = 0.;
            s->drhodt[i] = 0.; s->dhdt[i] = 0.;
        }
    }
    for (int i = 0; i < np; i++) hhin[i] = s->hh[i];
    for (int i = 0; i < np; i++) {
        if (s->hh[i] <= DBL_MIN) {
            s->err = NDSPH_E_H_NONPOS; snprintf(s->msg, sizeof s->msg, "error: h <= 0 in density call");
            goto out;
        }
    }
    for (int j = 0; j < np; j++) redolist[j] = j;
    while (ncalc > 0 && s->itsdensity <= itsmax) {
        s->itsdensity++;
        if (redolink) {
            if (any_ibound_gt1(s)) set_ghost_particles(s);
            if (set_linklist(s)) goto out;
            s->nrelink++;
        }
        if (ncalc == np) density_full(s, s->rhoalt);
        else density_partial(s, s->rhoalt, ncalc, redolist);
        if (s->err) goto out;
        s->ncalctotal += ncalc;
        int ncalcprev = ncalc;
        memcpy(redoprev, redolist, sizeof(int) * (size_t)ncalcprev);
        ncalc = 0;
        redolink = 0;
        for (int jj = 0; jj < ncalcprev; jj++) {
            int i = redoprev[jj];
            if (s->itype[i] == NDSPH_ITYPE_BND || s->itype[i] == NDSPH_ITYPE_BNDDUST) continue;
            if (s->rho[i] <= 1.e-6 && s->rho[i] <= 0.) {
                s->err = NDSPH_E_RHO_NONPOS; snprintf(s->msg, sizeof s->msg, "error: rho(%d) <= 0", i + 1);
                goto out;
            }
            double rhoi = s->pmass[i] / powi_f((s->hh[i] - h_min) / hfact, nd) - rhomin;
            double dhdrhoi = -(s->hh[i] - h_min) / (nd * (s->rho[i] + rhomin));
            double dwdhsumi = s->gradh[i];
            double omegai = 1. - dhdrhoi * s->gradh[i];
            if (omegai < 1.e-5) { if (fabs(omegai) == 0.) omegai = 1.; }
            s->gradh[i] = 1. / omegai;
            double func = rhoi - s->rho[i];
            double dfdh = omegai / dhdrhoi;
            s->gradsoft[i] = s->gradsoft[i] * dhdrhoi;
            double d2hdrho2i = s->hh[i] * (nd + 1) / powi_f(s->rho[i] * nd, 2);
            s->gradgradh[i] = s->rho[i] * (d2hdrho2i * dwdhsumi + powi_f(dhdrhoi, 2) * s->gradgradh[i]);
            double hnew = s->hh[i] - func / dfdh;
            if (hnew > 1.2 * s->hh[i]) hnew = 1.2 * s->hh[i];
            else if (hnew < 0.8 * s->hh[i]) hnew = 0.8 * s->hh[i];
            if (hnew <= 0 || s->gradh[i] <= DBL_MIN) {
                hnew = hfact * pow(s->pmass[i] / (s->rho[i] + rhomin), dndim);
            } else if (s->itsdensity > 100) {
                hnew = hfact * pow(s->pmass[i] / (s->rho[i] + rhomin), dndim);
            }
            if (s->numneigh[i] <= 1) {
                hnew = s->hh[i] + s->o.psep;
                redolink = 1;
            }
            int converged = (fabs((hnew - s->hh[i]) / hhin[i]) < tolh && omegai > 0.) || itsmax == 0;
            if (!converged) {
                redolist[ncalc++] = i;
                if (s->itsdensity <= itsmax && s->itype[i] != NDSPH_ITYPE_BND) s->hh[i] = hnew;
                if (hnew > s->hhmax) redolink = 1;
            } else {
                s->drhodt[i] = s->drhodt[i] * s->gradh[i];
                s->dhdt[i] = dhdrhoi * s->drhodt[i];
            }
        }
        copy_density_to_ghosts(s);
    }
    if (s->itsdensity > itsmax && itsmax > 0) {
        s->err = NDSPH_E_NOT_CONVERGED;
        snprintf(s->msg, sizeof s->msg, "ERROR: DENSITY NOT CONVERGED ON %d PARTICLES", ncalc);
    }
out:
    free(redolist); free(redoprev); free(hhin);
    return s->err;
}

/* equation_of_state eos.f90:40-106 on 1..npart; stops on u < 0 when
 * iener /= 0 (eos.f90:66-72) */
static void equation_of_state(orc_sim* s)
{
    double gamma = s->o.gamma, gamma1 = gamma - 1.;
    if (s->o.iener != 0) {
        for (int i = 0; i < s->npart; i++) {
            if (s->uu[i] < 0.) {
                s->err = NDSPH_E_U_NEG;
                snprintf(s->msg, sizeof s->msg, "eos: u_therm -ve at %d", i + 1);
                return;
            }
        }
    }
    for (int i = 0; i < s->npart; i++) {
        double rho = s->rho[i];
        if (s->o.iener == 0) {
            if (rho > 0. && s->itype[i] == NDSPH_ITYPE_GAS) {
                s->pr[i] = s->o.polyk * pow(rho, gamma);
                s->spsound[i] = sqrt(gamma * s->pr[i] / rho);
            } else if (s->itype[i] != NDSPH_ITYPE_BND) {
                s->pr[i] = 0.;
            }
            if (fabs(gamma1) > 1.e-3 && rho > 0.) s->uu[i] = s->pr[i] / (gamma1 * rho);
        } else {
            if (rho > 0.) {
                s->pr[i] = gamma1 * s->uu[i] * rho;
                s->spsound[i] = sqrt(gamma * s->pr[i] / rho);
            }
        }
    }
}

/* conservative2primitive conservative2primitive.f90:42-470, in-scope part:
 * dens = rho (:103), B from Bevol (:151-152, :196-199), uu = en (:360-372),
 * EOS (:424), fixed-particle copies (:430-441), ghost copies (:444-468)       */
static void conservative2primitive(orc_sim* s)
{
    for (int i = 0; i < s->cap; i++) s->dens[i] = s->rho[i];
    if (s->o.imhd >= 11) {
        for (int i = 0; i < 3 * s->cap; i++) s->Bfield[i] = s->Bevol[i];
    } else if (s->o.imhd >= 1 && s->o.imhd <= 9) {
        for (int i = 0; i < s->npart; i++)
            for (int d = 0; d < 3; d++) s->Bfield[i * 3 + d] = s->Bevol[i * 3 + d] * s->rho[i];
    }
    for (int i = 0; i < s->cap; i++) s->uu[i] = s->en[i];
    equation_of_state(s);
    int any1 = 0;
    for (int d = 0; d < s->ndim; d++) if (s->o.ibound[d] == 1) any1 = 1;
    if (any1) {
        for (int i = 0; i < s->npart; i++) {
            if (s->itype[i] == NDSPH_ITYPE_BND || s->itype[i] == NDSPH_ITYPE_BNDDUST) {
                int j = s->ireal[i];
                if (j >= 0) copy_particle(s, i, j);
            }
        }
    }
    if (any_ibound_gt1(s)) {
        for (int i = s->npart; i < s->ntotal; i++) {
            int j = s->ireal[i];
            for (int d = 0; d < 3; d++) s->curlB[i * 3 + d] = s->curlB[j * 3 + d];
            s->psi[i] = s->psi[j]; s->dens[i] = s->dens[j];
            s->uu[i] = s->uu[j]; s->spsound[i] = s->spsound[j]; s->pr[i] = s->pr[j];
            for (int d = 0; d < 3; d++) s->Bfield[i * 3 + d] = s->Bfield[j * 3 + d];
            copy_particle(s, i, j);
        }
    }
}

/* ------------------------------------------------------------------------- */
/* get_rates ratesND_mhd.f90:29-979                                           */
/* ------------------------------------------------------------------------- */
typedef struct {
    /* particle-i locals of get_rates :318-400 */
    int i, itypei;
    double rhoi, rho2i, rho1i, rho21i, pri, prneti, pmassi, Prho2i, spsoundi, uui;
    double veli[3], alphai, alphaui, alphaBi, Bi[3], Brhoi[3], B2i, Brho2i, valfven2i;
    double gradhi, hi, hi1, hi21, hfacwabi, hfacgrkerni;
    double forcei[3], dBevoldti[3];
    /* pair */
    int j;
    double dx[3], rij, rij2, q2i, q2j, dr[3];
    /* global reductions */
    double dtcourant, dtav, vsigmax, ts_min, h_on_csts_max, stressmax;
} rates_ctx;

static void artificial_dissipation(orc_sim* s, rates_ctx* c, double vsig, double vsigu, double vsigB,
                                   double rhoav1, double grkern, double dvdotr, const double* dvel,
                                   const double* dB, const double* velj, double rhoj, double pmassj,
                                   double* forcej, double* vsigav_out)
{
    /* artificial_dissipation ratesND_mhd.f90:1700-1894 (iav=2, cartesian) */
    int j = c->j;
    double alphaav = 0.5 * (c->alphai + s->alpha[j * 3 + 0]);
    double alphau = 0.5 * (c->alphaui + s->alpha[j * 3 + 1]);
    double alphaB = 0.5 * (c->alphaBi + s->alpha[j * 3 + 2]);
    double amax = alphaav;
    if (alphau > amax) amax = alphau;
    if (alphaB > amax) amax = alphaB;
    *vsigav_out = amax * vsig;
    double dpmomdotr = -dvdotr;
    double term = vsig * rhoav1 * grkern;
    double termv = term;
    double termu = vsigu * rhoav1 * grkern;
    double termB = vsigB * rhoav1 * grkern;
    if (dvdotr < 0 && s->o.iav <= 3) {
        double visc = alphaav * termv * dpmomdotr;
        for (int d = 0; d < 3; d++) {
            c->forcei[d] = c->forcei[d] - pmassj * visc * c->dr[d];
            forcej[d] = forcej[d] + c->pmassi * visc * c->dr[d];
        }
    }
    if (s->o.imhd != 0 && s->o.imhd > 0 && s->o.imhd != 10 && s->o.iav >= 2) {
        for (int d = 0; d < 3; d++) {
            double Bvisc = dB[d] * rhoav1;
            double dBdtvisc = alphaB * termB * Bvisc;
            c->dBevoldti[d] = c->dBevoldti[d] + c->rhoi * pmassj * dBdtvisc;
            s->dBevoldt[j * 3 + d] = s->dBevoldt[j * 3 + d] - rhoj * c->pmassi * dBdtvisc;
        }
    }
    if (s->o.iener > 0 && s->o.iener != 3) {
        double vissv;
        if (dvdotr < 0 && s->o.iav <= 3) {
            double t = dot3(c->veli, c->dr) - dot3(velj, c->dr);
            vissv = -alphaav * 0.5 * (t * t);
        } else {
            vissv = 0.;
        }
        double vissu = (s->o.iener == 1) ? 0. : alphau * (s->uu[c->i] - s->uu[j]);
        double vissB = 0.;
        if (s->o.imhd > 0 && s->o.imhd != 10 && s->o.iav >= 2) vissB = -alphaB * 0.5 * (dot3(dB, dB)) * rhoav1;
        s->dudt[c->i] = s->dudt[c->i] + pmassj * (term * (vissv) + termu * vissu + termB * (vissB));
        s->dudt[j] = s->dudt[j] + c->pmassi * (term * (vissv) - termu * vissu + termB * (vissB));
    }
    (void)dvel;
}

static inline void cross3(const double* a, const double* b, double* c)
{
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

/* rates_core ratesND_mhd.f90:1175-1690 + mhd_terms :2377-2720 (imagforce
 * default case, imhd 1 and 11)                                                 */
static int rates_core(orc_sim* s, rates_ctx* c)
{
    const orc_kernels* K = &s->K;
    const int nd = s->ndim;
    int i = c->i, j = c->j;
    double pmassj = s->pmass[j];
    double hj = s->hh[j], hj1 = 1. / hj;
    double wabi, grkerni, grkernalti, grgrkernalti;
    double wabj, grkernj, grkernaltj, grgrkernaltj;
    interp_rates(K, c->q2i, &wabi, &grkerni, &grkernalti, &grgrkernalti);
    wabi = wabi * c->hfacwabi;
    grkerni = grkerni * c->hfacgrkerni;
    double hfacwabj = powi_f(hj1, nd);
    double hfacgrkernj = hfacwabj * hj1;
    interp_rates(K, c->q2j, &wabj, &grkernj, &grkernaltj, &grgrkernaltj);
    wabj = wabj * hfacwabj;
    grkernj = grkernj * hfacgrkernj;
    grkerni = grkerni * c->gradhi;
    grkernj = grkernj * s->gradh[j];
    double grkern = 0.5 * (grkerni + grkernj);

    const double* velj = &s->vel[j * 3];
    double dvel[3];
    for (int d = 0; d < 3; d++) dvel[d] = c->veli[d] - velj[d];
    double dvdotr = dot3(dvel, c->dr);
    double rhoj = s->rho[j];
    double rho1j = 1. / rhoj;
    double rho21j = rho1j * rho1j;
    double rhoav1 = 0.5 * (c->rho1i + rho1j);
    double prj = fmax(s->pr[j] - 0.0, 0.);
    double prnetj = prj;
    double Prho2j = prj * rho21j;
    double spsoundj = s->spsound[j];

    double Bj[3] = {0, 0, 0}, Brhoj[3] = {0, 0, 0}, dB[3] = {0, 0, 0};
    double projBi = 0, projBj = 0, projdB = 0, projBrhoi = 0, projBrhoj = 0, B2j = 0, valfven2j = 0, Brho2j = 0;
    if (s->o.imhd != 0) {
        for (int d = 0; d < 3; d++) {
            Bj[d] = s->Bfield[j * 3 + d];
            Brhoj[d] = Bj[d] * rho1j;
            dB[d] = c->Bi[d] - Bj[d];
        }
        projBi = dot3(c->Bi, c->dr);
        projBj = dot3(Bj, c->dr);
        projdB = dot3(dB, c->dr);
        projBrhoi = dot3(c->Brhoi, c->dr);
        projBrhoj = dot3(Brhoj, c->dr);
        B2j = dot3(Bj, Bj);
        valfven2j = B2j * rho1j;
        Brho2j = B2j * rho21j;
    }
    double forcej[3] = {0, 0, 0};
    double vsig, vsigi, vsigj, vsigB, vsigu, vsigdtc, vsigav = 0.;
    if (s->o.imhd != 0) {
        double vsig2i = c->spsoundi * c->spsoundi + c->valfven2i;
        double vsig2j = spsoundj * spsoundj + valfven2j;
        double ti = c->spsoundi * projBi, tj = spsoundj * projBj;
        double vsigproji = vsig2i * vsig2i - 4. * (ti * ti) * c->rho1i;
        double vsigprojj = vsig2j * vsig2j - 4. * (tj * tj) * rho1j;
        if (vsigproji < 0. || vsigprojj < 0.) {
            s->err = NDSPH_E_VSIG_DET;
            snprintf(s->msg, sizeof s->msg, "rates: vsig det < 0 (i=%d j=%d)", i + 1, j + 1);
            return s->err;
        }
        vsigi = sqrt(0.5 * (vsig2i + sqrt(vsigproji)));
        vsigj = sqrt(0.5 * (vsig2j + sqrt(vsigprojj)));
        vsigB = sqrt(dot3(dvel, dvel));   /* norm2(dvel), iavlim(3) /= 2 */
    } else {
        vsigi = c->spsoundi;
        vsigj = spsoundj;
        vsigB = 0.;
    }
    vsig = 0.5 * fmax(vsigi + vsigj - s->o.beta * dvdotr, 0.0);
    vsigu = sqrt(fabs(c->prneti - prnetj) * rhoav1);
    vsigdtc = vsig;
    double t2 = 0.5 * (vsigi + vsigj + s->o.beta * fabs(dvdotr));
    if (t2 > vsigdtc) vsigdtc = t2;
    if (vsigB > vsigdtc) vsigdtc = vsigB;
    if (s->itype[i] == NDSPH_ITYPE_DUST) {
        vsig = 0.; vsigu = 0.;
    } else {
        double dvsigdtc = 1. / vsigdtc;
        if (vsigdtc > c->vsigmax) c->vsigmax = vsigdtc;
        if (vsigdtc > 1.e-10) {
            double a = c->hi * dvsigdtc, b = hj * dvsigdtc;
            double m = (a < b) ? a : b;
            if (m < c->dtcourant) c->dtcourant = m;
        }
    }
    if (s->o.iav > 0)
        artificial_dissipation(s, c, vsig, vsigu, vsigB, rhoav1, grkern, dvdotr, dvel, dB, velj, rhoj,
                               pmassj, forcej, &vsigav);
    if (vsigav > 1.e-10) {
        double a = c->hi / vsigav, b = hj / vsigav;
        double m = (a < b) ? a : b;
        if (m < c->dtav) c->dtav = m;
    }
    /* pressure term :1538-1568 (iprterm = 0, phi = 1, sqrtg = 1) */
    double prterm = 1. * c->Prho2i * 1. * grkerni + 1. * Prho2j * 1. * grkernj;
    for (int d = 0; d < 3; d++) {
        c->forcei[d] = c->forcei[d] - pmassj * prterm * c->dr[d];
        forcej[d] = forcej[d] + c->pmassi * prterm * c->dr[d];
    }
    if (s->o.imhd != 0) {
        /* mhd_terms, imagforce default (tensor) case :2522-2541 */
        double fiso = 0.5 * (c->Brho2i * 1. * grkerni * 1. + Brho2j * 1. * grkernj * 1.);
        double fmagi[3];
        for (int d = 0; d < 3; d++) {
            double faniso = (1. * c->Brhoi[d] * projBrhoi * 1. - c->stressmax * c->dr[d] * c->rho21i) * 1. * grkerni
                          + (1. * Brhoj[d] * projBrhoj * 1. - c->stressmax * c->dr[d] * rho21j) * 1. * grkernj;
            fmagi[d] = faniso - fiso * c->dr[d];
        }
        s->divB[i] = s->divB[i] - pmassj * projdB * grkern;
        s->divB[j] = s->divB[j] - c->pmassi * projdB * grkern;
        if (s->o.imhd > 0) {
            double cb[3];
            cross3(dB, c->dr, cb);
            for (int d = 0; d < 3; d++) {
                s->curlB[i * 3 + d] = s->curlB[i * 3 + d] + pmassj * cb[d] * grkern;
                s->curlB[j * 3 + d] = s->curlB[j * 3 + d] + c->pmassi * cb[d] * grkern;
            }
        }
        for (int d = 0; d < 3; d++) {
            c->forcei[d] = c->forcei[d] + pmassj * (fmagi[d]);
            forcej[d] = forcej[d] - c->pmassi * (fmagi[d]);
        }
        /* induction equation, imhd 1 / 11 :2663-2667 (dBdtambi = 0) */
        if (s->o.imhd == 1 || s->o.imhd == 11) {
            for (int d = 0; d < 3; d++) {
                c->dBevoldti[d] = c->dBevoldti[d] - 1. * pmassj * ((dvel[d] * projBrhoi) * grkerni + c->rhoi * 0.);
                s->dBevoldt[j * 3 + d] = s->dBevoldt[j * 3 + d] - 1. * c->pmassi * ((dvel[d] * projBrhoj) * grkernj - rhoj * 0.);
            }
        }
    }
    for (int d = 0; d < 3; d++) s->force[j * 3 + d] = s->force[j * 3 + d] + 0. + forcej[d];
    if (s->o.iav > 0) {
        if (s->o.iavlim[1] > 0) {
            double graduterm = (s->uu[i] - s->uu[j]) / c->rij;
            s->del2u[i] = s->del2u[i] + pmassj * rho1j * graduterm * grkerni;
            s->del2u[j] = s->del2u[j] - c->pmassi * c->rho1i * graduterm * grkernj;
        }
        if (s->o.iavlim[0] != 3) {
            for (int d = 0; d < 3; d++) {
                s->graddivv[i * 3 + d] = s->graddivv[i * 3 + d] + pmassj * (dvel[d] - dvdotr) * grkerni;
                s->graddivv[j * 3 + d] = s->graddivv[j * 3 + d] + c->pmassi * (-dvel[d] - dvdotr) * grkernj;
            }
        }
    }
    (void)wabi; (void)wabj; (void)grkernalti; (void)grgrkernalti; (void)grkernaltj; (void)grgrkernaltj;
    return 0;
}

/* drag_forces ratesND_mhd.f90:1074-1169, get_tstop dust.f90:77-101
 * (idrag_nature = 1, islope_limiter < 0, ibound(1) /= 5)                        */
static void drag_forces(orc_sim* s, rates_ctx* c)
{
    const orc_kernels* K = &s->K;
    const int nd = s->ndim;
    int i = c->i, j = c->j;
    double dvel[3], drdrag[3];
    for (int d = 0; d < 3; d++) dvel[d] = c->veli[d] - s->vel[j * 3 + d];
    double dv2 = dot3(dvel, dvel);
    if (c->rij <= DBL_EPSILON) {
        if (dv2 <= DBL_EPSILON) return;
        double vij = sqrt(dv2);
        for (int d = 0; d < 3; d++) drdrag[d] = dvel[d] / vij;
    } else {
        for (int d = 0; d < 3; d++) drdrag[d] = c->dr[d];
    }
    double wabi = interp_drag(K, c->q2i);
    double wabj = interp_drag(K, c->q2j);
    wabi = wabi * c->hfacwabi;
    double hfacwabj = 1. / powi_f(s->hh[j], nd);
    wabj = wabj * hfacwabj;
    int itypej = s->itype[j];
    double pmassj = s->pmass[j];
    double rhoj = s->rho[j];
    double projv = dot3(dvel, drdrag);
    double projvstar = projv;
    double wab, ts;
    const double Kd = s->o.Kdrag;
    if (c->itypei == NDSPH_ITYPE_GAS || c->itypei == NDSPH_ITYPE_BND) {
        double cs = s->spsound[i];
        wab = wabi;
        ts = rhoj * c->rhoi / (Kd * (c->rhoi + rhoj));
        double r = c->hi / (cs * ts);
        if (r > c->h_on_csts_max) c->h_on_csts_max = r;
    } else {
        if (itypej != NDSPH_ITYPE_GAS && itypej != NDSPH_ITYPE_BND) return;
        double cs = s->spsound[j];
        wab = wabj;
        ts = c->rhoi * rhoj / (Kd * (rhoj + c->rhoi));
        double r = s->hh[j] / (cs * ts);
        if (r > c->h_on_csts_max) c->h_on_csts_max = r;
    }
    if (ts < c->ts_min) c->ts_min = ts;
    double dragterm = nd * wab / ((c->rhoi + rhoj) * ts) * projvstar;
    double dragterm_en = dragterm * projv;
    for (int d = 0; d < 3; d++) {
        c->forcei[d] = c->forcei[d] - dragterm * pmassj * drdrag[d];
        s->force[j * 3 + d] = s->force[j * 3 + d] + dragterm * c->pmassi * drdrag[d];
    }
    if (c->itypei == NDSPH_ITYPE_GAS) s->dudt[i] = s->dudt[i] + pmassj * dragterm_en;
    if (itypej == NDSPH_ITYPE_GAS) s->dudt[j] = s->dudt[j] + c->pmassi * dragterm_en;
}

static int get_rates(orc_sim* s)
{
    const int nd = s->ndim, np = s->npart, nt = s->ntotal;
    const orc_kernels* K = &s->K;
    rates_ctx c;
    memset(&c, 0, sizeof c);
    c.dtcourant = 1.e6;
    c.dtav = DBL_MAX;
    s->dtvisc = DBL_MAX;
    c.ts_min = DBL_MAX;
    c.h_on_csts_max = 0.;
    c.vsigmax = 0.;
    for (int i = 0; i < nt; i++) {
        for (int d = 0; d < 3; d++) {
            s->force[i * 3 + d] = 0.; s->dBevoldt[i * 3 + d] = 0.; s->daldt[i * 3 + d] = 0.;
            if (s->o.imhd > 0) s->curlB[i * 3 + d] = 0.;
            s->graddivv[i * 3 + d] = 0.;
        }
        s->dudt[i] = 0.; s->dendt[i] = 0.; s->divB[i] = 0.; s->del2u[i] = 0.;
    }
    double stressmax = 0.;
    if (s->o.imhd != 0 && (s->o.imagforce == 2 || s->o.imagforce == 7)) {
        for (int i = 0; i < nt; i++) {
            double B2i = dot3(&s->Bfield[i * 3], &s->Bfield[i * 3]);
            double st = fmax(0.5 * B2i - s->pr[i], 0.);
            if (st > stressmax) stressmax = st;
            if (0.0 > stressmax) stressmax = 0.0;        /* maxval(Bconst) = 0 */
        }
    }
    c.stressmax = stressmax;
    s->stressmax = stressmax;
    double* h1 = malloc(sizeof(double) * (size_t)nt);
    for (int i = 0; i < nt; i++) h1[i] = 1. / s->hh[i];
    for (int icell = 0; icell < s->ncells && !s->err; icell++) {
        int nneigh = get_neighbour_list(s, icell, s->listneigh);
        int idone = -1;
        for (int i = s->ifirstincell[icell]; i >= 0 && !s->err; i = s->ll[i]) {
            idone++;
            c.i = i;
            c.itypei = s->itype[i];
            c.rhoi = s->rho[i];
            c.rho2i = c.rhoi * c.rhoi;
            c.rho1i = 1. / c.rhoi;
            c.rho21i = c.rho1i * c.rho1i;
            c.pri = fmax(s->pr[i] - 0.0, 0.);
            c.prneti = c.pri;
            c.pmassi = s->pmass[i];
            c.Prho2i = c.pri * c.rho21i;
            c.spsoundi = s->spsound[i];
            c.uui = s->uu[i];
            for (int d = 0; d < 3; d++) c.veli[d] = s->vel[i * 3 + d];
            c.alphai = s->alpha[i * 3 + 0];
            c.alphaui = s->alpha[i * 3 + 1];
            c.alphaBi = s->alpha[i * 3 + 2];
            if (s->o.imhd != 0) {
                for (int d = 0; d < 3; d++) { c.Bi[d] = s->Bfield[i * 3 + d]; c.Brhoi[d] = c.Bi[d] * c.rho1i; }
                c.B2i = dot3(c.Bi, c.Bi);
                c.Brho2i = c.B2i * c.rho21i;
                c.valfven2i = c.B2i * c.rho1i;
            } else {
                memset(c.Bi, 0, sizeof c.Bi); memset(c.Brhoi, 0, sizeof c.Brhoi);
                c.B2i = 0; c.Brho2i = 0; c.valfven2i = 0;
            }
            c.gradhi = s->gradh[i];
            c.hi = s->hh[i];
            if (c.hi <= 0.) { s->err = NDSPH_E_H_NONPOS; break; }
            c.hi1 = h1[i];
            c.hi21 = c.hi1 * c.hi1;
            c.hfacwabi = powi_f(c.hi1, nd);
            c.hfacgrkerni = c.hfacwabi * c.hi1;
            memset(c.forcei, 0, sizeof c.forcei);
            memset(c.dBevoldti, 0, sizeof c.dBevoldti);
            for (int n = idone; n < nneigh; n++) {
                int j = s->listneigh[n];
                if (j == i || (j >= np && i >= np)) continue;
                c.j = j;
                for (int d = 0; d < 3; d++) c.dx[d] = 0.;
                for (int d = 0; d < nd; d++) c.dx[d] = s->x[i * nd + d] - s->x[j * nd + d];
                double hj1 = h1[j];
                double hj21 = hj1 * hj1;
                c.rij2 = dotn(c.dx, c.dx, nd);
                c.q2i = c.rij2 * c.hi21;
                c.q2j = c.rij2 * hj21;
                if (!(c.q2i < K->radkern2 || c.q2j < K->radkern2)) continue;
                c.rij = sqrt(c.rij2);
                if (c.rij <= DBL_EPSILON && s->itype[j] == c.itypei) {
                    if (c.rij < DBL_MIN) {
                        c.dr[0] = c.dr[1] = c.dr[2] = 0.;
                        if (c.itypei != 2) {
                            s->err = NDSPH_E_CLUMP;
                            snprintf(s->msg, sizeof s->msg, "rates: dx = 0 i,j = %d %d", i + 1, j + 1);
                            break;
                        }
                    }
                } else if (c.rij <= DBL_EPSILON) {
                    c.dr[0] = c.dr[1] = c.dr[2] = 0.;
                } else {
                    c.dr[0] = c.dr[1] = c.dr[2] = 0.;
                    for (int d = 0; d < nd; d++) c.dr[d] = c.dx[d] / c.rij;
                }
                int itypej = s->itype[j];
                if (type_match(c.itypei, itypej)) {
                    if (rates_core(s, &c)) break;
                } else if (s->o.idust == 2 && s->o.idrag_nature > 0) {
                    drag_forces(s, &c);
                }
            }
            for (int d = 0; d < 3; d++) {
                s->force[i * 3 + d] = s->force[i * 3 + d] + 0. + c.forcei[d];
                s->dBevoldt[i * 3 + d] = s->dBevoldt[i * 3 + d] + c.dBevoldti[d];
            }
        }
    }
    free(h1);
    if (s->err) return s->err;
    s->dtcourant = c.dtcourant;
    s->dtav = c.dtav;
    s->vsigmax = c.vsigmax;

    /* per-particle post pass :532-924 */
    double fhmax = 0.0;
    s->dtdrag = DBL_MAX;
    s->dtforce = DBL_MAX;
    for (int i = 0; i < np; i++) {
        double rhoi = s->rho[i];
        double rho1i = 1. / rhoi;
        if (s->o.idust == 2 && s->o.idrag_nature != 0 && (s->o.Kdrag > 0. || s->o.idrag_nature > 1)) {
            if (c.ts_min < s->dtdrag) s->dtdrag = c.ts_min;
        }
        if (s->o.imhd != 0) {
            if (s->o.imhd > 0)
                for (int d = 0; d < 3; d++) s->curlB[i * 3 + d] = s->curlB[i * 3 + d] * rho1i;
            s->divB[i] = s->divB[i] * rho1i;
        }
        double forcemag = sqrt(dot3(&s->force[i * 3], &s->force[i * 3]));
        double fonh = forcemag / s->hh[i];
        if (fonh > fhmax && s->itype[i] != 1) fhmax = fonh;
        double valfven2i = 0.;
        if (s->o.imhd != 0) valfven2i = dot3(&s->Bfield[i * 3], &s->Bfield[i * 3]) / s->dens[i];
        double vsig2 = s->spsound[i] * s->spsound[i] + valfven2i;
        double vsig = sqrt(vsig2);
        if (s->o.imhd >= 11 && s->o.imhd <= 19) {
            for (int d = 0; d < 3; d++)
                s->dBevoldt[i * 3 + d] = 1. * s->dBevoldt[i * 3 + d] + s->Bevol[i * 3 + d] * rho1i * s->drhodt[i];
        } else if (s->o.imhd >= 1 && s->o.imhd <= 9) {
            for (int d = 0; d < 3; d++) s->dBevoldt[i * 3 + d] = 1. * s->dBevoldt[i * 3 + d] * rho1i;
        } else {
            for (int d = 0; d < 3; d++) s->dBevoldt[i * 3 + d] = 0.;
        }
        if (s->o.iener > 0 && s->o.iav >= 0 && s->o.iener != 3 && s->o.iener != 10 && s->o.iener != 11) {
            s->dudt[i] = s->dudt[i] + s->pr[i] * powi_f(rho1i, 2) * s->drhodt[i];
            s->dendt[i] = s->dudt[i];
        } else {
            s->dendt[i] = s->dudt[i];
        }
        if (s->itype[i] == NDSPH_ITYPE_DUST) s->dendt[i] = 0.;
        for (int d = 0; d < 3; d++) s->daldt[i * 3 + d] = 0.;
        if (s->o.iavlim[0] != 0 || s->o.iavlim[1] != 0 || s->o.iavlim[2] != 0) {
            double tdecay1 = (s->o.avdecayconst * vsig) / s->hh[i];
            if (s->o.iavlim[0] == 1 || s->o.iavlim[0] == 2) {
                double source = fmax(s->drhodt[i] * rho1i, 0.0);
                if (s->o.iavlim[0] == 2) source = source * (2.0 - s->alpha[i * 3 + 0]);
                s->daldt[i * 3 + 0] = (s->o.alphamin - s->alpha[i * 3 + 0]) * tdecay1 + s->avfact * source;
            }
            if (s->o.iener > 0 && s->o.iavlim[1] > 0) {
                double sourceu = 0.;
                if (s->uu[i] > DBL_EPSILON) sourceu = s->hh[i] * fabs(s->del2u[i]) / sqrt(s->uu[i]);
                s->daldt[i * 3 + 1] = (s->o.alphaumin - s->alpha[i * 3 + 1]) * tdecay1 + sourceu;
            }
        }
    }
    if (c.h_on_csts_max > 0.) { /* diagnostic only */ }
    if (fhmax < 0.) { s->err = NDSPH_E_NAN; return s->err; }
    if (fhmax > 0.) { double t = sqrt(1. / fhmax); if (t < s->dtforce) s->dtforce = t; }
    for (int i = 0; i < nt; i++) {
        if (s->itype[i] == NDSPH_ITYPE_BND || s->itype[i] == NDSPH_ITYPE_BNDDUST || i >= np) {
            for (int d = 0; d < 3; d++) {
                s->force[i * 3 + d] = 0.; s->dBevoldt[i * 3 + d] = 0.; s->daldt[i * 3 + d] = 0.;
                if (s->o.imhd >= 0) s->curlB[i * 3 + d] = 0.;
            }
            s->drhodt[i] = 0.; s->dhdt[i] = 0.; s->dudt[i] = 0.; s->dendt[i] = 0.; s->divB[i] = 0.;
        }
    }
    return 0;
}

/* boundary boundaryND.f90:30-164 (periodic wrap; fixed particles untouched) */
static void boundary(orc_sim* s)
{
    const int nd = s->ndim;
    for (int i = 0; i < s->npart; i++) {
        for (int d = 0; d < nd; d++) {
            if (s->o.ibound[d] != 3) continue;
            double* xp = &s->x[i * nd + d];
            if (*xp > s->o.xmax[d]) *xp = s->o.xmin[d] + *xp - s->o.xmax[d];
            else if (*xp < s->o.xmin[d]) *xp = s->o.xmax[d] - (s->o.xmin[d] - *xp);
        }
    }
}

/* derivs derivs.f90:27-287 (in-scope path) */
static int derivs(orc_sim* s)
{
    int anyb = 0;
    for (int d = 0; d < s->ndim; d++) if (s->o.ibound[d] != 0) anyb = 1;
    if (anyb) boundary(s);
    if (any_ibound_gt1(s)) set_ghost_particles(s);
    else s->ntotal = s->npart;
    if (set_linklist(s)) return s->err;
    if (iterate_density(s)) return s->err;
    conservative2primitive(s);
    if (s->err) return s->err;
    if (get_rates(s)) return s->err;
    return 0;
}

/* step stepND_leapfrog_mhd.f90:31-275 */
static int step(orc_sim* s)
{
    const int nd = s->ndim, np = s->npart;
    double dt = s->dt, hdt = 0.5 * dt;
    for (int i = 0; i < np; i++) {
        for (int d = 0; d < nd; d++) s->xin[i * nd + d] = s->x[i * nd + d];
        for (int d = 0; d < 3; d++) {
            s->velin[i * 3 + d] = s->vel[i * 3 + d];
            s->Bevolin[i * 3 + d] = s->Bevol[i * 3 + d];
            s->alphain[i * 3 + d] = s->alpha[i * 3 + d];
            s->forcein[i * 3 + d] = s->force[i * 3 + d];
            s->dBevoldtin[i * 3 + d] = s->dBevoldt[i * 3 + d];
            s->daldtin[i * 3 + d] = s->daldt[i * 3 + d];
        }
        s->hhin[i] = s->hh[i];
        s->enin[i] = s->en[i];
        s->dhdtin[i] = s->dhdt[i];
        s->dendtin[i] = s->dendt[i];
    }
    double* rhoin = malloc(sizeof(double) * (size_t)(np > 0 ? np : 1));
    for (int i = 0; i < np; i++) rhoin[i] = s->rho[i];
    int fixed_any = 0;
    for (int i = 0; i < np; i++) {
        int t = s->itype[i];
        if (t == NDSPH_ITYPE_BND || t == NDSPH_ITYPE_BNDDUST) {
            int j = s->ireal[i];
            int src = (j >= 0) ? j : i;
            for (int d = 0; d < nd; d++)
                s->x[i * nd + d] = s->xin[i * nd + d] + dt * s->velin[src * 3 + d] + 0.5 * dt * dt * s->forcein[src * 3 + d];
            for (int d = 0; d < 3; d++) s->Bevol[i * 3 + d] = s->Bevolin[i * 3 + d];
            s->rho[i] = rhoin[i];
            s->hh[i] = s->hhin[i];
            s->en[i] = s->enin[i];
            for (int d = 0; d < 3; d++) s->alpha[i * 3 + d] = s->alphain[i * 3 + d];
        } else {
            for (int d = 0; d < nd; d++)
                s->x[i * nd + d] = s->xin[i * nd + d] + dt * s->velin[i * 3 + d] + 0.5 * dt * dt * s->forcein[i * 3 + d];
            for (int d = 0; d < 3; d++) s->vel[i * 3 + d] = (s->velin[i * 3 + d] + dt * s->forcein[i * 3 + d]) / (1. + 0.);
            if (s->o.imhd != 0)
                for (int d = 0; d < 3; d++) s->Bevol[i * 3 + d] = s->Bevolin[i * 3 + d] + dt * s->dBevoldtin[i * 3 + d];
            s->hh[i] = s->hhin[i] + dt * s->dhdtin[i];
            if (s->o.iener != 0) s->en[i] = s->enin[i] + dt * s->dendtin[i];
            for (int d = 0; d < 3; d++)
                if (s->o.iavlim[d] != 0) s->alpha[i * 3 + d] = fmin(s->alphain[i * 3 + d] + dt * s->daldtin[i * 3 + d], 1.0);
        }
    }
    (void)fixed_any;
    if (derivs(s)) { free(rhoin); return s->err; }
    for (int i = 0; i < np; i++) {
        int t = s->itype[i];
        if (t == NDSPH_ITYPE_BND || t == NDSPH_ITYPE_BNDDUST) {
            for (int d = 0; d < 3; d++) s->vel[i * 3 + d] = s->velin[i * 3 + d];
            for (int d = 0; d < 3; d++) s->Bevol[i * 3 + d] = s->Bevolin[i * 3 + d];
            s->hh[i] = s->hhin[i];
            s->en[i] = s->enin[i];
            for (int d = 0; d < 3; d++) s->alpha[i * 3 + d] = s->alphain[i * 3 + d];
            s->rho[i] = rhoin[i];
        } else {
            for (int d = 0; d < 3; d++)
                s->vel[i * 3 + d] = (s->velin[i * 3 + d] + hdt * (s->force[i * 3 + d] + s->forcein[i * 3 + d])) / (1. + 0.);
            if (s->o.imhd != 0)
                for (int d = 0; d < 3; d++)
                    s->Bevol[i * 3 + d] = s->Bevolin[i * 3 + d] + hdt * (s->dBevoldt[i * 3 + d] + s->dBevoldtin[i * 3 + d]);
            s->hh[i] = s->hhin[i] + hdt * (s->dhdt[i] + s->dhdtin[i]);
            if (s->hh[i] <= 0.) { s->err = NDSPH_E_H_NONPOS; snprintf(s->msg, sizeof s->msg, "step: hh -ve"); free(rhoin); return s->err; }
            if (s->o.iener != 0) s->en[i] = s->enin[i] + hdt * (s->dendt[i] + s->dendtin[i]);
            for (int d = 0; d < 3; d++)
                if (s->o.iavlim[d] != 0)
                    s->alpha[i * 3 + d] = fmin(s->alphain[i * 3 + d] + hdt * (s->daldt[i * 3 + d] + s->daldtin[i * 3 + d]), 1.0);
        }
    }
    free(rhoin);
    int anyb = 0;
    for (int d = 0; d < nd; d++) if (s->o.ibound[d] != 0) anyb = 1;
    if (anyb) boundary(s);
    double dtn = s->o.C_force * s->dtforce;
    double t;
    t = s->o.C_cour * s->dtcourant; if (t < dtn) dtn = t;
    t = 0.9 * s->dtdrag; if (t < dtn) dtn = t;
    t = s->o.C_force * s->dtvisc; if (t < dtn) dtn = t;
    s->time += s->dt;
    s->dt = dtn;
    s->nsteps++;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* exported oracle API (ctypes)                                               */
/* ------------------------------------------------------------------------- */
void* orc_create(const ndsph_opts* o, int npart)
{
    orc_sim* s = calloc(1, sizeof(orc_sim));
    s->o = *o;
    s->ndim = o->ndim;
    s->npart = npart;
    s->ntotal = npart;
    s->cap = 0;
    sim_alloc(s, npart + 16);
    orc_setkern_tables(&s->K, s->ndim);
    if (fabs(o->gamma - 1.) > 1.e-3) s->avfact = log(4.) / (log((o->gamma + 1.) / (o->gamma - 1.)));
    else s->avfact = 1.0;
    int np = npart > 0 ? npart : 1;
    NCALLOC(s->xin, np * s->ndim); NCALLOC(s->velin, np * 3); NCALLOC(s->Bevolin, np * 3);
    NCALLOC(s->hhin, np); NCALLOC(s->enin, np); NCALLOC(s->alphain, np * 3);
    NCALLOC(s->forcein, np * 3); NCALLOC(s->dBevoldtin, np * 3); NCALLOC(s->dhdtin, np);
    NCALLOC(s->dendtin, np); NCALLOC(s->daldtin, np * 3);
    for (int i = 0; i < s->cap; i++) s->ireal[i] = -1;
    return s;
}

void orc_destroy(void* h)
{
    orc_sim* s = h;
    if (!s) return;
    void* ptrs[] = {s->x, s->vel, s->Bevol, s->Bfield, s->en, s->uu, s->hh, s->pmass, s->rho, s->rhoalt,
                    s->dens, s->pr, s->spsound, s->alpha, s->psi, s->itype, s->ireal, s->gradh, s->gradhn,
                    s->gradsoft, s->gradgradh, s->drhodt, s->dhdt, s->force, s->dBevoldt, s->dudt, s->dendt,
                    s->daldt, s->divB, s->curlB, s->del2u, s->graddivv, s->ll, s->iamincell, s->numneigh,
                    s->ifirstincell, s->listneigh, s->xin, s->velin, s->Bevolin, s->hhin, s->enin, s->alphain,
                    s->forcein, s->dBevoldtin, s->dhdtin, s->dendtin, s->daldtin};
    for (size_t k = 0; k < sizeof ptrs / sizeof ptrs[0]; k++) free(ptrs[k]);
    free(s);
}

const char* orc_message(void* h) { return ((orc_sim*)h)->msg; }

/* copy a full particle state in (inputs and previous-step rates) */
void orc_set_state(void* h, const ndsph_particles* p)
{
    orc_sim* s = h;
    int n = s->npart, nd = s->ndim;
#define IN(field, stride) do { if (p->field) memcpy(s->field, p->field, sizeof(*s->field) * (size_t)n * (stride)); } while (0)
    IN(x, nd); IN(vel, 3); IN(Bevol, 3); IN(en, 1); IN(hh, 1); IN(pmass, 1); IN(alpha, 3); IN(itype, 1);
    IN(rho, 1); IN(rhoalt, 1); IN(drhodt, 1); IN(dhdt, 1); IN(gradh, 1); IN(gradhn, 1); IN(gradgradh, 1);
    IN(dens, 1); IN(uu, 1); IN(pr, 1); IN(spsound, 1); IN(Bfield, 3); IN(force, 3); IN(dBevoldt, 3);
    IN(dudt, 1); IN(dendt, 1); IN(daldt, 3); IN(divB, 1); IN(curlB, 3); IN(del2u, 1); IN(graddivv, 3);
#undef IN
    if (p->ireal) for (int i = 0; i < n; i++) s->ireal[i] = p->ireal[i] - 1;   /* 1-based in */
    if (p->numneigh) memcpy(s->numneigh, p->numneigh, sizeof(int) * (size_t)n);
}

void orc_get_state(void* h, ndsph_particles* p)
{
    orc_sim* s = h;
    int n = s->npart, nd = s->ndim;
#define OUT(field, stride) do { if (p->field) memcpy(p->field, s->field, sizeof(*s->field) * (size_t)n * (stride)); } while (0)
    OUT(x, nd); OUT(vel, 3); OUT(Bevol, 3); OUT(en, 1); OUT(hh, 1); OUT(pmass, 1); OUT(alpha, 3); OUT(itype, 1);
    OUT(rho, 1); OUT(rhoalt, 1); OUT(drhodt, 1); OUT(dhdt, 1); OUT(gradh, 1); OUT(gradhn, 1); OUT(gradgradh, 1);
    OUT(numneigh, 1); OUT(dens, 1); OUT(uu, 1); OUT(pr, 1); OUT(spsound, 1); OUT(Bfield, 3); OUT(force, 3);
    OUT(dBevoldt, 3); OUT(dudt, 1); OUT(dendt, 1); OUT(daldt, 3); OUT(divB, 1); OUT(curlB, 3); OUT(del2u, 1);
    OUT(graddivv, 3);
#undef OUT
    if (p->ireal) for (int i = 0; i < n; i++) p->ireal[i] = s->ireal[i] + 1;
}

void orc_get_dt(void* h, ndsph_dt* d)
{
    orc_sim* s = h;
    d->dtcourant = s->dtcourant; d->dtforce = s->dtforce; d->dtav = s->dtav; d->dtdrag = s->dtdrag;
    d->dtvisc = s->dtvisc; d->vsigmax = s->vsigmax; d->stressmax = s->stressmax; d->hhmax = s->hhmax;
    d->dt = s->dt; d->time = s->time; d->its = s->itsdensity; d->ncalctotal = s->ncalctotal;
    d->nsteps = s->nsteps; d->nrelink = s->nrelink;
}

void orc_set_dt(void* h, double dt, double time)
{
    orc_sim* s = h;
    s->dt = dt; s->time = time;
}

int orc_derivs(void* h) { orc_sim* s = h; s->err = 0; return derivs(s); }

int orc_step(void* h, int nsteps)
{
    orc_sim* s = h;
    s->err = 0;
    for (int k = 0; k < nsteps; k++) if (step(s)) return s->err;
    return 0;
}

/* link + density iteration only (boundary, ghosts, set_linklist, iterate_density) */
int orc_iterate_density(void* h)
{
    orc_sim* s = h;
    s->err = 0;
    int anyb = 0;
    for (int d = 0; d < s->ndim; d++) if (s->o.ibound[d] != 0) anyb = 1;
    if (anyb) boundary(s);
    if (any_ibound_gt1(s)) set_ghost_particles(s); else s->ntotal = s->npart;
    if (set_linklist(s)) return s->err;
    return iterate_density(s);
}

/* cons2prim + get_rates on the current state (ghosts rebuilt first) */
int orc_get_rates(void* h)
{
    orc_sim* s = h;
    s->err = 0;
    if (any_ibound_gt1(s)) {
        set_ghost_particles(s);
    } else {
        s->ntotal = s->npart;
    }
    if (set_linklist(s)) return s->err;
    conservative2primitive(s);
    if (s->err) return s->err;
    return get_rates(s);
}

/* primitive2conservative conservative2primitive.f90:478-799 (in-scope) */
int orc_primitive2conservative(void* h)
{
    orc_sim* s = h;
    s->err = 0;
    const int nd = s->ndim, np = s->npart;
    for (int i = 0; i < np; i++) {
        s->rho[i] = s->dens[i];
        s->hh[i] = s->o.hfact * pow(s->pmass[i] / (s->rho[i] + 0.0), 1.0 / nd);
    }
    if (s->o.iener == 0) {
        for (int i = 0; i < np; i++) {
            if (s->itype[i] != NDSPH_ITYPE_GAS) continue;
            double gam1 = s->o.gamma - 1.;
            double polyki = (s->o.gamma <= 1.0001) ? 2. / 3. * s->uu[i] : gam1 * s->uu[i] / pow(s->dens[i], gam1);
            s->o.polyk = polyki;
            break;
        }
    }
    if (any_ibound_gt1(s)) set_ghost_particles(s); else s->ntotal = s->npart;
    if (set_linklist(s)) return s->err;
    if (iterate_density(s)) return s->err;
    for (int i = 0; i < s->cap; i++) s->dens[i] = s->rho[i];
    if (s->o.imhd >= 11) {
        for (int i = 0; i < 3 * s->cap; i++) s->Bevol[i] = s->Bfield[i];
    } else if (s->o.imhd >= 1 && s->o.imhd <= 9) {
        for (int i = 0; i < np; i++) for (int d = 0; d < 3; d++) s->Bevol[i * 3 + d] = s->Bfield[i * 3 + d] / s->rho[i];
    }
    for (int i = 0; i < s->cap; i++) s->en[i] = s->uu[i];
    return derivs(s);
}

double orc_polyk(void* h) { return ((orc_sim*)h)->o.polyk; }

/* kernel tables for the table test: wij, grwij, grgrwij, wijdrag, grwijdrag */
void orc_kernel_tables(int ndim, double* out)
{
    orc_kernels K;
    orc_setkern_tables(&K, ndim);
    memcpy(out + 0 * (IKERN + 1), K.wij, sizeof K.wij);
    memcpy(out + 1 * (IKERN + 1), K.grwij, sizeof K.grwij);
    memcpy(out + 2 * (IKERN + 1), K.grgrwij, sizeof K.grgrwij);
    memcpy(out + 3 * (IKERN + 1), K.wijdrag, sizeof K.wijdrag);
    memcpy(out + 4 * (IKERN + 1), K.grwijdrag, sizeof K.grwijdrag);
}

/* kernel value by table interpolation (W, dW/dq in q^2), for tests */
void orc_interp(int ndim, int n, const double* q2, double* w, double* gw)
{
    orc_kernels K;
    orc_setkern_tables(&K, ndim);
    for (int k = 0; k < n; k++) {
        double a, b, c, d, e;
        interp_dens(&K, q2[k], &a, &b, &c, &d, &e);
        w[k] = a; gw[k] = b;
    }
}

/* Neighbour sets of the oracle's link list, the way check_neighbourlist.f90
 * builds its reference: for each real particle, the real indices (1-based) of
 * every image within 2h_i (mode 0) or within 2h_i or 2h_j (mode 1).
 * Call after orc_iterate_density/orc_derivs (h and ghosts current).
 * Returns the number of entries written (or -needed if cap is too small).     */
long orc_neighbour_csr(void* h, int mode, long* offsets, int* neigh, long cap)
{
    orc_sim* s = h;
    const int nd = s->ndim, np = s->npart;
    if (any_ibound_gt1(s)) set_ghost_particles(s); else s->ntotal = s->npart;
    set_linklist(s);
    long total = 0;
    int* list = s->listneigh;
    for (int i = 0; i < np; i++) {
        offsets[i] = total;
        int nn = get_neighbour_list_partial(s, s->iamincell[i], list);
        double hi1 = 1. / s->hh[i];
        double hi21 = hi1 * hi1;
        for (int n = 0; n < nn; n++) {
            int j = list[n];
            if (j == i) continue;
            if (!type_match(s->itype[i], s->itype[j])) continue;
            double dx[MAXNDIM];
            for (int d = 0; d < nd; d++) dx[d] = s->x[i * nd + d] - s->x[j * nd + d];
            double rij2 = dotn(dx, dx, nd);
            double hj1 = 1. / s->hh[j];
            double q2i = rij2 * hi21;
            double q2j = rij2 * (hj1 * hj1);
            int ok = (mode == 0) ? (q2i < 4.0) : (q2i < 4.0 || q2j < 4.0);
            if (ok) {
                if (total < cap) neigh[total] = (j < np ? j : s->ireal[j]) + 1;
                total++;
            }
        }
    }
    offsets[np] = total;
    return total <= cap ? total : -total;
}
