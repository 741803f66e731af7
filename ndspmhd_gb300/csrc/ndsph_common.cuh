// ndsph_common.cuh -- device-side types shared by the hot-path kernels.
//
// Layout in HBM: one structure-of-arrays per particle field, in cell-sorted
// order (particles of one cell are contiguous, cells in row-major key order).
// Every per-particle double field lives in one slab `F` of NF*cap doubles so
// the cell sort can permute all live fields with one gather kernel.
#pragma once
#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>
#include "../../include/ndsph.h"

// Host-side count of every kernel launch this library issues (all contexts);
// ndsph_get_timing reports the launches of the last ndsph_dev_step call.
inline std::atomic<long long>& ndsph_launch_counter()
{
    static std::atomic<long long> c{0};
    return c;
}
#define NDSPH_COUNT_LAUNCH (void)ndsph_launch_counter().fetch_add(1, std::memory_order_relaxed)

namespace ndsph {

// sets the message ndsph_last_error(NULL) returns (the calling thread's)
void set_global_error(const char* msg);

constexpr int IKERN = 4000;            // kernelND.f90:37
constexpr int NTAB = IKERN + 1;

// double fields of the device slab
enum Field : int {
    X0, X1, X2, V0, V1, V2, BE0, BE1, BE2, EN, HH, PM, AL0, AL1, AL2,
    RHO, RHOALT, DRHODT, DHDT, GRADH, GRADHN, GRADGRADH,
    DENS, UU, PR, CS, BF0, BF1, BF2,
    F0, F1, F2, DB0, DB1, DB2, DUDT, DENDT, DAL0, DAL1, DAL2, DIVB, CB0, CB1, CB2, DEL2U,
    GDV0, GDV1, GDV2,
    // leapfrog saves (part_in module, stepND_leapfrog_mhd.f90:70-101)
    XIN0, XIN1, XIN2, VIN0, VIN1, VIN2, BIN0, BIN1, BIN2, HIN, ENIN, RHOIN, ALIN0, ALIN1, ALIN2,
    FIN0, FIN1, FIN2, DBIN0, DBIN1, DBIN2, DHIN, DENIN, DALIN0, DALIN1, DALIN2,
    // learned-h predictor: h_pred, and the six FP32 features packed two to
    // a field (bit patterns: the permutation gather moves 8-byte words)
    HPRED, FT0, FT1, FT2,
    HDEN0,      // h at entry of iterate_density (hhin, iterate_density.f90:87)
    HNEXT,      // NR scratch: next h of the first pass
    RHO1,       // 1/rho of the FP64 rates sweep (written with the EOS)
    HROOT,      // learned h: the Newton-Raphson estimate of the root at convergence
    NF
};

// options + derived constants, passed by value to kernels
struct DevOpts {
    int ndim;
    int ibound[3];
    int periodic[3];
    double xmin[3], xmax[3], L[3];
    double hfact, tolh, psep;
    int maxdensits;
    int imhd, imagforce, iener, iav, iavlim[3];
    double alphamin, alphaumin, alphaBmin, beta, avdecayconst, avfact;
    double gamma, polyk;
    int idust, idrag_nature;
    double Kdrag;
    double C_cour, C_force;
    int precision;
    int has_fixed;      // any ibound == 1 (fixed particles with ireal copies)
    int learned;        // learned-h predictor on: the density passes keep HROOT
    // batched form: nsim independent simulations in one state
    int batched;
    int nsim;
    unsigned long long* sim_red;   // [nsim][SIMRED] per-simulation reductions
    double* sim_dt;                // [nsim] dt of the current step
    unsigned long long* sim_aux;   // [nsim][SIMAUX] per-simulation drag constant and ghost hhmax
    int stacked;                   // periodic batch: one cell grid per simulation, stacked
};
// per-simulation reduction slots (batched form)
enum SimRed : int { SR_DTC = 0, SR_DTAV, SR_VSIG, SR_TS, SR_FH, SR_STRESS, SIMRED = 8 };
// per-simulation settings and link state (batched form, bit patterns of
// doubles): the drag constant K (dust.f90:91), the ghosts' hhmax of the
// simulation's last (re)link, the scratch max h of a relink, the relink
// request of its last Newton-Raphson pass (iterate_density.f90:122-126), and
// the full-pass rule of a run (iterate_density.f90:129-133: a pass is full
// while every particle of the run is unconverged): SA_FULL whether the
// simulation's next pass is full, SA_CONV whether a particle of it
// converged (or is fixed) in the current pass
enum SimAux : int { SA_KDRAG = 0, SA_HG, SA_HNOW, SA_RELINK, SA_FULL, SA_CONV, SIMAUX = 8 };

// cell grid (periodic dims wrap, the others are padded bounding boxes)
struct Grid {
    int nc[3];          // cells per dim (1 for unused dims)
    int ncells;
    // a periodic batch stacks one grid of ncs cells per simulation:
    // cell = sim * ncs + local cell (nstack = 1: one simulation)
    int ncs = 0;
    int nstack = 1;
    double origin[3];   // lower corner
    double cs[3];       // cell size per dim (>= 2 hmax / reach)
    double inv_cs[3];
    float csf[3];
    // search stencil: sw = 3 (cells of >= 2 hmax, reach 1) or 5 (cells of
    // >= hmax, reach 2); a neighbour-row entry packs (j << nlshift) | offset,
    // offset = (dx+r) + sw (dy+r) + sw^2 (dz+r), r = (sw-1)/2
    int sw = 3;
    int nlshift = 5;
};

// coordinates of cell c within its simulation's grid and the id of that
// grid's first cell
__host__ __device__ inline void cell_coords(int c, const Grid& g, int cc[3], int* base = nullptr)
{
    int b = 0;
    if (g.nstack > 1) {
        b = (c / g.ncs) * g.ncs;
        c -= b;
    }
    cc[0] = c % g.nc[0];
    cc[1] = (c / g.nc[0]) % g.nc[1];
    cc[2] = c / (g.nc[0] * g.nc[1]);
    if (base) *base = b;
}

// kernel tables: value and slope per entry, slope(i) = (t(i+1)-t(i))*ddq2table
// exactly as interpolate_kernel* form it (kernelND.f90:4382-4391)
struct Tables {
    const double2* w;       // W(q2)
    const double2* gw;      // dW/dq
    const double2* ggw;     // d2W/dq2
    const double2* wdrag;   // double-hump drag kernel
    const float2* wf;       // FP32 copies for the FP32 form
    const float2* gwf;
    const float2* ggwf;
    const float2* wdragf;
    double dq2table, ddq2table;
    float dq2tablef, ddq2tablef;
    float cnormf;           // W(0): the kernel's normalisation (FP32 form's analytic kernel)
};

// global reductions written by the sweeps (int64 bit patterns of
// non-negative doubles so integer atomics order them)
struct Reduce {
    unsigned long long dtcourant;   // min
    unsigned long long dtav;        // min
    unsigned long long vsigmax;     // max
    unsigned long long ts_min;      // min
    unsigned long long fhmax;       // max
    unsigned long long stressmax;   // max
    unsigned long long hmax;        // max
    unsigned long long hmax_ghost;  // max h of the last (re)link
    int ncalc;                      // unconverged count of the current pass
    int redolink;                   // NR asked for a relink
    int err;                        // first error code raised on the device
    int err_index;
    int nclumped;
    int pad;
    unsigned long long pairs;       // accepted pairs (diagnostic)
    double dt, time;                // leapfrog dt/time (device-resident form)
    unsigned long long xlo[3];      // order-preserving bits of min x (bounding box)
    unsigned long long xhi[3];      // order-preserving bits of max x
    double h_on_csts_max;
    int nl_stale;                   // some h outgrew the neighbour-list skin
    int nl_overflow;                // some particle had more candidates than the list stride
    int nl_maxcnt;                  // largest list length of the last build
    int pad2;
    // control words of the captured (CUDA graph) step
    int gfail;                      // the captured step met a case it leaves to the host path
    int g_its;                      // Newton-Raphson pass number
    int g_nlist;                    // active entries of the next partial pass
    int g_gate;                     // relink check of this pass (redolink of the previous pass)
    int g_rebuild;                  // rebuild the neighbour rows after this pass
    int g_pad;
    // neighbour-row reuse check of a step that skips the link
    unsigned reuse_d2;              // max squared displacement since the build (float bits)
    unsigned reuse_slack;           // min of skin*h_build - grow*h (order-preserving float bits)
    int sim_any_full;               // batched: some simulation's next pass is full
    int sim_pad;
};

__host__ __device__ inline unsigned long long dbits(double v)
{
#ifdef __CUDA_ARCH__
    return (unsigned long long)__double_as_longlong(v);
#else
    union { double d; unsigned long long u; } c; c.d = v; return c.u;
#endif
}
__host__ __device__ inline double bitsd(unsigned long long u)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    union { double d; unsigned long long u; } c; c.u = u; return c.d;
#endif
}

__host__ __device__ inline double unord_bits(unsigned long long u)
{
    u = (u & 0x8000000000000000ull) ? (u & ~0x8000000000000000ull) : ~u;
    return bitsd(u);
}

#ifdef __CUDACC__
__device__ inline void atomic_min_pos(unsigned long long* a, double v)
{
    if (v >= 0.0) atomicMin(a, dbits(v));
}
__device__ inline void atomic_max_pos(unsigned long long* a, double v)
{
    if (v >= 0.0) atomicMax(a, dbits(v));
}
// order-preserving map of any double to uint64 (for signed min/max atomics)
__device__ inline unsigned long long ord_bits(double v)
{
    unsigned long long u = dbits(v);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
// order-preserving map of a float to uint32 (signed min/max atomics)
__host__ __device__ inline unsigned ord_bitsf(float v)
{
#ifdef __CUDA_ARCH__
    unsigned u = __float_as_uint(v);
#else
    union { float f; unsigned u; } c; c.f = v; unsigned u = c.u;
#endif
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
// block-wide max of non-negative doubles through their bit patterns (the
// integer pipe orders them; the FP64 pipe is narrow on this part); every
// thread of the block must call it; the result is valid in thread 0
__device__ inline unsigned long long block_max_bits(unsigned long long b)
{
    __shared__ unsigned long long sm_bits[32];
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long o = __shfl_down_sync(0xffffffffu, b, off);
        b = o > b ? o : b;
    }
    const int warp = threadIdx.x >> 5;
    __syncthreads();   // a previous call's readers are done with sm_bits
    if ((threadIdx.x & 31) == 0) sm_bits[warp] = b;
    __syncthreads();
    if (threadIdx.x == 0)
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) b = sm_bits[w] > b ? sm_bits[w] : b;
    return b;
}
__device__ inline unsigned long long block_min_bits(unsigned long long b)
{
    __shared__ unsigned long long sm_bits_min[32];
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long o = __shfl_down_sync(0xffffffffu, b, off);
        b = o < b ? o : b;
    }
    const int warp = threadIdx.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sm_bits_min[warp] = b;
    __syncthreads();
    if (threadIdx.x == 0)
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) b = sm_bits_min[w] < b ? sm_bits_min[w] : b;
    return b;
}
__device__ inline void raise_err(Reduce* r, int code, int idx)
{
    if (atomicCAS(&r->err, 0, code) == 0) r->err_index = idx;
}
#endif

}  // namespace ndsph
