// ndsph_noalloc.cu -- ndsph_density_noalloc: one density pass (the first
// pass of iterate_density, with every particle treated as converged, i.e.
// the maxdensits = 0 case) that allocates no device memory.
//
// Who needs it: callers that may not allocate device memory at the point of
// the call -- codes whose device memory is owned by another runtime's pool
// (an OpenACC/OpenMP-offload Fortran host that maps the module arrays
// itself), real-time loops where the implicit device synchronisation of
// cudaMalloc/cudaFree is not allowed, or applications that reserve all
// device memory up front.  They pass device pointers for every input and
// output; the only other memory used is the fixed array g_noalloc_scratch
// below plus the kernel tables, both file-scope __device__ arrays that exist
// for as long as the library is loaded (on every GPU that loads it).
//
// Limits: npart <= NOALLOC_MAX_N and cells <= NOALLOC_MAX_CELLS (else
// NDSPH_E_CAPACITY; the cell count is worked out in floating point and
// checked before any integer conversion, so a very wide or non-finite
// bounding box is refused, never wrapped).  The scratch is shared by every
// call: calls that overlap on the GPU (two streams, two host threads) race
// on it.  Each call clears the parts that must start at zero.  The first
// call on a device fetches the scratch's device address with
// cudaGetSymbolAddress and uploads the kernel tables of all three
// dimensions; make that first call before any stream capture.  Errors come
// back as status codes, with the message in ndsph_last_error(NULL).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include "ndsph_common.cuh"

namespace {

using namespace ndsph;

constexpr int NOALLOC_MAX_N = 1 << 18;        // 262,144 particles
constexpr int NOALLOC_MAX_CELLS = 1 << 18;    // 262,144 cells
constexpr int NA_TILE = 1024;                 // scan tile (one thread per entry)
constexpr int NA_MAX_BLOCKS = (NOALLOC_MAX_CELLS + NA_TILE - 1) / NA_TILE + 1;

// scratch layout (ints): key[N] slot[N] perm2[N] perm[N] count[C] start[C+1]
// bsum[B] red[16] (7 order-preserving 64-bit words and the error code/index)
constexpr size_t NA_OFF_KEY = 0;
constexpr size_t NA_OFF_SLOT = NA_OFF_KEY + NOALLOC_MAX_N;
constexpr size_t NA_OFF_PERM2 = NA_OFF_SLOT + NOALLOC_MAX_N;
constexpr size_t NA_OFF_PERM = NA_OFF_PERM2 + NOALLOC_MAX_N;
constexpr size_t NA_OFF_COUNT = NA_OFF_PERM + NOALLOC_MAX_N;
constexpr size_t NA_OFF_START = NA_OFF_COUNT + NOALLOC_MAX_CELLS;
constexpr size_t NA_OFF_BSUM = NA_OFF_START + NOALLOC_MAX_CELLS + 1;
constexpr size_t NA_OFF_RED = NA_OFF_BSUM + NA_MAX_BLOCKS;
constexpr size_t NA_INTS = NA_OFF_RED + 16;
constexpr size_t NA_BYTES = NA_INTS * sizeof(int);   // about 6 MB
static_assert(NA_BYTES < (size_t(8) << 20), "the static scratch stays under 8 MB");

static __device__ __align__(256) int g_noalloc_scratch[NA_INTS];
// W, dW/dq, d2W/dq2 (value, slope) of the cubic spline for ndim = 1, 2, 3
static __device__ __align__(256) double2 g_noalloc_tab[3 * 3 * NTAB];

struct NaPtrs {
    int* key;
    int* slot;
    int* perm2;   // slots in atomic arrival order, before the per-cell rank
    int* perm;
    int* count;
    int* start;
    int* bsum;
    unsigned long long* red;   // [0] = hmax bits, [1..3] xlo, [4..6] xhi (order-preserving)
    int* err;                  // [0] first status raised by a kernel, [1] its particle
};

struct DeviceSetup {
    bool done = false;
    int* scratch = nullptr;
    double2* tab = nullptr;
};
DeviceSetup g_setup[64];
// errors are reported by status code, the message through ndsph_last_error(NULL)
struct NaErr {
    NaErr& operator=(const std::string& m)
    {
        set_global_error(m.c_str());
        return *this;
    }
    NaErr& operator=(const char* m) { return *this = std::string(m); }
} g_na_err;

__device__ inline unsigned long long na_ord(double v)
{
    unsigned long long u = (unsigned long long)__double_as_longlong(v);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
inline double na_unord(unsigned long long u)
{
    u = (u & 0x8000000000000000ull) ? (u & ~0x8000000000000000ull) : ~u;
    double d;
    memcpy(&d, &u, 8);
    return d;
}

__global__ void na_reset(NaPtrs p)
{
    if (threadIdx.x == 0) {
        p.red[0] = 0ull;
        for (int d = 0; d < 3; d++) { p.red[1 + d] = ~0ull; p.red[4 + d] = 0ull; }
        p.err[0] = 0;
        p.err[1] = 0;
    }
}
__device__ inline void na_raise(NaPtrs p, int code, int i)
{
    if (atomicCAS(&p.err[0], 0, code) == 0) p.err[1] = i;
}

__global__ void na_hmax_bbox(const double* __restrict__ x, const double* __restrict__ h, int ndim, int n,
                             NaPtrs p)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    atomicMax(&p.red[0], (unsigned long long)__double_as_longlong(h[i]));
    for (int d = 0; d < ndim; d++) {
        unsigned long long b = na_ord(x[(size_t)i * ndim + d]);
        atomicMin(&p.red[1 + d], b);
        atomicMax(&p.red[4 + d], b);
    }
}

__global__ void na_cell_key(const double* __restrict__ x, int ndim, int n, Grid g, NaPtrs p)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c[3] = {0, 0, 0};
    for (int d = 0; d < ndim; d++) {
        int cc = (int)floor((x[(size_t)i * ndim + d] - g.origin[d]) * g.inv_cs[d]);
        cc = cc < 0 ? 0 : (cc >= g.nc[d] ? g.nc[d] - 1 : cc);
        c[d] = cc;
    }
    int key = (c[2] * g.nc[1] + c[1]) * g.nc[0] + c[0];
    p.key[i] = key;
    p.slot[i] = atomicAdd(&p.count[key], 1);
}

// exclusive scan: per-tile sums, one-block scan of the tile sums, final pass
__device__ inline int na_block_scan(int v, int* sm, int* total)
{
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
    for (int off = 1; off < 32; off <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) sm[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int nw = blockDim.x >> 5;
        int w = (lane < nw) ? sm[lane] : 0;
        for (int off = 1; off < 32; off <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) w += y;
        }
        if (lane < nw) sm[lane] = w;
    }
    __syncthreads();
    int base = warp > 0 ? sm[warp - 1] : 0;
    if (total) *total = sm[(blockDim.x >> 5) - 1];
    __syncthreads();
    return base + x - v;
}
__global__ void na_scan_tiles(NaPtrs p, int nc)
{
    __shared__ int sm[32];
    int i = blockIdx.x * NA_TILE + threadIdx.x;
    int v = i < nc ? p.count[i] : 0;
    int tot;
    na_block_scan(v, sm, &tot);
    if (threadIdx.x == 0) p.bsum[blockIdx.x] = tot;
}
__global__ void na_scan_bsum(NaPtrs p, int nb)
{
    __shared__ int sm[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b0 = 0; b0 < nb; b0 += blockDim.x) {
        int i = b0 + threadIdx.x;
        int v = i < nb ? p.bsum[i] : 0;
        int tot;
        int ex = na_block_scan(v, sm, &tot);
        if (i < nb) p.bsum[i] = ex + carry;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
}
__global__ void na_scan_final(NaPtrs p, int nc, int n)
{
    __shared__ int sm[32];
    int i = blockIdx.x * NA_TILE + threadIdx.x;
    int v = i < nc ? p.count[i] : 0;
    int ex = na_block_scan(v, sm, nullptr) + p.bsum[blockIdx.x];
    if (i < nc) p.start[i] = ex;
    if (i == 0) p.start[nc] = n;
}
__global__ void na_scatter(NaPtrs p, int n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p.perm2[p.start[p.key[i]] + p.slot[i]] = i;
}
// each slot takes its rank by index among its cell's slots, so the order
// inside a cell does not depend on the atomics' arrival order
__global__ void na_cell_rank(NaPtrs p, int n)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int v = p.perm2[k];
    const int c = p.key[v];
    const int a = p.start[c], b = p.start[c + 1];
    int r = 0;
    for (int j = a; j < b; j++) r += (p.perm2[j] < v);
    p.perm[a + r] = v;
}

__device__ inline bool na_match(int ti, int tj)
{
    return (tj == ti) || (ti == NDSPH_ITYPE_GAS && tj == NDSPH_ITYPE_BND) ||
           (tj == NDSPH_ITYPE_GAS && ti == NDSPH_ITYPE_BND) ||
           (ti == NDSPH_ITYPE_DUST && tj == NDSPH_ITYPE_BNDDUST) ||
           (tj == NDSPH_ITYPE_DUST && ti == NDSPH_ITYPE_BNDDUST);
}

// density (density_sums.f90:38-379) as a gather, union criterion for
// numneigh, FP64 table kernel; then the per-particle normalisation of
// iterate_density.f90:172-278 with every particle converged
__global__ void na_density(const double* __restrict__ x, const double* __restrict__ h,
                           const double* __restrict__ m, const double* __restrict__ v,
                           const int* __restrict__ itype, int n, Grid g, DevOpts o, double dxbound,
                           double dq2, double ddq2, NaPtrs p, const double2* __restrict__ tab,
                           double* rho_out, double* drhodt_out, double* gradh_out, int* nn_out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int nd = o.ndim;
    double xi[3] = {0, 0, 0};
    for (int d = 0; d < nd; d++) xi[d] = x[(size_t)i * nd + d];
    const double hi = h[i];
    // iterate_density.f90:99-102
    if (!(hi > 2.2250738585072014e-308)) {
        na_raise(p, NDSPH_E_H_NONPOS, i);
        return;
    }
    const double hi1 = 1.0 / hi;
    const double hi21 = __dmul_rn(hi1, hi1);
    const int ti = itype[i];
    const bool fixed_i = (ti == NDSPH_ITYPE_BND || ti == NDSPH_ITYPE_BNDDUST);
    const int key = p.key[i];
    int cc[3] = {key % g.nc[0], (key / g.nc[0]) % g.nc[1], key / (g.nc[0] * g.nc[1])};
    double sw = 0, sg = 0, sd = 0;
    int nn = 0;
    const int nst = nd == 1 ? 3 : (nd == 2 ? 9 : 27);
    for (int so = 0; so < nst; so++) {
        int dd[3] = {so % 3 - 1, nd >= 2 ? (so / 3) % 3 - 1 : 0, nd >= 3 ? so / 9 - 1 : 0};
        int c[3], w[3];
        bool ok = true;
        for (int k = 0; k < 3; k++) {
            c[k] = cc[k] + dd[k];
            w[k] = 0;
            if (k < nd) {
                if (c[k] < 0) { if (!o.periodic[k]) ok = false; c[k] += g.nc[k]; w[k] = -1; }
                else if (c[k] >= g.nc[k]) { if (!o.periodic[k]) ok = false; c[k] -= g.nc[k]; w[k] = 1; }
            }
        }
        if (!ok) continue;
        const int cid = (c[2] * g.nc[1] + c[1]) * g.nc[0] + c[0];
        for (int s = p.start[cid]; s < p.start[cid + 1]; s++) {
            const int j = p.perm[s];
            if (!na_match(ti, itype[j])) continue;
            double dx[3] = {0, 0, 0};
            bool exists = true;
            for (int d = 0; d < nd; d++) {
                const double xj = x[(size_t)j * nd + d];
                double xim = xj;
                if (w[d] > 0) {
                    const double dist = __dsub_rn(xj, o.xmin[d]);
                    xim = __dadd_rn(o.xmax[d], dist);
                    exists = exists && dist < dxbound && dist > 0.0;
                } else if (w[d] < 0) {
                    const double dist = __dsub_rn(o.xmax[d], xj);
                    xim = __dadd_rn(o.xmin[d], __dsub_rn(xj, o.xmax[d]));
                    exists = exists && dist < dxbound && dist > 0.0;
                }
                dx[d] = __dsub_rn(xi[d], xim);
            }
            if (!exists) continue;
            double rij2 = __dmul_rn(dx[0], dx[0]);
            if (nd >= 2) rij2 = __dadd_rn(rij2, __dmul_rn(dx[1], dx[1]));
            if (nd >= 3) rij2 = __dadd_rn(rij2, __dmul_rn(dx[2], dx[2]));
            const double q2i = __dmul_rn(rij2, hi21);
            const double hj1 = 1.0 / h[j];
            const double q2j = __dmul_rn(__dmul_rn(rij2, hj1), hj1);
            if (!(q2i < 4.0 || q2j < 4.0)) continue;
            nn++;
            if (q2i >= 4.0 || fixed_i) continue;
            int idx = (int)__dmul_rn(q2i, ddq2);
            if (idx > IKERN || idx < 0) idx = IKERN;
            const double dxx = __dsub_rn(q2i, __dmul_rn((double)idx, dq2));
            const double2 ew = tab[idx], eg = tab[NTAB + idx];
            const double wv = ew.x + ew.y * dxx;
            const double gw = eg.x + eg.y * dxx;
            const double q = sqrt(q2i);
            const double mj = m[j];
            sw += mj * wv;
            sg += mj * (q * gw + (double)nd * wv);
            if (j != i) {
                double dvr = 0.0;
                for (int d = 0; d < nd; d++) dvr += (v[(size_t)i * 3 + d] - v[(size_t)j * 3 + d]) * dx[d];
                sd += mj * dvr * gw / (sqrt(rij2) + 2.220446049250313e-16);
            }
        }
    }
    nn_out[i] = nn;
    if (fixed_i) return;
    double hfac = hi1;
    if (nd >= 2) hfac *= hi1;
    if (nd >= 3) hfac *= hi1;
    const double rho = hfac * sw;
    // iterate_density.f90:168-170
    if (rho <= 1.e-6 && rho <= 0.0) {
        na_raise(p, NDSPH_E_RHO_NONPOS, i);
        return;
    }
    const double gsum = -hfac * hi1 * sg;
    const double dhdrhoi = -hi / ((double)nd * rho);
    double omegai = 1.0 - dhdrhoi * gsum;
    if (omegai < 1.e-5 && fabs(omegai) == 0.0) omegai = 1.0;
    const double gradh = 1.0 / omegai;
    rho_out[i] = rho;
    gradh_out[i] = gradh;
    drhodt_out[i] = hfac * hi1 * sd * gradh;
}

// the value/slope table of one dimension into out[0 .. 3*NTAB)
void build_tabs(int ndim, double2* out, double& dq2, double& ddq2)
{
    // cubic spline table (kernelND.f90:4143-4192, :4279-4289), as the main path builds it
    const double pi = 3.141592653589;
    dq2 = 4.0 / (double)IKERN;
    double cn = ndim == 1 ? 0.66666666666 : (ndim == 2 ? 10. / (7. * pi) : 1. / pi);
    std::vector<double> w(NTAB), gw(NTAB), ggw(NTAB);
    for (int i = 0; i <= IKERN; i++) {
        volatile double q2 = i * dq2;
        double q = sqrt(q2);
        double a = 0, b = 0, c = 0;
        if (q < 1.0) {
            volatile double t1 = 1.5 * q2, t2 = 0.75 * q;
            volatile double t3 = t2 * q2;
            a = (1. - t1) + t3;
            volatile double u1 = -3. * q, u2 = 2.25 * q2;
            b = u1 + u2;
            volatile double v1 = 4.5 * q;
            c = -3. + v1;
        } else if (q <= 2.0) {
            volatile double tt = 2. - q;
            volatile double t2 = tt * tt;
            volatile double t3 = t2 * tt;
            a = 0.25 * t3; b = -0.75 * t2; c = 1.5 * tt;
        }
        w[i] = cn * a; gw[i] = cn * b; ggw[i] = cn * c;
    }
    ddq2 = 1. / dq2;
    const std::vector<double>* t[3] = {&w, &gw, &ggw};
    for (int k = 0; k < 3; k++)
        for (int i = 0; i <= IKERN; i++) {
            int i1 = i + 1 > IKERN ? IKERN : i + 1;
            volatile double diff = (*t[k])[i1] - (*t[k])[i];
            out[k * NTAB + i] = make_double2((*t[k])[i], diff * ddq2);
        }
}

}  // namespace

// Allocation-free first density pass; see the file header and include/ndsph.h.
extern "C" int ndsph_density_noalloc(const ndsph_opts* opts, const double* d_x, const double* d_hh,
                                     const double* d_pmass, const double* d_vel, const int32_t* d_itype,
                                     int32_t npart, double* d_rho, double* d_drhodt, double* d_gradh,
                                     int32_t* d_numneigh, void* stream)
{
    if (!opts || npart < 0 || opts->ndim < 1 || opts->ndim > 3) {
        g_na_err = "ndsph_density_noalloc: bad arguments";
        return NDSPH_E_ARG;
    }
    // the boundary options ndsph_init accepts: none, fixed particles, periodic
    for (int d = 0; d < opts->ndim; d++) {
        if (opts->ibound[d] != 0 && opts->ibound[d] != 1 && opts->ibound[d] != 3) {
            g_na_err = "ndsph_density_noalloc: ibound must be 0, 1 or 3 (reflective/shearing ghosts are out of scope)";
            return NDSPH_E_ARG;
        }
        if (opts->ibound[d] == 3 && !(opts->xmax[d] > opts->xmin[d])) {
            g_na_err = "ndsph_density_noalloc: periodic box with xmax <= xmin";
            return NDSPH_E_ARG;
        }
    }
    if (npart > NOALLOC_MAX_N) {
        char buf[160];
        snprintf(buf, sizeof buf, "ndsph_density_noalloc: npart %d above the fixed maximum %d", npart,
                 NOALLOC_MAX_N);
        g_na_err = buf;
        return NDSPH_E_CAPACITY;
    }
    if (npart == 0) return 0;
    if (!d_x || !d_hh || !d_pmass || !d_vel || !d_itype || !d_rho || !d_drhodt || !d_gradh || !d_numneigh) {
        g_na_err = "ndsph_density_noalloc: null device pointer";
        return NDSPH_E_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        g_na_err = "ndsph_density_noalloc: no CUDA device";
        return NDSPH_E_CUDA;
    }
    DeviceSetup& su = g_setup[dev];
    if (!su.done) {
        // once per device (with that device current): device addresses of the
        // static arrays, and the kernel tables of the three dimensions
        cudaError_t e = cudaGetSymbolAddress((void**)&su.scratch, g_noalloc_scratch);
        if (e != cudaSuccess) { g_na_err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e); return NDSPH_E_CUDA; }
        e = cudaGetSymbolAddress((void**)&su.tab, g_noalloc_tab);
        if (e != cudaSuccess) { g_na_err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e); return NDSPH_E_CUDA; }
        std::vector<double2> tabs(3 * 3 * NTAB);
        double dq2, ddq2;
        for (int nd = 1; nd <= 3; nd++) build_tabs(nd, tabs.data() + (size_t)(nd - 1) * 3 * NTAB, dq2, ddq2);
        e = cudaMemcpyToSymbol(g_noalloc_tab, tabs.data(), sizeof(double2) * tabs.size());
        if (e != cudaSuccess) { g_na_err = std::string("cudaMemcpyToSymbol: ") + cudaGetErrorString(e); return NDSPH_E_CUDA; }
        su.done = true;
    }
    NaPtrs p;
    p.key = su.scratch + NA_OFF_KEY;
    p.slot = su.scratch + NA_OFF_SLOT;
    p.perm2 = su.scratch + NA_OFF_PERM2;
    p.perm = su.scratch + NA_OFF_PERM;
    p.count = su.scratch + NA_OFF_COUNT;
    p.start = su.scratch + NA_OFF_START;
    p.bsum = su.scratch + NA_OFF_BSUM;
    p.red = (unsigned long long*)(su.scratch + NA_OFF_RED);
    p.err = su.scratch + NA_OFF_RED + 14;
    const int nd = opts->ndim;
    const double2* tab = su.tab + (size_t)(nd - 1) * 3 * NTAB;
    const int bs = 256, nb = (npart + bs - 1) / bs;

    NDSPH_COUNT_LAUNCH, na_reset<<<1, 32, 0, st>>>(p);
    NDSPH_COUNT_LAUNCH, na_hmax_bbox<<<nb, bs, 0, st>>>(d_x, d_hh, nd, npart, p);
    unsigned long long red[7];
    cudaError_t e = cudaMemcpyAsync(red, p.red, sizeof(red), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { g_na_err = cudaGetErrorString(e); return NDSPH_E_CUDA; }
    double hmax;
    memcpy(&hmax, &red[0], 8);
    if (!(hmax > 0.0) || !std::isfinite(hmax)) { g_na_err = "ndsph_density_noalloc: max h <= 0 or not finite"; return NDSPH_E_H_NONPOS; }

    // cell grid (same rule as the main path: periodic dims tile the box with
    // cells >= 2 hmax, open dims pad the bounding box by one cell).  Counts
    // are taken in double and checked against the maximum before any
    // conversion to int.
    for (int d = 0; d < nd; d++) {
        if (!std::isfinite(na_unord(red[1 + d])) || !std::isfinite(na_unord(red[4 + d]))) {
            g_na_err = "ndsph_density_noalloc: non-finite position";
            return NDSPH_E_NAN;
        }
    }
    DevOpts o;
    memset(&o, 0, sizeof o);
    o.ndim = nd;
    Grid g{};   // zero sizes; the 3^ndim stencil (sw 3, nlshift 5)
    const double cmin = 2.0 * hmax * (1.0 + 1.e-9);
    double ncells_d = 1.0;
    for (int d = 0; d < 3; d++) {
        o.ibound[d] = d < nd ? opts->ibound[d] : 0;
        o.periodic[d] = (d < nd && opts->ibound[d] == 3);
        o.xmin[d] = opts->xmin[d];
        o.xmax[d] = opts->xmax[d];
        double ncd = 1.0;
        if (d >= nd) {
            g.cs[d] = 1.0; g.origin[d] = 0.0;
        } else if (o.periodic[d]) {
            const double L = opts->xmax[d] - opts->xmin[d];
            ncd = std::floor(L / cmin);
            if (!(ncd >= 3.0)) { g_na_err = "ndsph_density_noalloc: periodic box smaller than 3 cells of 2 hmax"; return NDSPH_E_CELLS; }
            if (ncd > 4096.0) ncd = 4096.0;
            g.origin[d] = opts->xmin[d];
            g.cs[d] = L / ncd;
        } else {
            const double lo = na_unord(red[1 + d]), hi = na_unord(red[4 + d]);
            ncd = std::floor(((hi - lo) + 2.0 * cmin) / cmin) + 1.0;
            g.cs[d] = cmin;
            g.origin[d] = lo - cmin;
        }
        if (!(ncd >= 1.0) || ncd > (double)NOALLOC_MAX_CELLS) ncd = (double)NOALLOC_MAX_CELLS + 1.0;
        ncells_d *= ncd;
        g.nc[d] = (ncd <= (double)NOALLOC_MAX_CELLS) ? (int)ncd : 1;
        g.inv_cs[d] = 1.0 / g.cs[d];
    }
    if (!(ncells_d <= (double)NOALLOC_MAX_CELLS)) {
        char buf[200];
        snprintf(buf, sizeof buf, "ndsph_density_noalloc: %.0f cells above the fixed maximum %d", ncells_d,
                 NOALLOC_MAX_CELLS);
        g_na_err = buf;
        return NDSPH_E_CAPACITY;
    }
    g.ncells = (int)ncells_d;
    const int nc = g.ncells;

    // the counts must start at zero on every call (the scratch keeps the last call's contents)
    e = cudaMemsetAsync(p.count, 0, sizeof(int) * (size_t)nc, st);
    if (e != cudaSuccess) { g_na_err = cudaGetErrorString(e); return NDSPH_E_CUDA; }
    NDSPH_COUNT_LAUNCH, na_cell_key<<<nb, bs, 0, st>>>(d_x, nd, npart, g, p);
    const int ntiles = (nc + NA_TILE - 1) / NA_TILE;
    NDSPH_COUNT_LAUNCH, na_scan_tiles<<<ntiles, NA_TILE, 0, st>>>(p, nc);
    NDSPH_COUNT_LAUNCH, na_scan_bsum<<<1, NA_TILE, 0, st>>>(p, ntiles);
    NDSPH_COUNT_LAUNCH, na_scan_final<<<ntiles, NA_TILE, 0, st>>>(p, nc, npart);
    NDSPH_COUNT_LAUNCH, na_scatter<<<nb, bs, 0, st>>>(p, npart);
    NDSPH_COUNT_LAUNCH, na_cell_rank<<<nb, bs, 0, st>>>(p, npart);
    const double dq2 = 4.0 / (double)IKERN, ddq2 = 1.0 / dq2;
    NDSPH_COUNT_LAUNCH, na_density<<<(npart + 127) / 128, 128, 0, st>>>(d_x, d_hh, d_pmass, d_vel, d_itype, npart, g, o, 2.0 * hmax,
                                                    dq2, ddq2, p, tab, d_rho, d_drhodt, d_gradh, d_numneigh);
    int err[2] = {0, 0};
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(err, p.err, sizeof(err), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { g_na_err = cudaGetErrorString(e); return NDSPH_E_CUDA; }
    if (err[0]) {
        char buf[160];
        snprintf(buf, sizeof buf, "ndsph_density_noalloc: %s at particle %d",
                 err[0] == NDSPH_E_H_NONPOS ? "h <= 0 in density call (iterate_density.f90:99-102)"
                                            : "rho <= 0 (iterate_density.f90:168-170)",
                 err[1] + 1);
        g_na_err = buf;
        return err[0];
    }
    return 0;
}
