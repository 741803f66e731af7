// ndsph_kernels.cu -- link (cell keys, counting sort by cell, permutation
// gather), host-layout conversion, EOS, fixed-particle copies and leapfrog.
//
// All kernels are HBM-bound streaming passes over per-particle SoA arrays:
// one thread per particle, grid = ceil(n/256) blocks (a multiple of the 152 SMs
// for any n above ~40k), coalesced 8-byte loads and stores.
#include <algorithm>
#include <cstdio>
#include <cmath>
#include "ndsph_launch.h"
#include "ndsph_step.cuh"

namespace ndsph {

static inline int nblk(long n, int bs) { return (int)((n + bs - 1) / bs); }

// ---------------------------------------------------------------------------
// boundary boundaryND.f90:30-90: periodic wrap (x > xmax -> (xmin + x) - xmax,
// x < xmin -> xmax - (xmin - x)); fixed particles are wrapped as well because
// the reference loops over all npart.
// ---------------------------------------------------------------------------
__global__ void k_boundary_wrap(FieldPtrs F, DevOpts o, int n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int d = 0; d < o.ndim; d++) {
        if (o.ibound[d] != 3) continue;
        double x = F.f[X0 + d][i];
        if (x > o.xmax[d]) x = __dsub_rn(__dadd_rn(o.xmin[d], x), o.xmax[d]);
        else if (x < o.xmin[d]) x = __dsub_rn(o.xmax[d], __dsub_rn(o.xmin[d], x));
        F.f[X0 + d][i] = x;
    }
}
void launch_boundary_wrap(FieldPtrs F, DevOpts o, int n, cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_boundary_wrap<<<nblk(n, 256), 256, 0, st>>>(F, o, n);
}

// The reductions below run a grid-stride loop on a grid of at most
// RED_BLOCKS blocks: one block per particle group made every block's
// atomics land on the same few words (8192 blocks at 2.1 M particles), and
// the atomics, not the 32 B a particle, set the kernel's time.  Maxima and
// minima do not depend on the order, so the results are the same.
constexpr int RED_BLOCKS = 152 * 4;
inline int red_blocks(int n) { return std::min(nblk(n, 256), RED_BLOCKS); }

// max h (bound module hhmax, linkND.f90:70 / ghostND_mhd.f90:77) and the
// particle bounding box (linkND.f90:80-89) in one pass
__global__ void k_hmax_bbox(FieldPtrs F, int ndim, int n, Reduce* red, unsigned long long* dst, const int* gate)
{
    if (gate && *gate == 0) return;
    // block-level reduction first: one set of atomics per block, not per warp
    __shared__ double sh[8];
    __shared__ unsigned long long slo[8][3], shi[8][3];
    double h = 0.0;
    unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0ull, 0ull, 0ull};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        h = fmax(h, F.f[HH][i]);
        for (int d = 0; d < ndim; d++) {
            const unsigned long long b = ord_bits(F.f[X0 + d][i]);
            lo[d] = b < lo[d] ? b : lo[d];
            hi[d] = b > hi[d] ? b : hi[d];
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        h = fmax(h, __shfl_down_sync(0xffffffffu, h, off));
        for (int d = 0; d < 3; d++) {
            unsigned long long a = __shfl_down_sync(0xffffffffu, lo[d], off);
            unsigned long long b = __shfl_down_sync(0xffffffffu, hi[d], off);
            lo[d] = a < lo[d] ? a : lo[d];
            hi[d] = b > hi[d] ? b : hi[d];
        }
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        sh[warp] = h;
        for (int d = 0; d < 3; d++) { slo[warp][d] = lo[d]; shi[warp][d] = hi[d]; }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = blockDim.x >> 5;
        for (int w = 1; w < nw; w++) {
            h = fmax(h, sh[w]);
            for (int d = 0; d < 3; d++) {
                lo[d] = slo[w][d] < lo[d] ? slo[w][d] : lo[d];
                hi[d] = shi[w][d] > hi[d] ? shi[w][d] : hi[d];
            }
        }
        atomicMax(dst, dbits(h));
        for (int d = 0; d < ndim; d++) {
            atomicMin(&red->xlo[d], lo[d]);
            atomicMax(&red->xhi[d], hi[d]);
        }
    }
}
void launch_hmax_bbox(FieldPtrs F, int ndim, int n, Reduce* red, unsigned long long* dst, cudaStream_t st,
                      const int* gate)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_hmax_bbox<<<red_blocks(n), 256, 0, st>>>(F, ndim, n, red, dst, gate);
}

// ---------------------------------------------------------------------------
// cell keys + counting: key = (cz*ny + cy)*nx + cx, row-major like the
// reference's icell (linkND.f90:127-135).  The atomic slot is made
// deterministic afterwards by sorting each cell's segment by index.
// ---------------------------------------------------------------------------
__device__ inline int cell_coord(double x, double origin, double inv_cs, int nc)
{
    int c = (int)floor((x - origin) * inv_cs);
    c = c < 0 ? 0 : c;
    c = c >= nc ? nc - 1 : c;
    return c;
}

__global__ void k_cell_key(FieldPtrs F, Grid g, int ndim, int n, const int* sim, SortScratch s)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c[3] = {0, 0, 0};
    for (int d = 0; d < ndim; d++) c[d] = cell_coord(F.f[X0 + d][i], g.origin[d], g.inv_cs[d], g.nc[d]);
    int key = (c[2] * g.nc[1] + c[1]) * g.nc[0] + c[0];
    if (g.nstack > 1) key += sim[i] * g.ncs;   // the simulation's own grid
    s.key[i] = key;
    s.slot[i] = atomicAdd(&s.count[key], 1);
}
void launch_cell_key(FieldPtrs F, Grid g, DevOpts o, int n, const int* sim, SortScratch s, Reduce* red,
                     cudaStream_t st)
{
    (void)red;
    cudaMemsetAsync(s.count, 0, sizeof(int) * (size_t)g.ncells, st);
    if (n > 0) NDSPH_COUNT_LAUNCH, k_cell_key<<<nblk(n, 256), 256, 0, st>>>(F, g, o.ndim, n, sim, s);
}

// ---------------------------------------------------------------------------
// exclusive scan of the cell counts (three passes: block sums, scan of the
// block sums in one CTA, block-local scan plus offset)
// ---------------------------------------------------------------------------
constexpr int SCAN_BS = 1024;
constexpr int SCAN_IPT = 4;
constexpr int SCAN_TILE = SCAN_BS * SCAN_IPT;

__device__ inline int block_exclusive_scan(int v, int* smem, int* total)
{
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
    for (int off = 1; off < 32; off <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) smem[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int nw = blockDim.x >> 5;
        int w = (lane < nw) ? smem[lane] : 0;
        for (int off = 1; off < 32; off <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) w += y;
        }
        if (lane < nw) smem[lane] = w;
    }
    __syncthreads();
    int base = (warp > 0) ? smem[warp - 1] : 0;
    if (total) *total = smem[(blockDim.x >> 5) - 1];
    __syncthreads();
    return base + x - v;
}

__global__ void k_scan_blocksum(const int* in, int n, int* bsum)
{
    __shared__ int sm[32];
    int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_IPT;
    int s = 0;
    for (int k = 0; k < SCAN_IPT; k++) s += (base + k < n) ? in[base + k] : 0;
    int tot;
    block_exclusive_scan(s, sm, &tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void k_scan_bsum(int* bsum, int nb)
{
    __shared__ int sm[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b0 = 0; b0 < nb; b0 += blockDim.x) {
        int i = b0 + threadIdx.x;
        int v = (i < nb) ? bsum[i] : 0;
        int tot;
        int ex = block_exclusive_scan(v, sm, &tot);
        if (i < nb) bsum[i] = ex + carry;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
}

__global__ void k_scan_final(const int* in, int n, const int* bsum, int* out)
{
    __shared__ int sm[32];
    int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_IPT;
    int v[SCAN_IPT];
    int s = 0;
    for (int k = 0; k < SCAN_IPT; k++) { v[k] = (base + k < n) ? in[base + k] : 0; s += v[k]; }
    int ex = block_exclusive_scan(s, sm, nullptr) + bsum[blockIdx.x];
    for (int k = 0; k < SCAN_IPT; k++) {
        if (base + k < n) out[base + k] = ex;
        ex += v[k];
    }
    // out[n] = total (written by the last block's last thread)
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[n] = ex;
}

void launch_scan(SortScratch s, int ncells, cudaStream_t st)
{
    int nb = nblk(ncells, SCAN_TILE);
    NDSPH_COUNT_LAUNCH, k_scan_blocksum<<<nb, SCAN_BS, 0, st>>>(s.count, ncells, s.blocksums);
    NDSPH_COUNT_LAUNCH, k_scan_bsum<<<1, SCAN_BS, 0, st>>>(s.blocksums, nb);
    NDSPH_COUNT_LAUNCH, k_scan_final<<<nb, SCAN_BS, 0, st>>>(s.count, ncells, s.blocksums, s.start);
}

__global__ void k_scatter(SortScratch s, int n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    s.perm2[s.start[s.key[i]] + s.slot[i]] = i;
}

// deterministic order inside each cell: every slot takes its rank by index
// among the cell's slots (the indices are distinct, so the ranks fill the
// cell; one thread per slot, the cell's indices read by all its threads)
__global__ void k_cell_rank(SortScratch s, int n)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int v = s.perm2[k];
    const int c = s.key[v];
    const int a = s.start[c], b = s.start[c + 1];
    int r = 0;
    for (int j = a; j < b; j++) r += (s.perm2[j] < v);
    s.perm[a + r] = v;
}

void launch_scatter_sort(SortScratch s, int n, int ncells, cudaStream_t st)
{
    (void)ncells;
    if (n <= 0) return;
    NDSPH_COUNT_LAUNCH, k_scatter<<<nblk(n, 256), 256, 0, st>>>(s, n);
    NDSPH_COUNT_LAUNCH, k_cell_rank<<<nblk(n, 256), 256, 0, st>>>(s, n);
}

// permutation gather of the live fields: dst[f][k] = src[f][perm[k]]
__global__ void k_gather_fields(FieldPtrs dst, FieldPtrs src, const int* __restrict__ fields, int nfields,
                                const int* __restrict__ perm, int n)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int p = perm[k];
    for (int q = 0; q < nfields; q++) {
        int f = fields[q];
        dst.f[f][k] = src.f[f][p];
    }
}
void launch_gather_fields(FieldPtrs dst, FieldPtrs src, const int* fields, int nfields, const int* perm, int n,
                          cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_gather_fields<<<nblk(n, 256), 256, 0, st>>>(dst, src, fields, nfields, perm, n);
}

__global__ void k_gather_int(int* dst, const int* src, const int* perm, int n)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) dst[k] = src[perm[k]];
}
void launch_gather_int(int* dst, const int* src, const int* perm, int n, cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_gather_int<<<nblk(n, 256), 256, 0, st>>>(dst, src, perm, n);
}

// after the gather: cell id per slot, inverse of id
__global__ void k_post_sort(Side S, SortScratch s, int n)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    S.cell[k] = s.key[s.perm[k]];
    S.pos_of_id[S.id[k]] = k;
}

// FP32 position of each particle relative to its cell's lower corner, and h
__global__ void k_xs(FieldPtrs F, Side S, Grid g, int ndim, int n)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int cc[3];
    cell_coords(S.cell[k], g, cc);
    float r[3] = {0.f, 0.f, 0.f};
    for (int d = 0; d < ndim; d++) r[d] = (float)(F.f[X0 + d][k] - (g.origin[d] + cc[d] * g.cs[d]));
    S.xs[k] = make_float4(r[0], r[1], r[2], (float)F.f[HH][k]);
}

void launch_post_sort(Side S, SortScratch s, int n, int ncells, Grid g, FieldPtrs F, DevOpts o, cudaStream_t st)
{
    (void)ncells;
    if (n > 0) NDSPH_COUNT_LAUNCH, k_post_sort<<<nblk(n, 256), 256, 0, st>>>(S, s, n);
    if (n > 0) NDSPH_COUNT_LAUNCH, k_xs<<<nblk(n, 256), 256, 0, st>>>(F, S, g, o.ndim, n);
}
void launch_xs(FieldPtrs F, Side S, Grid g, DevOpts o, int n, cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_xs<<<nblk(n, 256), 256, 0, st>>>(F, S, g, o.ndim, n);
}

// A step that keeps the previous link (same slot order, cells and rows).
// Each slot's position is taken relative to the lower corner of the cell it
// was sorted into, with a periodic jump of the boundary wrap undone, so the
// stencil offsets stored in the rows stay the cell offsets between the two
// slots.  Reduced: the largest displacement since the rows were built, the
// smallest row slack skin*h_build - grow*h, and the largest h.  A pair with
// r < 2 max(h_i, h_j) now was within 2 max(h) + 2 dmax when the rows were
// built, so every such pair is in the rows while h + dmax <= skin*h_build
// holds for every particle (the host checks it with dmax and the slack).
__global__ void k_reuse_check(FieldPtrs F, Side S, Grid g, DevOpts o, int n, float skin, float grow, Reduce* red)
{
    __shared__ float sd[8], ss[8];
    __shared__ unsigned long long sh[8];
    float d2 = 0.f, slack = 3.0e38f;
    // h as its bit pattern: h >= 0 orders like its bits (integer pipe)
    unsigned long long hb = 0ull;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        int cc[3];
        cell_coords(S.cell[k], g, cc);
        float r[3] = {0.f, 0.f, 0.f};
        for (int d = 0; d < o.ndim; d++) {
            const double v = F.f[X0 + d][k] - (g.origin[d] + cc[d] * g.cs[d]);
            r[d] = (float)v;
            // the periodic jump is undone only for a separation beyond half
            // the box; |v| <= L/4 (tested in FP32, where it is conservative)
            // never is one, so the FP64 tests run only for the rare rest
            if (o.periodic[d] && !(fabsf(r[d]) <= 0.25f * (float)o.L[d])) {
                double w = v;
                if (w > 0.5 * o.L[d]) w -= o.L[d];
                else if (w < -0.5 * o.L[d]) w += o.L[d];
                r[d] = (float)w;
            }
        }
        const double h = F.f[HH][k];
        S.xs[k] = make_float4(r[0], r[1], r[2], (float)h);
        const float4 b = S.xsb[k];
        const float e0 = r[0] - b.x, e1 = r[1] - b.y, e2 = r[2] - b.z;
        float dk = e0 * e0 + e1 * e1 + e2 * e2;
        float sk = skin * S.hb[k] - grow * (float)h;
        if (!(dk <= 3.0e38f)) dk = 3.0e38f;          // non-finite position: fails the check
        if (!(sk >= -3.0e38f)) sk = -3.0e38f;
        d2 = fmaxf(d2, dk);
        slack = fminf(slack, sk);
        const unsigned long long hk = dbits(h);
        hb = hk > hb ? hk : hb;
    }
    for (int off = 16; off > 0; off >>= 1) {
        d2 = fmaxf(d2, __shfl_down_sync(0xffffffffu, d2, off));
        slack = fminf(slack, __shfl_down_sync(0xffffffffu, slack, off));
        const unsigned long long o = __shfl_down_sync(0xffffffffu, hb, off);
        hb = o > hb ? o : hb;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { sd[warp] = d2; ss[warp] = slack; sh[warp] = hb; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
            d2 = fmaxf(d2, sd[w]);
            slack = fminf(slack, ss[w]);
            hb = sh[w] > hb ? sh[w] : hb;
        }
        atomicMax(&red->reuse_d2, __float_as_uint(d2));
        atomicMin(&red->reuse_slack, ord_bitsf(slack));
        atomicMax(&red->hmax, hb);
    }
}
void launch_reuse_check(FieldPtrs F, Side S, Grid g, DevOpts o, int n, float skin, float grow, Reduce* red,
                        cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_reuse_check<<<red_blocks(n), 256, 0, st>>>(F, S, g, o, n, skin, grow, red);
}

// ---------------------------------------------------------------------------
// host layout <-> slab
// ---------------------------------------------------------------------------
__global__ void k_aos_to_slab(FieldPtrs F, int f0, int ncomp, const double* __restrict__ aos, int stride,
                             const int* __restrict__ id, int n)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int src = id ? id[k] : k;
    for (int c = 0; c < ncomp; c++) F.f[f0 + c][k] = aos[(size_t)src * stride + c];
}
void launch_aos_to_slab(FieldPtrs F, int f0, int ncomp, const double* aos, int stride, const int* id, int n,
                        cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_aos_to_slab<<<nblk(n, 256), 256, 0, st>>>(F, f0, ncomp, aos, stride, id, n);
}

// gather in host order: particle p comes from slot pos[p] (pos = inverse of
// the slot -> particle map), so the stores -- to a staging buffer or straight
// to the caller's array over the CPU-GPU link -- are coalesced and the
// scattered reads hit the slab's L2-resident field
__global__ void k_slab_to_aos(double* __restrict__ aos, int stride, FieldPtrs F, int f0, int ncomp,
                              const int* __restrict__ pos, int n)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int src = pos ? pos[p] : p;
    for (int c = 0; c < ncomp; c++) aos[(size_t)p * stride + c] = F.f[f0 + c][src];
}
void launch_slab_to_aos(double* aos, int stride, FieldPtrs F, int f0, int ncomp, const int* pos, int n,
                        cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_slab_to_aos<<<nblk(n, 256), 256, 0, st>>>(aos, stride, F, f0, ncomp, pos, n);
}

__global__ void k_int_to_slab(int* dst, const int* src, const int* id, int n)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) dst[k] = src[id ? id[k] : k];
}
void launch_int_to_slab(int* dst, const int* src, const int* id, int n, cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_int_to_slab<<<nblk(n, 256), 256, 0, st>>>(dst, src, id, n);
}
__global__ void k_slab_to_int(int* dst, const int* src, const int* pos, int n)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) dst[p] = src[pos ? pos[p] : p];
}
__global__ void k_int_shift(int* dst, const int* src, int n, int add)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[i] + add;
}
void launch_int_shift(int* dst, const int* src, int n, int add, cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_int_shift<<<nblk(n, 256), 256, 0, st>>>(dst, src, n, add);
}
void launch_slab_to_int(int* dst, const int* src, const int* pos, int n, cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_slab_to_int<<<nblk(n, 256), 256, 0, st>>>(dst, src, pos, n);
}
__global__ void k_iota(int* a, int n)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) a[k] = k;
}
void launch_iota(int* a, int n, cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_iota<<<nblk(n, 256), 256, 0, st>>>(a, n);
}
__global__ void k_fill(double* a, double v, int n)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) a[k] = v;
}
void launch_fill(double* a, double v, int n, cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_fill<<<nblk(n, 256), 256, 0, st>>>(a, v, n);
}
__global__ void k_copy(double* dst, const double* src, int n)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) dst[k] = src[k];
}
void launch_copy(double* dst, const double* src, int n, cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_copy<<<nblk(n, 256), 256, 0, st>>>(dst, src, n);
}

// ---------------------------------------------------------------------------
// density pass set-up
// ---------------------------------------------------------------------------
__global__ void k_h1(FieldPtrs F, Side S, int n)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double h = F.f[HH][k];
    S.h1[k] = 1.0 / h;
    float4 x = S.xs[k];
    x.w = (float)h;
    S.xs[k] = x;
}
void launch_h1(FieldPtrs F, Side S, int n, cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_h1<<<nblk(n, 256), 256, 0, st>>>(F, S, n);
}

// iterate_density.f90:79-86 (zero gradh.. on non-fixed particles) and
// hhin = hh (:87); h <= 0 check (:99-102)
__global__ void k_density_init(FieldPtrs F, Side S, int n, Reduce* red)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    density_init_one(F, S, k, red);
}
void launch_density_init(FieldPtrs F, Side S, int n, Reduce* red, cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_density_init<<<nblk(n, 256), 256, 0, st>>>(F, S, n, red);
}

// fixed particles take rho.. from their source after each NR pass
// (iterate_density.f90:312-328)
__global__ void k_fixed_density_copy(FieldPtrs F, Side S, int n)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    fixed_density_copy_one(F, S, k);
}
void launch_fixed_density_copy(FieldPtrs F, Side S, int n, cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_fixed_density_copy<<<nblk(n, 256), 256, 0, st>>>(F, S, n);
}

// ---------------------------------------------------------------------------
// conservative2primitive (in-scope part) + equation_of_state eos.f90:40-106;
// also the stressmax reduction of get_rates (ratesND_mhd.f90:232-245)
// ---------------------------------------------------------------------------
__global__ void k_eos(FieldPtrs F, Side S, DevOpts o, int n, Reduce* red)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    const double st = (k < n) ? eos_one(F, S, o, k, red) : 0.0;
    if (o.batched) {
        if (k < n && st > 0.0) atomic_max_pos(&o.sim_red[(size_t)S.sim[k] * SIMRED + SR_STRESS], st);
        return;
    }
    // one atomic per block (one per warp serialised ~65k same-address
    // atomics at the 128^3 box)
    const unsigned long long sb = block_max_bits(dbits(st));   // st >= 0
    if (threadIdx.x == 0 && sb != 0ull) atomicMax(&red->stressmax, sb);
}
void launch_eos(FieldPtrs F, Side S, DevOpts o, int n, Reduce* red, cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_eos<<<nblk(n, 256), 256, 0, st>>>(F, S, o, n, red);
}

// copy_particle copy_particle.f90:28-80 for fixed particles
// (conservative2primitive.f90:430-441): everything but x and vel
__global__ void k_fixed_copy(FieldPtrs F, Side S, int n)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    fixed_copy_one(F, S, k);
}
void launch_fixed_copy(FieldPtrs F, Side S, DevOpts o, int n, cudaStream_t st)
{
    if (o.has_fixed && n > 0) NDSPH_COUNT_LAUNCH, k_fixed_copy<<<nblk(n, 256), 256, 0, st>>>(F, S, n);
}

// ---------------------------------------------------------------------------
// leapfrog stepND_leapfrog_mhd.f90:31-275
// ---------------------------------------------------------------------------
// leapfrog save and predictor (stepND_leapfrog_mhd.f90:70-101, :107-160) in one pass:
// each particle reads only its own fields (a fixed particle's position,
// which follows its source particle's saves, is set afterwards by
// k_predictor_fixed_x).  part 0: every field; 1: position, velocity and h
// (with the saves of x, v, force, h, dh/dt, rho); 2: Bevol, energy and alpha
// (with their saves and the saves of their rates) -- a host-buffer step
// uploads the latter while the link and the density passes run
__global__ void k_predictor_fused(FieldPtrs F, Side S, DevOpts o, int n, const Reduce* red, int part)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double dt = o.batched ? o.sim_dt[S.sim[i]] : red->dt;
    predictor_one(F, S, o, dt, i, part);
}

void launch_predictor_part(FieldPtrs F, Side S, DevOpts o, int n, Reduce* red, int part, cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_predictor_fused<<<nblk(n, 256), 256, 0, st>>>(F, S, o, n, red, part);
}

// fixed particles after k_predictor_fused: the position moves by the source
// particle's saved velocity and force (stepND_leapfrog_mhd.f90:110-116);
// every other field of theirs is held, as k_predictor_fused leaves it
__global__ void k_predictor_fixed_x(FieldPtrs F, Side S, DevOpts o, int n, const Reduce* red)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double dt = o.batched ? o.sim_dt[S.sim[i]] : red->dt;
    predictor_fixed_x_one(F, S, o, dt, i);
}

void launch_predictor(FieldPtrs F, Side S, DevOpts o, int n, Reduce* red, cudaStream_t st)
{
    if (n <= 0) return;
    // save and predictor in one pass; with fixed particles their positions
    // then follow their sources' saves (complete when the first kernel ends)
    NDSPH_COUNT_LAUNCH, k_predictor_fused<<<nblk(n, 256), 256, 0, st>>>(F, S, o, n, red, 0);
    if (o.has_fixed) NDSPH_COUNT_LAUNCH, k_predictor_fixed_x<<<nblk(n, 256), 256, 0, st>>>(F, S, o, n, red);
}

__global__ void k_corrector(FieldPtrs F, Side S, DevOpts o, int n, Reduce* red)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (red->gfail) return;   // a captured step that failed is redone from the predicted state
    const double dt = o.batched ? o.sim_dt[S.sim[i]] : red->dt;
    corrector_one(F, S, o, dt, i, red);
}
void launch_corrector(FieldPtrs F, Side S, DevOpts o, int n, Reduce* red, cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_corrector<<<nblk(n, 256), 256, 0, st>>>(F, S, o, n, red);
}

// one simulation without fixed particles, between two steps of a
// device-resident run: this step's corrector and the next step's save and
// predictor (with the next dt, dtnext) in one pass over the particles -- the
// same arithmetic as k_corrector followed by k_predictor_fused.  A batch
// (no fixed particles) takes each simulation's dt and next dt (dtnext[sim]).
__global__ void k_corrector_predictor(FieldPtrs F, Side S, DevOpts o, int n, Reduce* red, const double* dtnext)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double dt = o.batched ? o.sim_dt[S.sim[i]] : red->dt;
    const double dtn = o.batched ? dtnext[S.sim[i]] : *dtnext;
    Corrected c;
    corrector_values(F, S, o, dt, i, c);
    if (!(c.h > 0.0)) raise_err(red, NDSPH_E_H_NONPOS, S.id[i]);
    for (int d = 0; d < 3; d++) F.f[V0 + d][i] = c.v[d];
    if (o.imhd != 0)
        for (int d = 0; d < 3; d++) F.f[BE0 + d][i] = c.be[d];
    for (int d = 0; d < 3; d++)
        if (o.iavlim[d] != 0) F.f[AL0 + d][i] = c.al[d];
    F.f[HH][i] = c.h;
    if (o.iener != 0) F.f[EN][i] = c.en;
#pragma unroll
    for (int d = 0; d < 3; d++)
        if (d < o.ndim && o.ibound[d] == 3) F.f[X0 + d][i] = c.x[d];
    predictor_one(F, S, o, dtn, i, 0);
}
void launch_corrector_predictor(FieldPtrs F, Side S, DevOpts o, int n, Reduce* red, const double* dtnext,
                                cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_corrector_predictor<<<nblk(n, 256), 256, 0, st>>>(F, S, o, n, red, dtnext);
}

__global__ void k_read_words(const unsigned* __restrict__ src, unsigned* __restrict__ dst, int nw)
{
    for (int k = threadIdx.x; k < nw; k += blockDim.x) dst[k] = src[k];
}
void launch_read_words(void* dst, const void* src, size_t bytes, cudaStream_t st)
{
    NDSPH_COUNT_LAUNCH, k_read_words<<<1, 128, 0, st>>>((const unsigned*)src, (unsigned*)dst, (int)(bytes / 4));
}

// stable partition of the slots by host chunk, in three passes: counts per
// block and chunk, a scan over the blocks of each chunk, then each block
// places its slots (warp ballots give the rank among the block's slots of
// the same chunk)
constexpr int PL_BS = 1024;
constexpr int PL_MAXCHUNK = 8;
__global__ void __launch_bounds__(PL_BS) k_piece_count(const int* __restrict__ id, int n, int nchunk, int len,
                                                       int* __restrict__ cnt)
{
    __shared__ int c[PL_MAXCHUNK];
    if (threadIdx.x < PL_MAXCHUNK) c[threadIdx.x] = 0;
    __syncthreads();
    const int s = blockIdx.x * PL_BS + threadIdx.x;
    if (s < n) atomicAdd(&c[id[s] / len], 1);
    __syncthreads();
    if (threadIdx.x < nchunk) cnt[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = c[threadIdx.x];
}
// one block: exclusive scan of each chunk's counts over the blocks, offset by
// the chunk's start c*len
__global__ void __launch_bounds__(PL_BS) k_piece_scan(int* cnt, int nblocks, int nchunk, int len)
{
    __shared__ int wsum[PL_BS / 32];
    __shared__ int carry;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int c = 0; c < nchunk; c++) {
        if (threadIdx.x == 0) carry = c * len;
        __syncthreads();
        for (int b0 = 0; b0 < nblocks; b0 += PL_BS) {
            const int b = b0 + threadIdx.x;
            const int v = (b < nblocks) ? cnt[(size_t)c * nblocks + b] : 0;
            int x = v;   // inclusive warp scan
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (lane == 31) wsum[w] = x;
            __syncthreads();
            if (w == 0) {
                int z = wsum[lane];
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, z, o);
                    if (lane >= o) z += y;
                }
                wsum[lane] = z;   // inclusive over warps
            }
            __syncthreads();
            const int before = carry + (w > 0 ? wsum[w - 1] : 0) + x - v;
            if (b < nblocks) cnt[(size_t)c * nblocks + b] = before;
            __syncthreads();
            if (threadIdx.x == PL_BS - 1) carry += wsum[31];
            __syncthreads();
        }
    }
}
__global__ void __launch_bounds__(PL_BS) k_piece_place(const int* __restrict__ id, int n, int nchunk, int len,
                                                       const int* __restrict__ off, int* __restrict__ plist)
{
    __shared__ int wc[PL_BS / 32][PL_MAXCHUNK];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int s = blockIdx.x * PL_BS + threadIdx.x;
    const int c = (s < n) ? id[s] / len : -1;
    int rank = 0;
    for (int k = 0; k < nchunk; k++) {
        const unsigned m = __ballot_sync(0xffffffffu, c == k);
        if (c == k) rank = __popc(m & ((1u << lane) - 1u));
        if (lane == 0) wc[w][k] = __popc(m);
    }
    __syncthreads();
    if (c >= 0) {
        int before = 0;
        for (int v = 0; v < w; v++) before += wc[v][c];
        plist[off[(size_t)c * gridDim.x + blockIdx.x] + before + rank] = s;
    }
}
void launch_piece_list(const int* id, int n, int nchunk, int len, int* cnt, int* plist, cudaStream_t st)
{
    if (n <= 0 || nchunk < 1 || nchunk > PL_MAXCHUNK) return;
    const int nb = (n + PL_BS - 1) / PL_BS;
    NDSPH_COUNT_LAUNCH, k_piece_count<<<nb, PL_BS, 0, st>>>(id, n, nchunk, len, cnt);
    NDSPH_COUNT_LAUNCH, k_piece_scan<<<1, PL_BS, 0, st>>>(cnt, nb, nchunk, len);
    NDSPH_COUNT_LAUNCH, k_piece_place<<<nb, PL_BS, 0, st>>>(id, n, nchunk, len, cnt, plist);
}

// dt = min(C_force*dtforce, C_cour*dtcourant, 0.9*dtdrag, C_force*dtvisc)
// (stepND_leapfrog_mhd.f90:252); out = {dtcourant, dtforce, dtav, dtdrag,
// vsigmax, stressmax, dtnext}
__global__ void k_finalize_dt(Reduce* red, DevOpts o, double* out)
{
    double dtcourant = bitsd(red->dtcourant);
    double dtav = bitsd(red->dtav);
    double fhmax = bitsd(red->fhmax);
    double dtforce = 1.7976931348623157e308;
    if (fhmax > 0.0) dtforce = fmin(dtforce, sqrt(1.0 / fhmax));
    double dtdrag = 1.7976931348623157e308;
    if (o.idust == 2 && o.idrag_nature != 0 && (o.Kdrag > 0.0 || o.idrag_nature > 1))
        dtdrag = fmin(dtdrag, bitsd(red->ts_min));
    double dtvisc = 1.7976931348623157e308;
    double dtn = o.C_force * dtforce;
    dtn = fmin(dtn, o.C_cour * dtcourant);
    dtn = fmin(dtn, 0.9 * dtdrag);
    dtn = fmin(dtn, o.C_force * dtvisc);
    out[0] = dtcourant; out[1] = dtforce; out[2] = dtav; out[3] = dtdrag;
    out[4] = bitsd(red->vsigmax); out[5] = bitsd(red->stressmax); out[6] = dtn;
}
void launch_finalize_dt(Reduce* red, DevOpts o, double* out, cudaStream_t st)
{
    NDSPH_COUNT_LAUNCH, k_finalize_dt<<<1, 1, 0, st>>>(red, o, out);
}

__global__ void k_reduce_reset(Reduce* red)
{
    red->dtcourant = dbits(1.e6);
    red->dtav = dbits(1.7976931348623157e308);
    red->vsigmax = 0ull;
    red->ts_min = dbits(1.7976931348623157e308);
    red->fhmax = 0ull;
    red->stressmax = 0ull;
    red->pairs = 0ull;
    red->nclumped = 0;
}
void launch_reduce_reset(Reduce* red, cudaStream_t st)
{
    NDSPH_COUNT_LAUNCH, k_reduce_reset<<<1, 1, 0, st>>>(red);
}

// ---------------------------------------------------------------------------
// batched form: per-simulation reductions and clocks
// ---------------------------------------------------------------------------
__global__ void k_sim_reset(DevOpts o)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= o.nsim) return;
    unsigned long long* r = o.sim_red + (size_t)s * SIMRED;
    r[SR_DTC] = dbits(1.e6);
    r[SR_DTAV] = dbits(1.7976931348623157e308);
    r[SR_VSIG] = 0ull;
    r[SR_TS] = dbits(1.7976931348623157e308);
    r[SR_FH] = 0ull;
    r[SR_STRESS] = 0ull;
}
void launch_sim_reset(DevOpts o, cudaStream_t st)
{
    if (o.nsim > 0) NDSPH_COUNT_LAUNCH, k_sim_reset<<<nblk(o.nsim, 256), 256, 0, st>>>(o);
}
// dt_next per simulation (stepND_leapfrog_mhd.f90:252) and its clock;
// sim_out[s*4..] = {dtcourant, dtforce, dtnext, time}
__global__ void k_sim_finalize(DevOpts o, double* dt_next, double* sim_out)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= o.nsim) return;
    const unsigned long long* r = o.sim_red + (size_t)s * SIMRED;
    const double dtcourant = bitsd(r[SR_DTC]);
    const double fhmax = bitsd(r[SR_FH]);
    double dtforce = 1.7976931348623157e308;
    if (fhmax > 0.0) dtforce = fmin(dtforce, sqrt(1.0 / fhmax));
    double dtdrag = 1.7976931348623157e308;
    const double kdrag = o.sim_aux ? bitsd(o.sim_aux[(size_t)s * SIMAUX + SA_KDRAG]) : o.Kdrag;
    if (o.idust == 2 && o.idrag_nature != 0 && (kdrag > 0.0 || o.idrag_nature > 1)) dtdrag = fmin(dtdrag, bitsd(r[SR_TS]));
    double dtn = o.C_force * dtforce;
    dtn = fmin(dtn, o.C_cour * dtcourant);
    dtn = fmin(dtn, 0.9 * dtdrag);
    dtn = fmin(dtn, o.C_force * 1.7976931348623157e308);
    const double t = sim_out[s * 4 + 3] + o.sim_dt[s];
    dt_next[s] = dtn;
    sim_out[s * 4 + 0] = dtcourant;
    sim_out[s * 4 + 1] = dtforce;
    sim_out[s * 4 + 2] = dtn;
    sim_out[s * 4 + 3] = t;
}
void launch_sim_finalize(DevOpts o, double* dt_next, double* sim_out, cudaStream_t st)
{
    if (o.nsim > 0) NDSPH_COUNT_LAUNCH, k_sim_finalize<<<nblk(o.nsim, 256), 256, 0, st>>>(o, dt_next, sim_out);
}
// ghosts' hhmax per simulation of a periodic batch: the largest h of each
// simulation at its link (ghostND_mhd.f90:218 takes hhmax of the run's own
// particles), for every simulation (all = 1) or for the simulations whose
// last Newton-Raphson pass asked for a relink (iterate_density.f90:122-126)
__global__ void k_sim_hmax(FieldPtrs F, const int* __restrict__ sim, int n, DevOpts o)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int si = (i < n) ? sim[i] : -1;
    unsigned long long hb = (i < n) ? dbits(fmax(F.f[HH][i], 0.0)) : 0ull;
    // one atomic per warp when the warp holds one simulation (slots are
    // sorted by simulation)
    const int s0 = __shfl_sync(0xffffffffu, si, 0);
    if (__all_sync(0xffffffffu, si == s0 || si < 0)) {
        for (int off = 16; off > 0; off >>= 1) {
            const unsigned long long q = __shfl_down_sync(0xffffffffu, hb, off);
            hb = q > hb ? q : hb;
        }
        if ((threadIdx.x & 31) == 0 && s0 >= 0) atomicMax(&o.sim_aux[(size_t)s0 * SIMAUX + SA_HNOW], hb);
    } else if (si >= 0) {
        atomicMax(&o.sim_aux[(size_t)si * SIMAUX + SA_HNOW], hb);
    }
}
__global__ void k_sim_hg_apply(DevOpts o, int all)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= o.nsim) return;
    unsigned long long* x = o.sim_aux + (size_t)s * SIMAUX;
    if (all || x[SA_RELINK]) x[SA_HG] = x[SA_HNOW];
    x[SA_RELINK] = 0ull;
    x[SA_HNOW] = 0ull;
}
void launch_sim_ghost_h(FieldPtrs F, const int* sim, DevOpts o, int n, int all, cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_sim_hmax<<<nblk(n, 256), 256, 0, st>>>(F, sim, n, o);
    if (o.nsim > 0) NDSPH_COUNT_LAUNCH, k_sim_hg_apply<<<nblk(o.nsim, 256), 256, 0, st>>>(o, all);
}

// the full-pass rule per simulation of a batch (iterate_density.f90:129-133
// in each run): every simulation's first pass is full; its next pass is full
// while no particle of it converged in a full pass
__global__ void k_sim_nr_init(DevOpts o)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= o.nsim) return;
    o.sim_aux[(size_t)s * SIMAUX + SA_FULL] = 1ull;
    o.sim_aux[(size_t)s * SIMAUX + SA_CONV] = 0ull;
}
__global__ void k_sim_full_update(DevOpts o, Reduce* red)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= o.nsim) return;
    unsigned long long* x = o.sim_aux + (size_t)s * SIMAUX;
    const bool full = x[SA_FULL] != 0ull && x[SA_CONV] == 0ull;
    x[SA_FULL] = full ? 1ull : 0ull;
    x[SA_CONV] = 0ull;
    if (full) red->sim_any_full = 1;
}
void launch_sim_nr_init(DevOpts o, cudaStream_t st)
{
    if (o.nsim > 0) NDSPH_COUNT_LAUNCH, k_sim_nr_init<<<nblk(o.nsim, 256), 256, 0, st>>>(o);
}
void launch_sim_full_update(DevOpts o, Reduce* red, cudaStream_t st)
{
    if (o.nsim > 0) NDSPH_COUNT_LAUNCH, k_sim_full_update<<<nblk(o.nsim, 256), 256, 0, st>>>(o, red);
}

// x += sign * off[sim]  (tubes laid side by side along x)
__global__ void k_add_offset(FieldPtrs F, const int* sim, const double* off, int n, int sign)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    F.f[X0][i] += (double)sign * off[sim[i]];
}
void launch_add_offset(FieldPtrs F, const int* sim, const double* off, int n, int sign, cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_add_offset<<<nblk(n, 256), 256, 0, st>>>(F, sim, off, n, sign);
}

// primitive2conservative (conservative2primitive.f90:488-509): rho = dens,
// h = hfact*(m/rho)^(1/ndim)
__global__ void k_p2c_init(FieldPtrs F, DevOpts o, int n)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double rho = F.f[DENS][k];
    F.f[RHO][k] = rho;
    F.f[HH][k] = o.hfact * pow(F.f[PM][k] / (rho + 0.0), 1.0 / o.ndim);
}
void launch_p2c_init(FieldPtrs F, Side S, DevOpts o, int n, cudaStream_t st)
{
    (void)S;
    if (n > 0) NDSPH_COUNT_LAUNCH, k_p2c_init<<<nblk(n, 256), 256, 0, st>>>(F, o, n);
}
// after the density iteration: Bevol from Bfield (:608-619), en = uu (:743)
__global__ void k_p2c_post(FieldPtrs F, DevOpts o, int n)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double rho = F.f[RHO][k];
    if (o.imhd >= 11) {
        for (int d = 0; d < 3; d++) F.f[BE0 + d][k] = F.f[BF0 + d][k];
    } else if (o.imhd >= 1 && o.imhd <= 9) {
        for (int d = 0; d < 3; d++) F.f[BE0 + d][k] = F.f[BF0 + d][k] / rho;
    }
    F.f[EN][k] = F.f[UU][k];
}
void launch_p2c_post(FieldPtrs F, Side S, DevOpts o, int n, cudaStream_t st)
{
    (void)S;
    if (n > 0) NDSPH_COUNT_LAUNCH, k_p2c_post<<<nblk(n, 256), 256, 0, st>>>(F, o, n);
}


// ---------------------------------------------------------------------------
// Control kernels of the captured (CUDA graph) step.  The host loop of the
// eager step reads the Newton-Raphson counts and flags back after every pass;
// the captured step keeps those decisions on the device: a WHILE conditional
// node runs the partial passes, and every case the eager host loop handles by
// reallocating or relinking (a grid that no longer fits, a neighbour row that
// overflows, a relink, another full pass, the pass limit) sets `gfail`; the
// corrector and the dt update then skip, and the host redoes the step from the
// predicted state on the eager path.
// ---------------------------------------------------------------------------
__global__ void k_link_reset(Reduce* red)
{
    for (int d = 0; d < 3; d++) { red->xlo[d] = ~0ull; red->xhi[d] = 0ull; }
    red->hmax = 0ull;
}
void launch_link_reset(Reduce* red, cudaStream_t st)
{
    NDSPH_COUNT_LAUNCH, k_link_reset<<<1, 1, 0, st>>>(red);
}

__global__ void k_grid_check(Reduce* red, Grid g, DevOpts o)
{
    const double hmax = bitsd(red->hmax);
    double cap = 1e300;
    const double reach = (double)((g.sw - 1) / 2);
    for (int d = 0; d < o.ndim; d++) cap = fmin(cap, 0.5 * reach * g.cs[d] / (1.0 + 1.e-9));
    bool ok = (hmax > 0.0) && (hmax <= cap);
    for (int d = 0; d < o.ndim; d++) {
        if (o.periodic[d]) continue;
        const double lo = unord_bits(red->xlo[d]), hi = unord_bits(red->xhi[d]);
        const double top = g.origin[d] + g.cs[d] * (double)g.nc[d];
        if (!(lo >= g.origin[d] + g.cs[d]) || !(hi < top - g.cs[d])) ok = false;
    }
    if (!ok) red->gfail |= 1;
    red->hmax_ghost = red->hmax;   // the ghosts' hhmax is the max h at the link
}
void launch_grid_check(Reduce* red, Grid g, DevOpts o, cudaStream_t st)
{
    NDSPH_COUNT_LAUNCH, k_grid_check<<<1, 1, 0, st>>>(red, g, o);
}

__global__ void k_graph_begin(Reduce* red)
{
    red->gfail = 0;
    red->g_its = 0;
    red->g_nlist = 0;
    red->g_gate = 0;
    red->g_rebuild = 0;
}
void launch_graph_begin(Reduce* red, cudaStream_t st)
{
    NDSPH_COUNT_LAUNCH, k_graph_begin<<<1, 1, 0, st>>>(red);
}

// start of a pass: count it; the relink check of iterate_density.f90:122-126
// runs when the previous pass asked for a relink
__global__ void k_nr_pre(Reduce* red, int* d_ncalc)
{
    red->g_its += 1;
    red->g_gate = red->redolink;
    red->redolink = 0;
    red->hmax = 0ull;
    *d_ncalc = 0;
}
void launch_nr_pre(Reduce* red, int* d_ncalc, cudaStream_t st)
{
    NDSPH_COUNT_LAUNCH, k_nr_pre<<<1, 1, 0, st>>>(red, d_ncalc);
}

// the relink refreshes the ghosts' hhmax when h still fits the cells; a
// relink that needs new cells is left to the host path
__global__ void k_nr_relink_apply(Reduce* red, double cap)
{
    if (!red->g_gate) return;
    const double hmax_now = bitsd(red->hmax);
    if (hmax_now <= cap) red->hmax_ghost = red->hmax;
    else red->gfail |= 4;
}
void launch_nr_relink_apply(Reduce* red, double cap, cudaStream_t st)
{
    NDSPH_COUNT_LAUNCH, k_nr_relink_apply<<<1, 1, 0, st>>>(red, cap);
}

// end of a pass: the next active count, the row-rebuild gate, and the loop
// condition (more unconverged particles, no failure, pass limit not reached)
__global__ void k_nr_post(Reduce* red, const int* d_ncalc, int n, int its_cap, cudaGraphConditionalHandle h)
{
    const int nc = *d_ncalc;
    red->g_nlist = nc;
    const int rebuild = (red->nl_stale != 0 && red->redolink == 0) ? 1 : 0;
    red->g_rebuild = rebuild;
    if (rebuild) { red->nl_stale = 0; red->nl_overflow = 0; red->nl_maxcnt = 0; }
    if (nc > 0 && nc == n) red->gfail |= 8;               // another full pass
    if (nc > 0 && red->g_its >= its_cap) red->gfail |= 16; // pass limit of the captured loop
    const bool more = nc > 0 && red->gfail == 0;
    cudaGraphSetConditional(h, more ? 1u : 0u);
}
void launch_nr_post(Reduce* red, const int* d_ncalc, int n, int its_cap, cudaGraphConditionalHandle h,
                    cudaStream_t st)
{
    NDSPH_COUNT_LAUNCH, k_nr_post<<<1, 1, 0, st>>>(red, d_ncalc, n, its_cap, h);
}

__global__ void k_copy_active(int* dst, const int* src, const int* count, int n)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = *count;
    if (k >= c || k >= n) return;
    dst[k] = src[k];
}
void launch_copy_active(int* dst, const int* src, const int* count, int n, cudaStream_t st)
{
    if (n > 0) NDSPH_COUNT_LAUNCH, k_copy_active<<<nblk(n, 256), 256, 0, st>>>(dst, src, count, n);
}

__global__ void k_sim_dt_advance(double* dt, const double* dtnext, int nsim, const Reduce* red)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsim || red->gfail) return;
    dt[s] = dtnext[s];
}
void launch_sim_dt_advance(double* dt, const double* dtnext, int nsim, const Reduce* red, cudaStream_t st)
{
    if (nsim > 0) NDSPH_COUNT_LAUNCH, k_sim_dt_advance<<<nblk(nsim, 256), 256, 0, st>>>(dt, dtnext, nsim, red);
}

}  // namespace ndsph
