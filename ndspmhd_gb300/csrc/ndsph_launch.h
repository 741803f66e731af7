// ndsph_launch.h -- host-side launch wrappers of the device kernels.
#pragma once
#include "ndsph_common.cuh"

namespace ndsph {

// pointer table of the field slab (passed by value to kernels)
struct FieldPtrs {
    double* f[NF];
};

// per-particle int / float side arrays (sorted order unless noted)
struct Side {
    int* itype;       // particle type
    int* id;          // original (host) index of the particle in this slot
    int* ireal;       // original index of the source particle of a fixed particle (-1 none)
    int* pos_of_id;   // inverse of id
    int* numneigh;
    int* cell;        // cell id of the slot
    float4* xs;       // FP32 cell-relative position + h (screen / FP32 form)
    double* h1;       // 1/h of the pass
    int* active;      // NR active list (current pass)
    int* active_next; // NR active list (next pass)
    int* flag;        // NR converged flag scratch
    // FP32 packs of the neighbour data (FP32 form only), one float4 each:
    float4* pk_v;     // (vx, vy, vz, m)
    float4* pk_t;     // (rho, max(P,0), c_s, u)
    float4* pk_b;     // (Bx, By, Bz, gradh)
    float4* pk_a;     // (alpha1, alpha2, alpha3, h)
    // neighbour lists, one row per slot: entry k of slot i at nl[i*stride + k];
    // each entry packs (j << 5) | stencil offset of j's cell
    unsigned* nl;
    int* nl_cnt;
    // two particle types (gas + dust, 3D FP32 form): nl/nl_cnt then hold the
    // candidates of the slot's own type (the ones the density sums see) and
    // nl2/nl_cnt2 those of the other type (the drag pairs of the rates sweep)
    unsigned* nl2;
    int* nl_cnt2;
    float* hb;        // h of each slot when its list was built
    float4* xsb;      // xs of each slot when its list was built (reuse check)
    float4* xg;       // FP32 position relative to the grid origin + h (3D row build)
    int* sim;         // simulation of the slot (batched form)
};

struct SortScratch {
    int* key;         // cell id per particle (unsorted order)
    int* slot;        // rank inside the cell from the atomic count
    int* count;       // per-cell counts (ncells)
    int* start;       // exclusive scan (ncells + 1)
    int* perm;        // sorted slot -> unsorted index
    int* perm2;       // the scatter's order inside each cell (atomic, varies run to run)
    int* blocksums;   // scan scratch
    float* cell_h;    // largest h of each cell's particles (1D row-build pruning)
    int cap_cells;
    int cap_blocks;
};

// host-layout staging of the outputs a host-buffer step returns last: the
// corrected state and the rates (nullptr: not returned)
struct StepTail {
    double *x, *v, *be, *en, *hh, *al, *drhodt, *dhdt;
    double *force, *db, *dudt, *dendt, *dal, *divb, *curlb, *del2u, *gdv;
};

struct SweepArgs {
    FieldPtrs F;
    Side S;
    const int* cell_start;   // ncells + 1
    float* cell_h;           // ncells: largest h per cell (filled by the 1D row build)
    Grid g;
    DevOpts o;
    Tables t;
    Reduce* red;
    int n;
    int its;                 // NR pass number (1-based)
    int nlist;               // partial pass: entries in S.active
    int* ncalc_next;         // partial: counter of the next active list
    long long nl_ld;         // leading dimension of the list (>= n)
    int nl_stride;           // entries per particle
    float nl_skin;           // list radius = 2 max(h_i,h_j) skin (h may grow by skin before a rebuild)
    float nl_dmax;           // largest displacement since the rows were built (0 right after a build)
    int typed_rows;          // rows split by type (nl: matching types, nl2: the other type)
    int mixed;               // batched full pass over the active list: the simulations whose
                             // SA_FULL is set take the full pass's rule, the others a partial's
    // device-side control (captured step): when set, the pass number, the
    // active count and the row-build gate are read from device memory
    const int* d_its;
    const int* d_nlist;
    const int* gate;
    int graph;               // captured step: a row overflow sets gfail
    // rates sweep in pieces: when set, the sweep covers slots
    // plist[pi0 .. pi0 + pn) instead of 0 .. n, and with tail_on each
    // particle's outputs and corrected state also go to the host-order
    // staging `tail` at its host index
    const int* plist;
    int pi0, pn;
    int tail_on;
    StepTail tail;
};

// ---- link / sort (ndsph_kernels.cu) ------------------------------------------
void launch_boundary_wrap(FieldPtrs F, DevOpts o, int n, cudaStream_t st);
// max h and bounding box; skipped when `gate` is set and points to 0
void launch_hmax_bbox(FieldPtrs F, int ndim, int n, Reduce* red, unsigned long long* dst, cudaStream_t st,
                      const int* gate = nullptr);
void launch_cell_key(FieldPtrs F, Grid g, DevOpts o, int n, const int* sim, SortScratch s, Reduce* red,
                     cudaStream_t st);
void launch_scan(SortScratch s, int ncells, cudaStream_t st);
void launch_scatter_sort(SortScratch s, int n, int ncells, cudaStream_t st);
void launch_gather_fields(FieldPtrs dst, FieldPtrs src, const int* fields, int nfields, const int* perm,
                          int n, cudaStream_t st);
void launch_gather_int(int* dst, const int* src, const int* perm, int n, cudaStream_t st);
void launch_post_sort(Side S, SortScratch s, int n, int ncells, Grid g, FieldPtrs F, DevOpts o,
                      cudaStream_t st);
void launch_xs(FieldPtrs F, Side S, Grid g, DevOpts o, int n, cudaStream_t st);
// step that keeps the last link: xs relative to each slot's cell of that link
// (periodic jumps undone), max displacement since the row build, min row
// slack skin*h_build - grow*h, max h (red->hmax, red->reuse_d2, red->reuse_slack)
void launch_reuse_check(FieldPtrs F, Side S, Grid g, DevOpts o, int n, float skin, float grow, Reduce* red,
                        cudaStream_t st);

// ---- host layout <-> device slab ------------------------------------------
// AoS host-layout staging buffer (one field: stride comps) -> sorted slab fields
void launch_aos_to_slab(FieldPtrs F, int f0, int ncomp, const double* aos, int stride, const int* id, int n,
                        cudaStream_t st);
// slab fields -> host layout; particle p from slot pos[p] (pos_of_id)
void launch_slab_to_aos(double* aos, int stride, FieldPtrs F, int f0, int ncomp, const int* pos, int n,
                        cudaStream_t st);
void launch_int_to_slab(int* dst, const int* src, const int* id, int n, cudaStream_t st);
void launch_slab_to_int(int* dst, const int* src, const int* pos, int n, cudaStream_t st);
void launch_iota(int* a, int n, cudaStream_t st);
void launch_int_shift(int* dst, const int* src, int n, int add, cudaStream_t st);   // dst = src + add
void launch_fill(double* a, double v, int n, cudaStream_t st);
void launch_copy(double* dst, const double* src, int n, cudaStream_t st);

// ---- per-particle physics (ndsph_kernels.cu) --------------------------------
void launch_h1(FieldPtrs F, Side S, int n, cudaStream_t st);
// zero the hterms of non-fixed particles, save h at entry (hhin), check h > 0
void launch_density_init(FieldPtrs F, Side S, int n, Reduce* red, cudaStream_t st);
void launch_fixed_density_copy(FieldPtrs F, Side S, int n, cudaStream_t st);
void launch_eos(FieldPtrs F, Side S, DevOpts o, int n, Reduce* red, cudaStream_t st);
void launch_fixed_copy(FieldPtrs F, Side S, DevOpts o, int n, cudaStream_t st);
void launch_predictor(FieldPtrs F, Side S, DevOpts o, int n, Reduce* red, cudaStream_t st);
// states without fixed particles: part 1 = x, v, h; part 2 = Bevol, energy, alpha
void launch_predictor_part(FieldPtrs F, Side S, DevOpts o, int n, Reduce* red, int part, cudaStream_t st);
void launch_corrector(FieldPtrs F, Side S, DevOpts o, int n, Reduce* red, cudaStream_t st);
// one simulation, no fixed particles: the corrector and the next step's save
// and predictor (dt from dtnext, a device value) in one pass
void launch_corrector_predictor(FieldPtrs F, Side S, DevOpts o, int n, Reduce* red, const double* dtnext,
                                cudaStream_t st);
// slots grouped by the host chunk of their particle (chunk c = particles
// c*len .. (c+1)*len), ascending within a chunk: plist[c*len + r] is the
// r-th slot of chunk c.  cnt: scratch of nchunk * ceil(n / 1024) ints
void launch_piece_list(const int* id, int n, int nchunk, int len, int* cnt, int* plist, cudaStream_t st);
// small device -> host read into mapped pinned memory (dst: its device
// address) by a one-block kernel; bytes a multiple of 4
void launch_read_words(void* dst, const void* src, size_t bytes, cudaStream_t st);
void launch_finalize_dt(Reduce* red, DevOpts o, double* out, cudaStream_t st);
void launch_reduce_reset(Reduce* red, cudaStream_t st);
void launch_p2c_init(FieldPtrs F, Side S, DevOpts o, int n, cudaStream_t st);
void launch_p2c_post(FieldPtrs F, Side S, DevOpts o, int n, cudaStream_t st);
// batched form
void launch_sim_reset(DevOpts o, cudaStream_t st);
void launch_sim_finalize(DevOpts o, double* dt_next, double* sim_out, cudaStream_t st);
void launch_sim_ghost_h(FieldPtrs F, const int* sim, DevOpts o, int n, int all, cudaStream_t st);
void launch_sim_nr_init(DevOpts o, cudaStream_t st);
void launch_sim_full_update(DevOpts o, Reduce* red, cudaStream_t st);
void launch_add_offset(FieldPtrs F, const int* sim, const double* off, int n, int sign, cudaStream_t st);
// captured step (CUDA graph) control kernels
void launch_link_reset(Reduce* red, cudaStream_t st);
void launch_grid_check(Reduce* red, Grid g, DevOpts o, cudaStream_t st);
void launch_graph_begin(Reduce* red, cudaStream_t st);
void launch_nr_pre(Reduce* red, int* d_ncalc, cudaStream_t st);
void launch_nr_relink_apply(Reduce* red, double cap, cudaStream_t st);
void launch_nr_post(Reduce* red, const int* d_ncalc, int n, int its_cap, cudaGraphConditionalHandle h,
                    cudaStream_t st);
void launch_copy_active(int* dst, const int* src, const int* count, int n, cudaStream_t st);
void launch_sim_dt_advance(double* dt, const double* dtnext, int nsim, const Reduce* red, cudaStream_t st);

// ---- sweeps (ndsph_sweeps.cu) --------------------------------------------
void launch_density(const SweepArgs& a, bool full, cudaStream_t st);
void launch_rates(const SweepArgs& a, cudaStream_t st);
// fused step of a 1D batch, one block per tube (tubes contiguous in slots;
// tube_start[nsim+1], order[nsim] largest first; maxm the largest tube)
constexpr int TUBE_MAX = 4096;
size_t tube_smem_bytes(int maxm);
// predicted: the previous launch already ran this step's save and predictor;
// predict_next: the corrector also runs the next step's (several steps of one
// ndsph_batch_step call)
void launch_tube_step(const SweepArgs& a, const int* tube_start, const int* order, int nsim, double* dt_next,
                      double* sim_out, int maxm, bool predicted, bool predict_next, cudaStream_t st);
void launch_pack_v(const SweepArgs& a, cudaStream_t st);
void launch_build_nlist(const SweepArgs& a, cudaStream_t st);
void launch_pack_rates(const SweepArgs& a, cudaStream_t st);
// neighbour CSR for parity tests: counts (mode) then fill
void launch_neigh_count(const SweepArgs& a, int mode, long long* counts, cudaStream_t st);
void launch_neigh_fill(const SweepArgs& a, int mode, const long long* offsets, int* out, cudaStream_t st);

}  // namespace ndsph
