// ndsph_api.cu -- the C-ABI of include/ndsph.h: context, device memory,
// kernel tables and the host orchestration of link -> iterate_density ->
// conservative2primitive -> get_rates (-> leapfrog).
//
// One context = one CUDA stream on the current device.  All device memory is
// owned here (cudaMalloc at init / on growth, freed in ndsph_finalize); the
// caller's host arrays are only read and written inside the entry points.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#include "ndsph_launch.h"
#include "ndsph_mlp.h"

using namespace ndsph;

struct ndsph_ctx {
    ndsph_opts opts;
    DevOpts o;
    cudaStream_t st = nullptr;
    int device = 0;
    int cap = 0;          // particle capacity
    int n = 0;            // particles currently on the device
    // slab double buffers
    double* slab[2] = {nullptr, nullptr};
    int cur = 0;
    FieldPtrs F;          // pointer table of the current slab (HH/HNEXT may be swapped)
    // side arrays (two sets of the permuted ints)
    Side S;
    int* itype2 = nullptr;
    int* id2 = nullptr;
    int* ireal2 = nullptr;
    SortScratch srt;
    int* d_fields = nullptr;     // field index list for the gather
    // tables
    double2* tab64 = nullptr;
    float2* tab32 = nullptr;
    Tables t;
    // grid
    Grid g;
    double cell_hmax = 0.0;      // hmax the grid was built for
    double grid_cf = 1.0;        // cell size / (2 hmax) of the grid
    bool linked = false;
    // reductions
    Reduce* red = nullptr;
    Reduce* h_red = nullptr;     // pinned mirror
    double* d_dtout = nullptr;
    double* h_dtout = nullptr;
    Reduce* hd_red = nullptr;    // device addresses of the pinned mirrors (null: not mapped)
    double* hd_dtout = nullptr;
    int* h_ncalc = nullptr;      // pinned: the next pass's active count
    int* hd_ncalc = nullptr;
    int* d_ncalc = nullptr;
    // host staging
    double* d_stage = nullptr;   // n*3 doubles
    int* d_istage = nullptr;
    // host arrays the kernels read and write in place (no staging copy):
    // 1 when possible (pinned memory, or any memory where the device reads
    // pageable host memory), 0 always stage through device buffers
    int host_access = 0;
    bool pageable_access = false;
    // copy stream: staging copies overlap the layout kernels (two staging
    // buffers), and outputs final before the rates sweep go back under it
    cudaStream_t st_cp = nullptr;
    cudaEvent_t ev_cp[2] = {nullptr, nullptr}, ev_used[2] = {nullptr, nullptr}, ev_dl = nullptr;
    cudaEvent_t ev_pfork = nullptr, ev_pjoin = nullptr;   // rates pieces on two streams
    cudaStream_t st_g = nullptr;   // gathers of the staged downloads
    cudaEvent_t ev_g = nullptr;
    int stage_k = 0;
    ndsph_particles* dl_early = nullptr;   // ndsph_step: where the early outputs go
    // ndsph_step: the inputs only the EOS and the Bevol/energy/alpha predictor
    // read are uploaded on their own stream while the link and density run
    cudaStream_t st_up = nullptr;
    cudaEvent_t ev_late = nullptr, ev_up0 = nullptr;
    // late inputs staged whole, in host order (16 doubles per particle), so
    // a relink before they are used lays them out again in the new order
    double* d_stage_late = nullptr;
    struct LateField { int f0, ncomp, stride; const double* buf; };
    LateField late_f[8];
    int late_nf = 0;
    size_t late_used = 0;
    bool late_relayout = false;
    bool late_pending = false;
    bool dl_density_done = false, dl_prim_done = false;
    // device-resident steps: the last step's corrector also ran this step's
    // save and predictor (k_corrector_predictor)
    bool predicted = false;
    bool packs_valid = false;    // FP32 packs hold the last rates sweep's values of each slot
    // ndsph_step: the rates sweep runs in dl_pieces pieces, one per chunk of
    // the host arrays, and each chunk's last outputs go back while the later
    // pieces run (dl_tail: where they go; null: all after the corrector)
    ndsph_particles* dl_tail = nullptr;
    bool dl_tail_done = false;
    bool dl_x_done = false;      // positions went back before the density passes
    int dl_pieces = 8;
    int* d_plist = nullptr;      // slots grouped by host chunk
    int* d_pcnt = nullptr;       // its scratch: dl_pieces counts per 1024 slots
    double* d_arena = nullptr;   // download staging: every output field side by side
    size_t arena_cap = 0;        // doubles
    size_t arena_used = 0;
    // neighbour lists
    int nl_stride = 0;
    float nl_skin = 1.1f;
    // reuse of the rows across steps (FP32 form, one simulation): a step
    // keeps the slot order, the cells and the rows of the last link while
    // every particle has h + dmax <= skin * h_build (dmax: the largest
    // displacement since the rows were built) and hmax + dmax <= cell / 2;
    // the cells are then sized 2 hmax * skin so the stencil covers the rows'
    // radius.  The pair sums see the same pairs either way.
    int nl_reuse = 1;            // tuning switch
    int nl_sw5 = 1;              // tuning switch: FP32 form searches 5-wide stencils of half cells
    bool nl_valid = false;       // order, cells and rows match the device state
    float nl_dmax = 0.f;         // displacement bound of this step (0 after a build)
    float nl_grow = 1.005f;      // room left for Newton-Raphson growth of h
    int nl_reused = 0;           // steps that kept the last link
    int keep_fails = 0;          // consecutive failed checks
    int keep_skip = 0;           // steps left before the check is tried again
    // learned-h predictor
    float* mlp_p = nullptr;      // FP32 master weights
    float* mlp_m = nullptr;      // Adam moments
    float* mlp_v = nullptr;
    float* mlp_g = nullptr;      // gradient
    float* mlp_loss = nullptr;
    MlpFrag* mlp_frag = nullptr; // BF16 tensor-core operands
    int mlp_step = 0;
    float mlp_lr = 2.e-3f;
    int mlp_batch = 16384;
    int mlp_iters = 1;
    // the training runs on its own stream from the end of the density
    // iteration to the corrector, beside the EOS and the rates sweep
    cudaStream_t st_mlp = nullptr;
    cudaEvent_t ev_mfork = nullptr, ev_mjoin = nullptr;
    bool mlp_train_here = false;   // do_derivs starts the training after the iteration
    bool mlp_pending = false;      // training issued, not yet joined
    // batched form
    int nsim = 0;
    int* sim2 = nullptr;             // gather partner of S.sim
    unsigned long long* d_sim_red = nullptr;
    double* d_sim_dt = nullptr;
    double* d_sim_dtnext = nullptr;
    double* d_sim_out = nullptr;     // [nsim][4] dtcourant, dtforce, dtnext, time
    double* d_sim_off = nullptr;
    double* h_sim_out = nullptr;
    unsigned long long* d_sim_aux = nullptr;   // [nsim][SIMAUX] drag constant, ghosts' hhmax
    std::vector<double> h_kdrag;     // per-simulation drag constants set by the caller
    // captured batched step: two CUDA graphs (the link swaps the slabs, so
    // consecutive steps alternate between two pointer states)
    struct PtrState {
        int cur;
        FieldPtrs F;
        Side S;
        int *itype2, *id2, *ireal2, *sim2;
    };
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    PtrState gptr[2];
    int gparity = 0;
    bool gvalid = false;
    int graph_mode = 1;          // 1: one launch per batched step (fused per-tube kernel for 1D
                                 //    batches, else a captured graph); 2: captured graph; 0: eager
    // fused per-tube step (1D batches): tube slot ranges and launch order
    int* d_tube_start = nullptr;
    int* d_tube_order = nullptr;
    int tube_maxm = 0;           // largest tube; 0: the batch does not qualify
    int tube_cap = 0;
    int fsteps = 0;              // steps run by the fused per-tube kernel
    bool tubes_predicted = false;  // the last fused launch also ran the next step's predictor
    bool tubes_valid = false;    // ranges match the slot order (reset by every link)
    int gredo = 0;               // captured steps redone on the eager path
    int gsteps = 0;              // captured steps launched
    double g_hmax = 0.0;         // max h the graph's cells were sized for
    double gmargin = 1.05;       // cell size = 2 hmax gmargin at capture
    long long gl_main[2] = {0, 0};  // kernel nodes of each graph outside the loop body
    long long gl_body[2] = {0, 0};  // kernel nodes of the loop body
    int* d_live = nullptr;       // field list of the captured gather
    int nlive = 0;
    cudaStream_t st2 = nullptr;  // capture stream of the Newton-Raphson loop body
    // timing
    bool profiling = false;
    cudaEvent_t ev[16];
    ndsph_timing timing;
    ndsph_dt last_dt;
    std::string err;
    double time = 0.0, dt = 0.0;
    int nsteps = 0;
};

static thread_local std::string g_err;
namespace ndsph {
// the message ndsph_last_error(NULL) returns, for entry points without a
// context (ndsph_density_noalloc)
void set_global_error(const char* msg) { g_err = msg ? msg : ""; }
}  // namespace ndsph
static int build_nlist(ndsph_ctx* ctx);
static void link_sort_gather(ndsph_ctx* ctx, const int* d_fields, int nfields, cudaStream_t st);
static int download_density_group(ndsph_ctx* ctx, ndsph_particles* p);
static int download_prim_group(ndsph_ctx* ctx, ndsph_particles* p);
#define CK_VOID(call) do { (void)(call); } while (0)

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            if (ctx) ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);        \
            return NDSPH_E_CUDA;                                                          \
        }                                                                                 \
    } while (0)

// ---------------------------------------------------------------------------
// kernel tables, kernelND.f90:127-157 (structure), cubic spline :4143-4192 and
// normalisation :4279-4289 (truncated pi, 1D constant 0.66666666666), drag
// kernel 41 :1659-1697; slope(i) = (t(i+1)-t(i))*ddq2table with the last
// entry's slope 0 (index1 clamped to ikern, kernelND.f90:4383-4384)
// ---------------------------------------------------------------------------
static void build_tables(int ndim, std::vector<double>& w, std::vector<double>& gw, std::vector<double>& ggw,
                         std::vector<double>& wd, std::vector<double>& gwd, double& dq2, double& ddq2)
{
    const double pi = 3.141592653589;
    const double radkern = 2.0;
    dq2 = radkern * radkern / (double)IKERN;
    double cn = 0.0, cd = 0.0;
    if (ndim == 1) { cn = 0.66666666666; cd = 2.0; }
    if (ndim == 2) { cn = 10. / (7. * pi); cd = 70. / (31. * pi); }
    if (ndim == 3) { cn = 1. / pi; cd = 10. / (9. * pi); }
    w.assign(NTAB, 0.0); gw.assign(NTAB, 0.0); ggw.assign(NTAB, 0.0); wd.assign(NTAB, 0.0); gwd.assign(NTAB, 0.0);
    for (int i = 0; i <= IKERN; i++) {
        volatile double q2 = i * dq2;
        double q = sqrt(q2);
        double a = 0, b = 0, c = 0, da = 0, db = 0;
        if (q < 1.0) {
            volatile double t1 = 1.5 * q2;
            volatile double t2 = 0.75 * q;
            volatile double t3 = t2 * q2;
            a = (1. - t1) + t3;
            volatile double u1 = -3. * q;
            volatile double u2 = 2.25 * q2;
            b = u1 + u2;
            volatile double v1 = 4.5 * q;
            c = -3. + v1;
            volatile double q4 = q2 * q2;
            volatile double s1 = 1.5 * q4;
            volatile double s2 = 0.75 * q4;
            volatile double s3 = s2 * q;
            da = (q2 - s1) + s3;
            volatile double r1 = 2. * q;
            volatile double r2 = 6. * q2;
            volatile double r3 = r2 * q;
            volatile double r4 = 3.75 * q4;
            db = (r1 - r3) + r4;
        } else if (q <= 2.0) {
            volatile double tt = 2. - q;
            volatile double t2 = tt * tt;
            volatile double t3 = t2 * tt;
            a = 0.25 * t3;
            b = -0.75 * t2;
            c = 1.5 * tt;
            volatile double x1 = 0.25 * q2;
            da = x1 * t3;
            volatile double y1 = 0.5 * q;
            volatile double y2 = y1 * t3;
            volatile double y3 = 0.75 * q2;
            volatile double y4 = y3 * t2;
            db = y2 - y4;
        }
        w[i] = cn * a; gw[i] = cn * b; ggw[i] = cn * c; wd[i] = cd * da; gwd[i] = cd * db;
    }
    ddq2 = 1. / dq2;
}

static void pack_tab(const std::vector<double>& t, double ddq2, double2* out64, float2* out32)
{
    for (int i = 0; i <= IKERN; i++) {
        int i1 = std::min(i + 1, IKERN);
        volatile double diff = t[i1] - t[i];
        double slope = diff * ddq2;
        out64[i] = make_double2(t[i], slope);
        out32[i] = make_float2((float)t[i], (float)slope);
    }
}

extern "C" int ndsph_kernel_tables(int32_t ndim, double* out)
{
    if (ndim < 1 || ndim > 3 || !out) return NDSPH_E_ARG;
    std::vector<double> w, gw, ggw, wd, gwd;
    double dq2, ddq2;
    build_tables(ndim, w, gw, ggw, wd, gwd, dq2, ddq2);
    memcpy(out + 0 * NTAB, w.data(), NTAB * 8);
    memcpy(out + 1 * NTAB, gw.data(), NTAB * 8);
    memcpy(out + 2 * NTAB, ggw.data(), NTAB * 8);
    memcpy(out + 3 * NTAB, wd.data(), NTAB * 8);
    memcpy(out + 4 * NTAB, gwd.data(), NTAB * 8);
    return 0;
}

extern "C" void ndsph_default_opts(ndsph_opts* o, int32_t ndim)
{
    memset(o, 0, sizeof(*o));
    o->ndim = ndim;
    o->xmax[0] = o->xmax[1] = o->xmax[2] = 1.0;
    o->hfact = 1.2; o->tolh = 1.e-3; o->psep = 0.01; o->maxdensits = 250;
    o->imhd = 0; o->imagforce = 2; o->iener = 2; o->iav = 2;
    o->iavlim[0] = 2; o->iavlim[1] = 1; o->iavlim[2] = 0;
    o->alphamin = 0.1; o->alphaumin = 0.0; o->alphaBmin = 1.0; o->beta = 2.0; o->avdecayconst = 0.1;
    o->gamma = 5. / 3.; o->polyk = 1.0; o->C_cour = 0.3; o->C_force = 0.25;
}

extern "C" const char* ndsph_last_error(ndsph_ctx* ctx)
{
    return ctx ? ctx->err.c_str() : g_err.c_str();
}

static int check_opts(const ndsph_opts* p, std::string& why)
{
    if (p->ndim < 1 || p->ndim > 3) { why = "ndim must be 1..3"; return NDSPH_E_ARG; }
    for (int d = 0; d < p->ndim; d++) {
        if (p->ibound[d] != 0 && p->ibound[d] != 1 && p->ibound[d] != 3) {
            why = "ibound must be 0, 1 or 3 (reflective/shearing ghosts are out of scope)";
            return NDSPH_E_ARG;
        }
        if (p->ibound[d] == 3 && !(p->xmax[d] > p->xmin[d])) { why = "periodic box with xmax <= xmin"; return NDSPH_E_ARG; }
    }
    if (!(p->imhd == 0 || p->imhd == 1 || p->imhd == 11)) { why = "imhd must be 0, 1 or 11"; return NDSPH_E_ARG; }
    if (p->imhd != 0 && p->imagforce != 2) { why = "imagforce must be 2"; return NDSPH_E_ARG; }
    if (!(p->iener == 0 || p->iener == 2)) { why = "iener must be 0 or 2"; return NDSPH_E_ARG; }
    if (!(p->iav == 2)) { why = "iav must be 2"; return NDSPH_E_ARG; }
    if (!(p->idust == 0 || p->idust == 2)) { why = "idust must be 0 or 2"; return NDSPH_E_ARG; }
    if (p->idust == 2 && p->idrag_nature != 1) { why = "idrag_nature must be 1"; return NDSPH_E_ARG; }
    if (p->iavlim[0] == 3 || p->iavlim[2] != 0) { why = "iavlim must be (0|1|2, *, 0)"; return NDSPH_E_ARG; }
    if (p->precision != NDSPH_PREC_FP64 && p->precision != NDSPH_PREC_FP32) { why = "bad precision"; return NDSPH_E_ARG; }
    return 0;
}

static void set_devopts(ndsph_ctx* ctx)
{
    const ndsph_opts& p = ctx->opts;
    DevOpts& o = ctx->o;
    memset(&o, 0, sizeof(o));
    o.ndim = p.ndim;
    o.has_fixed = 0;
    for (int d = 0; d < 3; d++) {
        o.ibound[d] = (d < p.ndim) ? p.ibound[d] : 0;
        o.periodic[d] = (d < p.ndim && p.ibound[d] == 3) ? 1 : 0;
        o.xmin[d] = p.xmin[d]; o.xmax[d] = p.xmax[d];
        o.L[d] = p.xmax[d] - p.xmin[d];
        if (d < p.ndim && p.ibound[d] == 1) o.has_fixed = 1;
    }
    o.hfact = p.hfact; o.tolh = p.tolh; o.psep = p.psep; o.maxdensits = p.maxdensits;
    o.imhd = p.imhd; o.imagforce = p.imagforce; o.iener = p.iener; o.iav = p.iav;
    for (int k = 0; k < 3; k++) o.iavlim[k] = p.iavlim[k];
    o.alphamin = p.alphamin; o.alphaumin = p.alphaumin; o.alphaBmin = p.alphaBmin;
    o.beta = p.beta; o.avdecayconst = p.avdecayconst;
    o.gamma = p.gamma; o.polyk = p.polyk;
    // initialiseND_mhd.f90:168-172
    o.avfact = (fabs(p.gamma - 1.) > 1.e-3) ? log(4.) / (log((p.gamma + 1.) / (p.gamma - 1.))) : 1.0;
    o.idust = p.idust; o.idrag_nature = p.idrag_nature; o.Kdrag = p.Kdrag;
    o.C_cour = p.C_cour; o.C_force = p.C_force; o.precision = p.precision;
    o.learned = p.learned_h ? 1 : 0;
}

static void free_particles(ndsph_ctx* ctx)
{
    void* ptrs[] = {ctx->slab[0], ctx->slab[1], ctx->S.itype, ctx->S.id, ctx->S.ireal, ctx->S.pos_of_id,
                    ctx->S.numneigh, ctx->S.cell, ctx->S.xs, ctx->S.h1, ctx->S.active, ctx->S.active_next,
                    ctx->S.flag, ctx->itype2, ctx->id2, ctx->ireal2, ctx->srt.key, ctx->srt.slot, ctx->srt.perm, ctx->srt.perm2,
                    ctx->d_stage, ctx->d_stage_late, ctx->d_istage, ctx->S.pk_v, ctx->S.pk_t, ctx->S.pk_b, ctx->S.pk_a,
                    ctx->S.nl, ctx->S.nl_cnt, ctx->S.nl2, ctx->S.nl_cnt2, ctx->S.hb, ctx->S.xsb, ctx->S.xg, ctx->S.sim, ctx->sim2, ctx->d_plist,
                    ctx->d_pcnt};
    for (void* p : ptrs) if (p) cudaFree(p);
    ctx->slab[0] = ctx->slab[1] = nullptr;
    memset(&ctx->S, 0, sizeof(ctx->S));
    ctx->itype2 = ctx->id2 = ctx->ireal2 = nullptr;
    ctx->sim2 = nullptr;
    ctx->srt.key = ctx->srt.slot = ctx->srt.perm = ctx->srt.perm2 = nullptr;
    ctx->d_stage = nullptr; ctx->d_istage = nullptr; ctx->d_stage_late = nullptr;
    ctx->d_plist = ctx->d_pcnt = nullptr;
    ctx->cap = 0;
}

static void set_field_ptrs(ndsph_ctx* ctx)
{
    for (int f = 0; f < NF; f++) ctx->F.f[f] = ctx->slab[ctx->cur] + (size_t)f * ctx->cap;
}

static int ensure_capacity(ndsph_ctx* ctx, int n)
{
    if (n <= ctx->cap) return 0;
    free_particles(ctx);
    int cap = std::max(n, 1024);
    size_t sz = (size_t)NF * cap * sizeof(double);
    CK(cudaMalloc(&ctx->slab[0], sz));
    CK(cudaMalloc(&ctx->slab[1], sz));
    CK(cudaMemsetAsync(ctx->slab[0], 0, sz, ctx->st));
    CK(cudaMemsetAsync(ctx->slab[1], 0, sz, ctx->st));
    size_t ib = sizeof(int) * (size_t)cap;
    CK(cudaMalloc(&ctx->S.itype, ib)); CK(cudaMalloc(&ctx->S.id, ib)); CK(cudaMalloc(&ctx->S.ireal, ib));
    CK(cudaMalloc(&ctx->S.pos_of_id, ib)); CK(cudaMalloc(&ctx->S.numneigh, ib)); CK(cudaMalloc(&ctx->S.cell, ib));
    CK(cudaMalloc(&ctx->S.xs, sizeof(float4) * (size_t)cap)); CK(cudaMalloc(&ctx->S.h1, sizeof(double) * (size_t)cap));
    CK(cudaMalloc(&ctx->S.active, ib)); CK(cudaMalloc(&ctx->S.active_next, ib)); CK(cudaMalloc(&ctx->S.flag, ib));
    CK(cudaMalloc(&ctx->itype2, ib)); CK(cudaMalloc(&ctx->id2, ib)); CK(cudaMalloc(&ctx->ireal2, ib));
    CK(cudaMalloc(&ctx->srt.key, ib)); CK(cudaMalloc(&ctx->srt.slot, ib)); CK(cudaMalloc(&ctx->srt.perm, ib));
    CK(cudaMalloc(&ctx->srt.perm2, ib));
    CK(cudaMalloc(&ctx->d_stage, sizeof(double) * 6 * (size_t)cap));   // two staging buffers
    CK(cudaMalloc(&ctx->d_stage_late, sizeof(double) * 16 * (size_t)cap));
    CK(cudaMalloc(&ctx->S.pk_v, sizeof(float4) * (size_t)cap));
    CK(cudaMalloc(&ctx->S.pk_t, sizeof(float4) * (size_t)cap));
    CK(cudaMalloc(&ctx->S.pk_b, sizeof(float4) * (size_t)cap));
    CK(cudaMalloc(&ctx->S.pk_a, sizeof(float4) * (size_t)cap));
    CK(cudaMalloc(&ctx->S.nl_cnt, ib));
    CK(cudaMalloc(&ctx->S.nl_cnt2, ib));
    CK(cudaMalloc(&ctx->S.sim, ib));
    CK(cudaMalloc(&ctx->sim2, ib));
    CK(cudaMalloc(&ctx->d_plist, ib));
    CK(cudaMalloc(&ctx->d_pcnt, sizeof(int) * 8 * ((size_t)cap / 1024 + 1)));
    CK(cudaMemsetAsync(ctx->S.sim, 0, ib, ctx->st));
    CK(cudaMalloc(&ctx->S.hb, sizeof(float) * (size_t)cap));
    CK(cudaMalloc(&ctx->S.xsb, sizeof(float4) * (size_t)cap));
    CK(cudaMalloc(&ctx->S.xg, sizeof(float4) * (size_t)cap));
    ctx->S.nl = nullptr;
    ctx->S.nl2 = nullptr;
    ctx->nl_valid = false;
    ctx->nl_stride = 0;
    CK(cudaMalloc(&ctx->d_istage, ib));
    CK(cudaMemsetAsync(ctx->S.numneigh, 0, ib, ctx->st));
    ctx->cap = cap;
    ctx->cur = 0;
    set_field_ptrs(ctx);
    ctx->linked = false;
    return 0;
}

static int ensure_cells(ndsph_ctx* ctx, int ncells)
{
    if (ncells + 1 <= ctx->srt.cap_cells) return 0;
    if (ctx->srt.count) cudaFree(ctx->srt.count);
    if (ctx->srt.start) cudaFree(ctx->srt.start);
    if (ctx->srt.blocksums) cudaFree(ctx->srt.blocksums);
    if (ctx->srt.cell_h) cudaFree(ctx->srt.cell_h);
    int cap = std::max(ncells + 1, 4096);
    cap = cap + cap / 4;
    CK(cudaMalloc(&ctx->srt.count, sizeof(int) * (size_t)cap));
    CK(cudaMalloc(&ctx->srt.start, sizeof(int) * (size_t)(cap + 1)));
    CK(cudaMalloc(&ctx->srt.cell_h, sizeof(float) * (size_t)cap));
    int nb = (cap + 4095) / 4096 + 1;
    CK(cudaMalloc(&ctx->srt.blocksums, sizeof(int) * (size_t)nb));
    ctx->srt.cap_cells = cap;
    ctx->srt.cap_blocks = nb;
    return 0;
}

extern "C" int ndsph_init(ndsph_ctx** out, const ndsph_opts* opts, int32_t nmax)
{
    if (!out || !opts) return NDSPH_E_ARG;
    std::string why;
    int rc = check_opts(opts, why);
    if (rc) { g_err = why; return rc; }
    ndsph_ctx* ctx = new ndsph_ctx();
    ctx->opts = *opts;
    set_devopts(ctx);
    memset(&ctx->S, 0, sizeof(ctx->S));
    memset(&ctx->srt, 0, sizeof(ctx->srt));
    memset(&ctx->timing, 0, sizeof(ctx->timing));
    memset(&ctx->last_dt, 0, sizeof(ctx->last_dt));
    cudaError_t e = cudaGetDevice(&ctx->device);
    if (e != cudaSuccess) { g_err = cudaGetErrorString(e); delete ctx; return NDSPH_E_CUDA; }
    {
        int pa = 0;
        if (cudaDeviceGetAttribute(&pa, cudaDevAttrPageableMemoryAccess, ctx->device) == cudaSuccess)
            ctx->pageable_access = pa != 0;
        cudaGetLastError();
    }
    // the gathers of the downloads run on their own stream at the highest
    // priority (their blocks go in as the sweeps' blocks retire), ahead of
    // the copies that wait for them one by one on the copy stream
    int prio_lo = 0, prio_hi = 0;
    if (cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi) != cudaSuccess) prio_hi = 0;
    if (cudaStreamCreateWithFlags(&ctx->st_cp, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithPriority(&ctx->st_g, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_g, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_cp[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_cp[1], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_used[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_used[1], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_dl, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_pfork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_pjoin, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->st_up, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_late, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_up0, cudaEventDisableTiming) != cudaSuccess) {
        g_err = "stream/event creation failed";
        delete ctx;
        return NDSPH_E_CUDA;
    }
    e = cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) { g_err = cudaGetErrorString(e); delete ctx; return NDSPH_E_CUDA; }
    for (int k = 0; k < 16; k++) cudaEventCreate(&ctx->ev[k]);
    // tables (setkernels / setkerndrag)
    std::vector<double> w, gw, ggw, wd, gwd;
    double dq2, ddq2;
    build_tables(opts->ndim, w, gw, ggw, wd, gwd, dq2, ddq2);
    std::vector<double2> h64(4 * NTAB);
    std::vector<float2> h32(4 * NTAB);
    pack_tab(w, ddq2, &h64[0 * NTAB], &h32[0 * NTAB]);
    pack_tab(gw, ddq2, &h64[1 * NTAB], &h32[1 * NTAB]);
    pack_tab(ggw, ddq2, &h64[2 * NTAB], &h32[2 * NTAB]);
    pack_tab(wd, ddq2, &h64[3 * NTAB], &h32[3 * NTAB]);
    if (cudaMalloc(&ctx->tab64, sizeof(double2) * 4 * NTAB) != cudaSuccess ||
        cudaMalloc(&ctx->tab32, sizeof(float2) * 4 * NTAB) != cudaSuccess ||
        cudaMalloc(&ctx->red, sizeof(Reduce)) != cudaSuccess ||
        cudaMallocHost(&ctx->h_red, sizeof(Reduce)) != cudaSuccess ||
        cudaMalloc(&ctx->d_dtout, sizeof(double) * 8) != cudaSuccess ||
        cudaMallocHost(&ctx->h_dtout, sizeof(double) * 8) != cudaSuccess ||
        cudaMallocHost(&ctx->h_ncalc, sizeof(int) * 4) != cudaSuccess ||
        cudaMalloc(&ctx->d_ncalc, sizeof(int) * 4) != cudaSuccess ||
        cudaMalloc(&ctx->d_fields, sizeof(int) * NF) != cudaSuccess) {
        g_err = "cudaMalloc failed in ndsph_init";
        ndsph_finalize(ctx);
        return NDSPH_E_CUDA;
    }
    if (cudaHostGetDevicePointer((void**)&ctx->hd_red, ctx->h_red, 0) != cudaSuccess ||
        cudaHostGetDevicePointer((void**)&ctx->hd_dtout, ctx->h_dtout, 0) != cudaSuccess ||
        cudaHostGetDevicePointer((void**)&ctx->hd_ncalc, ctx->h_ncalc, 0) != cudaSuccess) {
        cudaGetLastError();
        ctx->hd_red = nullptr;
        ctx->hd_dtout = nullptr;
        ctx->hd_ncalc = nullptr;
    }
    cudaMemcpy(ctx->tab64, h64.data(), sizeof(double2) * 4 * NTAB, cudaMemcpyHostToDevice);
    cudaMemcpy(ctx->tab32, h32.data(), sizeof(float2) * 4 * NTAB, cudaMemcpyHostToDevice);
    cudaMemset(ctx->red, 0, sizeof(Reduce));
    ctx->t.w = ctx->tab64 + 0 * NTAB; ctx->t.gw = ctx->tab64 + 1 * NTAB;
    ctx->t.ggw = ctx->tab64 + 2 * NTAB; ctx->t.wdrag = ctx->tab64 + 3 * NTAB;
    ctx->t.wf = ctx->tab32 + 0 * NTAB; ctx->t.gwf = ctx->tab32 + 1 * NTAB;
    ctx->t.ggwf = ctx->tab32 + 2 * NTAB; ctx->t.wdragf = ctx->tab32 + 3 * NTAB;
    ctx->t.dq2table = dq2; ctx->t.ddq2table = ddq2;
    ctx->t.dq2tablef = (float)dq2; ctx->t.ddq2tablef = (float)ddq2;
    ctx->t.cnormf = (float)w[0];
    if (opts->learned_h) {
        if (cudaMalloc(&ctx->mlp_p, sizeof(float) * MLP_NPARAM) != cudaSuccess ||
            cudaMalloc(&ctx->mlp_m, sizeof(float) * MLP_NPARAM) != cudaSuccess ||
            cudaMalloc(&ctx->mlp_v, sizeof(float) * MLP_NPARAM) != cudaSuccess ||
            cudaMalloc(&ctx->mlp_g, sizeof(float) * MLP_NPARAM) != cudaSuccess ||
            cudaMalloc(&ctx->mlp_loss, sizeof(float)) != cudaSuccess ||
            cudaMalloc(&ctx->mlp_frag, sizeof(MlpFrag)) != cudaSuccess) {
            g_err = "cudaMalloc failed (learned h)";
            ndsph_finalize(ctx);
            return NDSPH_E_CUDA;
        }
        std::vector<float> p0;
        mlp_init_params(p0, 12345u);
        cudaMemcpy(ctx->mlp_p, p0.data(), sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice);
        cudaMemset(ctx->mlp_m, 0, sizeof(float) * MLP_NPARAM);
        cudaMemset(ctx->mlp_v, 0, sizeof(float) * MLP_NPARAM);
        cudaMemset(ctx->mlp_g, 0, sizeof(float) * MLP_NPARAM);
        cudaMemset(ctx->mlp_loss, 0, sizeof(float));
        launch_mlp_pack(ctx->mlp_p, ctx->mlp_frag, ctx->st);
        cudaStreamSynchronize(ctx->st);
    }
    if (nmax > 0 && ensure_capacity(ctx, nmax)) {
        g_err = ctx->err;
        ndsph_finalize(ctx);
        return NDSPH_E_CUDA;
    }
    *out = ctx;
    return 0;
}

extern "C" int ndsph_finalize(ndsph_ctx* ctx)
{
    if (!ctx) return 0;
    if (ctx->st_mlp) { cudaStreamSynchronize(ctx->st_mlp); cudaStreamDestroy(ctx->st_mlp); }
    if (ctx->ev_mfork) cudaEventDestroy(ctx->ev_mfork);
    if (ctx->ev_mjoin) cudaEventDestroy(ctx->ev_mjoin);
    if (ctx->st) cudaStreamSynchronize(ctx->st);
    free_particles(ctx);
    void* ptrs[] = {ctx->tab64, ctx->tab32, ctx->red, ctx->d_dtout, ctx->d_ncalc, ctx->d_fields,
                    ctx->srt.count, ctx->srt.start, ctx->srt.blocksums, ctx->srt.cell_h, ctx->mlp_p, ctx->mlp_m, ctx->mlp_v,
                    ctx->mlp_g, ctx->mlp_loss, ctx->mlp_frag, ctx->d_sim_red, ctx->d_sim_dt, ctx->d_sim_dtnext,
                    ctx->d_sim_out, ctx->d_sim_off, ctx->d_sim_aux};
    for (void* p : ptrs) if (p) cudaFree(p);
    if (ctx->h_red) cudaFreeHost(ctx->h_red);
    if (ctx->d_arena) cudaFree(ctx->d_arena);
    if (ctx->h_dtout) cudaFreeHost(ctx->h_dtout);
    if (ctx->h_ncalc) cudaFreeHost(ctx->h_ncalc);
    if (ctx->h_sim_out) cudaFreeHost(ctx->h_sim_out);
    for (int k = 0; k < 16; k++) if (ctx->ev[k]) cudaEventDestroy(ctx->ev[k]);
    for (int k = 0; k < 2; k++) if (ctx->gexec[k]) cudaGraphExecDestroy(ctx->gexec[k]);
    if (ctx->st_cp) { cudaStreamSynchronize(ctx->st_cp); cudaStreamDestroy(ctx->st_cp); }
    if (ctx->st_up) { cudaStreamSynchronize(ctx->st_up); cudaStreamDestroy(ctx->st_up); }
    if (ctx->st_g) { cudaStreamSynchronize(ctx->st_g); cudaStreamDestroy(ctx->st_g); }
    if (ctx->ev_late) cudaEventDestroy(ctx->ev_late);
    if (ctx->ev_up0) cudaEventDestroy(ctx->ev_up0);
    for (cudaEvent_t ev : {ctx->ev_cp[0], ctx->ev_cp[1], ctx->ev_used[0], ctx->ev_used[1], ctx->ev_dl,
                            ctx->ev_pfork, ctx->ev_pjoin, ctx->ev_g})
        if (ev) cudaEventDestroy(ev);
    if (ctx->d_live) cudaFree(ctx->d_live);
    if (ctx->d_tube_start) cudaFree(ctx->d_tube_start);
    if (ctx->d_tube_order) cudaFree(ctx->d_tube_order);
    if (ctx->st2) cudaStreamDestroy(ctx->st2);
    if (ctx->st) cudaStreamDestroy(ctx->st);
    delete ctx;
    return 0;
}

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
// the reductions (and dt results) the host reads between kernels: a
// one-block kernel writes them into the mapped pinned mirror, so the read is
// not queued behind the bulk output copies on the copy engines
static_assert(sizeof(Reduce) % 4 == 0, "Reduce is read back in 4-byte words");
static cudaError_t read_red(ndsph_ctx* ctx, const Reduce* src, cudaStream_t st)
{
    if (ctx->hd_red) {
        launch_read_words(ctx->hd_red, src, sizeof(Reduce), st);
        return cudaGetLastError();
    }
    return cudaMemcpyAsync(ctx->h_red, src, sizeof(Reduce), cudaMemcpyDeviceToHost, st);
}
static cudaError_t read_dtout(ndsph_ctx* ctx, cudaStream_t st)
{
    if (ctx->hd_dtout) {
        launch_read_words(ctx->hd_dtout, ctx->d_dtout, sizeof(double) * 8, st);
        return cudaGetLastError();
    }
    return cudaMemcpyAsync(ctx->h_dtout, ctx->d_dtout, sizeof(double) * 8, cudaMemcpyDeviceToHost, st);
}

// the message of a status raised by a kernel, naming the reference's stop
// site and the (1-based) particle that raised it first
static std::string device_err_msg(int code, int index)
{
    const char* what = "device error";
    switch (code) {
    case NDSPH_E_H_NONPOS: what = "h <= 0 in density call (iterate_density.f90:99-102)"; break;
    case NDSPH_E_RHO_NONPOS: what = "rho <= 0 (iterate_density.f90:168-170)"; break;
    case NDSPH_E_NOT_CONVERGED: what = "density not converged (iterate_density.f90:349-351)"; break;
    case NDSPH_E_VSIG_DET: what = "rates: vsig det < 0 (ratesND_mhd.f90:1422-1429)"; break;
    case NDSPH_E_NAN: what = "non-finite value"; break;
    case NDSPH_E_CLUMP: what = "rates: dx = 0 between particles of one type (ratesND_mhd.f90:419-424)"; break;
    case NDSPH_E_U_NEG: what = "eos: u_therm -ve (eos.f90:66-72)"; break;
    default: break;
    }
    char buf[200];
    snprintf(buf, sizeof buf, "%s: status %d at particle %d", what, code, index + 1);
    return buf;
}

static int sync_red(ndsph_ctx* ctx)
{
    CK(read_red(ctx, ctx->red, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    if (ctx->h_red->err) {
        const int code = ctx->h_red->err;
        ctx->err = device_err_msg(code, ctx->h_red->err_index);
        return code;
    }
    return 0;
}

// Device address of a host array the kernels may access in place: pinned
// memory (cudaHostAlloc / cudaHostRegister) is mapped into the device's
// address space, and where the device reads pageable memory (Grace with
// NVLink-C2C and address translation) any host pointer is; the layout
// kernels then read and write the caller's arrays directly over the
// coherent link.  nullptr: stage through a device buffer.
static const void* host_view(ndsph_ctx* ctx, const void* host)
{
    if (!ctx->host_access || !host) return nullptr;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, host) == cudaSuccess) {
        if (at.type == cudaMemoryTypeHost && at.devicePointer) return at.devicePointer;
        if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) return host;
    } else {
        cudaGetLastError();
    }
    return ctx->pageable_access ? host : nullptr;
}

// host array (AoS, `stride` doubles per particle) -> slab fields; slot k
// takes particle id[k] (id = nullptr: particle k)
static int upload_aos(ndsph_ctx* ctx, const double* host, int f0, int ncomp, int stride, int n,
                      const int* id = nullptr)
{
    if (!host) return 0;
    const double* src = (const double*)host_view(ctx, host);
    if (src) {
        launch_aos_to_slab(ctx->F, f0, ncomp, src, stride, id, n, ctx->st);
        return 0;
    }
    // copy into one staging buffer on the copy stream while the layout kernel
    // of the previous array reads the other one
    const int b = (ctx->stage_k++) & 1;
    double* buf = ctx->d_stage + (size_t)b * 3 * ctx->cap;
    CK(cudaStreamWaitEvent(ctx->st_cp, ctx->ev_used[b], 0));
    CK(cudaMemcpyAsync(buf, host, sizeof(double) * (size_t)stride * n, cudaMemcpyHostToDevice, ctx->st_cp));
    CK(cudaEventRecord(ctx->ev_cp[b], ctx->st_cp));
    CK(cudaStreamWaitEvent(ctx->st, ctx->ev_cp[b], 0));
    launch_aos_to_slab(ctx->F, f0, ncomp, buf, stride, id, n, ctx->st);
    CK(cudaEventRecord(ctx->ev_used[b], ctx->st));
    return 0;
}
// an input of the host-buffer step that the link and the density passes do
// not read: copied whole into the late staging (host order) and laid out on
// the upload stream, behind the early ones.  A relink before the main stream
// uses them lays them out again from the staging in the new order.
static int upload_aos_late(ndsph_ctx* ctx, const double* host, int f0, int ncomp, int stride, int n,
                           const int* id)
{
    if (!host) return 0;
    if (const double* src = (const double*)host_view(ctx, host)) {
        launch_aos_to_slab(ctx->F, f0, ncomp, src, stride, id, n, ctx->st_up);
        if (ctx->late_nf < 8) ctx->late_f[ctx->late_nf++] = {f0, ncomp, stride, src};
        return 0;
    }
    const size_t need = (size_t)stride * n;
    if (ctx->late_used + need > (size_t)16 * ctx->cap || ctx->late_nf >= 8) {
        ctx->err = "late staging overflow";
        return NDSPH_E_ARG;
    }
    double* buf = ctx->d_stage_late + ctx->late_used;
    ctx->late_used += need;
    CK(cudaMemcpyAsync(buf, host, sizeof(double) * need, cudaMemcpyHostToDevice, ctx->st_up));
    launch_aos_to_slab(ctx->F, f0, ncomp, buf, stride, id, n, ctx->st_up);
    ctx->late_f[ctx->late_nf++] = {f0, ncomp, stride, buf};
    return 0;
}

// the late inputs of a host-buffer step have arrived: the main stream waits
// for them (laying them out again in the current slot order when a relink
// came in between) and runs their part of the predictor (before the EOS)
static int wait_late(ndsph_ctx* ctx)
{
    if (!ctx->late_pending) return 0;
    ctx->late_pending = false;
    CK(cudaStreamWaitEvent(ctx->st, ctx->ev_late, 0));
    if (ctx->late_relayout) {
        for (int k = 0; k < ctx->late_nf; k++) {
            const auto& L = ctx->late_f[k];
            launch_aos_to_slab(ctx->F, L.f0, L.ncomp, L.buf, L.stride, ctx->S.id, ctx->n, ctx->st);
        }
        ctx->late_relayout = false;
    }
    launch_predictor_part(ctx->F, ctx->S, ctx->o, ctx->n, ctx->red, 2, ctx->st);
    CK(cudaGetLastError());
    return 0;
}

// downloads are staged in an arena and copied out asynchronously; the
// caller synchronises once (download_end)
// room for `need` more doubles in the arena; growing it first finishes the
// pending copies out of it (the staging handed out before is then free)
static int arena_reserve(ndsph_ctx* ctx, size_t need)
{
    if (ctx->arena_used + need <= ctx->arena_cap) return 0;
    CK(cudaStreamSynchronize(ctx->st));
    CK(cudaStreamSynchronize(ctx->st_cp));
    if (ctx->d_arena) CK(cudaFree(ctx->d_arena));
    ctx->d_arena = nullptr;
    size_t cap = std::max(std::max(ctx->arena_cap * 2, (size_t)ctx->cap * 80), need);
    CK(cudaMalloc(&ctx->d_arena, sizeof(double) * cap));
    ctx->arena_cap = cap;
    ctx->arena_used = 0;
    return 0;
}
static int download_aos(ndsph_ctx* ctx, double* host, int f0, int ncomp, int stride, int n)
{
    if (!host) return 0;
    if (double* direct = (double*)host_view(ctx, host)) {
        launch_slab_to_aos(direct, stride, ctx->F, f0, ncomp, ctx->S.pos_of_id, n, ctx->st);
        return 0;
    }
    const size_t need = (size_t)stride * n;
    int rc = arena_reserve(ctx, need);
    if (rc) return rc;
    double* dst = ctx->d_arena + ctx->arena_used;
    ctx->arena_used += need;
    // the gather runs on the gather stream beside whatever the main stream
    // does next (a field is downloaded once it is final for the call), its
    // copy on the copy stream behind it
    CK(cudaEventRecord(ctx->ev_dl, ctx->st));
    CK(cudaStreamWaitEvent(ctx->st_g, ctx->ev_dl, 0));
    launch_slab_to_aos(dst, stride, ctx->F, f0, ncomp, ctx->S.pos_of_id, n, ctx->st_g);
    CK(cudaEventRecord(ctx->ev_g, ctx->st_g));
    CK(cudaStreamWaitEvent(ctx->st_cp, ctx->ev_g, 0));
    CK(cudaMemcpyAsync(host, dst, sizeof(double) * need, cudaMemcpyDeviceToHost, ctx->st_cp));
    return 0;
}
// as download_aos, with the gather on the main stream (ordered before what
// the main stream does next, e.g. a relink that rewrites pos_of_id) and the
// copy on the copy stream
static int download_aos_ordered(ndsph_ctx* ctx, double* host, int f0, int ncomp, int stride, int n)
{
    if (!host) return 0;
    const size_t need = (size_t)stride * n;
    int rc = arena_reserve(ctx, need);
    if (rc) return rc;
    double* dst = ctx->d_arena + ctx->arena_used;
    ctx->arena_used += need;
    launch_slab_to_aos(dst, stride, ctx->F, f0, ncomp, ctx->S.pos_of_id, n, ctx->st);
    CK(cudaEventRecord(ctx->ev_dl, ctx->st));
    CK(cudaStreamWaitEvent(ctx->st_cp, ctx->ev_dl, 0));
    CK(cudaMemcpyAsync(host, dst, sizeof(double) * need, cudaMemcpyDeviceToHost, ctx->st_cp));
    return 0;
}
static int download_end(ndsph_ctx* ctx)
{
    CK(cudaStreamSynchronize(ctx->st));
    CK(cudaStreamSynchronize(ctx->st_cp));
    ctx->arena_used = 0;
    return 0;
}
static int download_int(ndsph_ctx* ctx, int* host, const int* dsrc, int n, bool is_index)
{
    if (!host) return download_end(ctx);
    if (int* direct = (int*)host_view(ctx, host)) {
        launch_slab_to_int(direct, dsrc, ctx->S.pos_of_id, n, ctx->st);
    } else {
        launch_slab_to_int(ctx->d_istage, dsrc, ctx->S.pos_of_id, n, ctx->st);
        CK(cudaMemcpyAsync(host, ctx->d_istage, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, ctx->st));
    }
    CK(cudaStreamSynchronize(ctx->st));
    CK(cudaStreamSynchronize(ctx->st_cp));
    ctx->arena_used = 0;
    if (is_index) for (int i = 0; i < n; i++) host[i] = host[i] + 1;
    return 0;
}

static void tmark(ndsph_ctx* ctx, int k)
{
    if (ctx->profiling) cudaEventRecord(ctx->ev[k], ctx->st);
}
static float tdiff(ndsph_ctx* ctx, int a, int b)
{
    float ms = 0.f;
    if (ctx->profiling) cudaEventElapsedTime(&ms, ctx->ev[a], ctx->ev[b]);
    return ms;
}

// state fields the host hands over (x, vel, Bevol, en, hh, pmass, alpha)
static const int STATE_FIELDS[] = {X0, X1, X2, V0, V1, V2, BE0, BE1, BE2, EN, HH, PM, AL0, AL1, AL2,
                                   RHO, RHOALT, DRHODT, DHDT, GRADH, GRADHN, GRADGRADH};
static const int INCOPY_FIELDS[] = {XIN0, XIN1, XIN2, VIN0, VIN1, VIN2, BIN0, BIN1, BIN2, HIN, ENIN, RHOIN,
                                    ALIN0, ALIN1, ALIN2, FIN0, FIN1, FIN2, DBIN0, DBIN1, DBIN2, DHIN, DENIN,
                                    DALIN0, DALIN1, DALIN2};

// upload all inputs the drop-in entry points read (unsorted: slot = index)
static int upload_inputs(ndsph_ctx* ctx, const ndsph_particles* p, int n, bool with_density, bool with_prim)
{
    const int nd = ctx->o.ndim;
    ctx->packs_valid = false;
    int rc = ensure_capacity(ctx, n);
    if (rc) return rc;
    ctx->n = n;
    ctx->nl_valid = false;   // slot order reset below
    rc |= upload_aos(ctx, p->x, X0, nd, nd, n);
    rc |= upload_aos(ctx, p->vel, V0, 3, 3, n);
    rc |= upload_aos(ctx, p->Bevol, BE0, 3, 3, n);
    rc |= upload_aos(ctx, p->en, EN, 1, 1, n);
    rc |= upload_aos(ctx, p->hh, HH, 1, 1, n);
    rc |= upload_aos(ctx, p->pmass, PM, 1, 1, n);
    rc |= upload_aos(ctx, p->alpha, AL0, 3, 3, n);
    // the density outputs are module arrays in the reference: fixed particles
    // (and any particle the NR loop does not touch) carry them through
    (void)with_density;
    rc |= upload_aos(ctx, p->rho, RHO, 1, 1, n);
    rc |= upload_aos(ctx, p->rhoalt, RHOALT, 1, 1, n);
    rc |= upload_aos(ctx, p->drhodt, DRHODT, 1, 1, n);
    rc |= upload_aos(ctx, p->dhdt, DHDT, 1, 1, n);
    rc |= upload_aos(ctx, p->gradh, GRADH, 1, 1, n);
    rc |= upload_aos(ctx, p->gradhn, GRADHN, 1, 1, n);
    rc |= upload_aos(ctx, p->gradgradh, GRADGRADH, 1, 1, n);
    if (with_prim) {
        rc |= upload_aos(ctx, p->dens, DENS, 1, 1, n);
        rc |= upload_aos(ctx, p->uu, UU, 1, 1, n);
        rc |= upload_aos(ctx, p->pr, PR, 1, 1, n);
        rc |= upload_aos(ctx, p->spsound, CS, 1, 1, n);
        rc |= upload_aos(ctx, p->Bfield, BF0, 3, 3, n);
    }
    if (rc) return rc;
    if (const int* v = (const int*)host_view(ctx, p->itype))
        launch_int_shift(ctx->S.itype, v, n, 0, ctx->st);
    else
        CK(cudaMemcpyAsync(ctx->S.itype, p->itype, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, ctx->st));
    launch_iota(ctx->S.id, n, ctx->st);
    launch_iota(ctx->S.pos_of_id, n, ctx->st);
    // ireal: 1-based host index -> 0-based id (-1 none)
    if (!p->ireal) {
        CK(cudaMemsetAsync(ctx->S.ireal, 0xff, sizeof(int) * (size_t)n, ctx->st));
    } else if (const int* v = (const int*)host_view(ctx, p->ireal)) {
        launch_int_shift(ctx->S.ireal, v, n, -1, ctx->st);
    } else {
        CK(cudaMemcpyAsync(ctx->d_istage, p->ireal, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, ctx->st));
        launch_int_shift(ctx->S.ireal, ctx->d_istage, n, -1, ctx->st);
    }
    CK(cudaStreamSynchronize(ctx->st));
    ctx->linked = false;
    return 0;
}

// cell grid for the current hmax: periodic dims tile [xmin,xmax] with
// nc = floor(L/(2 hmax (1+1e-9))) >= 3 cells, open dims pad the bounding box
// by one cell each side (like linkND.f90:80-89)
static bool reuse_on(const ndsph_ctx* ctx)
{
    return ctx->nl_reuse && ctx->o.precision == NDSPH_PREC_FP32 && (!ctx->o.batched || ctx->o.stacked);
}

static int build_grid(ndsph_ctx* ctx, double hmax, const double* lo, const double* hi)
{
    Grid& g = ctx->g;
    // cells of 2 hmax skin when the rows may be kept across steps (their
    // radius is 2 h skin), 2 hmax otherwise.  The FP32 form of one simulation
    // searches a 5^ndim stencil of half-size cells (the candidates screened
    // per particle roughly halve); the FP64 form keeps the reference's 3^ndim
    // cells of 2 hmax.  A periodic box needs at least `sw` cells per dim (no
    // particle may meet two images of another): smaller boxes fall back to
    // the 3-wide stencil, then to the plain cell size.
    const double base = 2.0 * hmax * (1.0 + 1.e-9);
    const double skin_cf = reuse_on(ctx) ? (double)ctx->nl_skin : 1.0;
    // the wide stencil: 5^3 cells of hmax in 3D (FP32 form, one simulation);
    // in 1D (every form, batches included) a run of 17 cells of hmax/4, which
    // keeps cells small in the dense tubes of a batch whose cell size the
    // sparsest tube sets
    int wide = 3;
    if (ctx->nl_sw5 && ctx->o.ndim == 1) wide = 17;
    else if (ctx->nl_sw5 && ctx->o.ndim == 3 && ctx->o.precision == NDSPH_PREC_FP32 &&
             (!ctx->o.batched || ctx->o.stacked) && ctx->n < (1 << 25))
        wide = 5;
    const int tries_sw[3] = {wide, 3, 3};
    const double tries_cf[3] = {skin_cf, skin_cf, 1.0};
    int sw = 3;
    double cf = 1.0;
    for (int t = (wide > 3) ? 0 : 1; t < 3; t++) {
        const int reach = (tries_sw[t] - 1) / 2;
        bool fits = true;
        for (int d = 0; d < ctx->o.ndim; d++)
            if (ctx->o.periodic[d] && (long)floor(ctx->o.L[d] / (base * tries_cf[t] / reach)) < tries_sw[t])
                fits = false;
        if (fits || t == 2) { sw = tries_sw[t]; cf = tries_cf[t]; break; }
    }
    ctx->grid_cf = cf;
    g.sw = sw;
    g.nlshift = (ctx->o.ndim == 3 && sw == 5) ? 7 : 5;   // offsets < 32 otherwise
    const double cmin = base * cf / (double)((sw - 1) / 2);
    long ncells = 1;
    for (int d = 0; d < 3; d++) {
        if (d >= ctx->o.ndim) {
            g.nc[d] = 1; g.origin[d] = 0.0; g.cs[d] = 1.0;
        } else if (ctx->o.periodic[d]) {
            double L = ctx->o.L[d];
            long nc = (long)floor(L / cmin);
            if (nc < sw) {
                ctx->err = "periodic box smaller than 3 cells of 2*hmax";
                return NDSPH_E_CELLS;
            }
            if (nc > 4096) nc = 4096;
            g.nc[d] = (int)nc;
            g.origin[d] = ctx->o.xmin[d];
            g.cs[d] = L / (double)nc;
        } else {
            double ext = (hi[d] - lo[d]) + 2.0 * cmin;
            long nc = (long)floor(ext / cmin) + 1;
            if (nc > 1 << 22) { ctx->err = "too many cells"; return NDSPH_E_CELLS; }
            g.nc[d] = (int)std::max(nc, 1L);
            g.cs[d] = cmin;
            g.origin[d] = lo[d] - cmin;
        }
        g.inv_cs[d] = 1.0 / g.cs[d];
        g.csf[d] = (float)g.cs[d];
        ncells *= g.nc[d];
    }
    // a periodic batch: one grid per simulation, stacked
    g.ncs = (int)std::min(ncells, 200000001L);
    g.nstack = ctx->o.stacked ? ctx->o.nsim : 1;
    ncells *= g.nstack;
    if (ncells > 200000000L) { ctx->err = "too many cells"; return NDSPH_E_CELLS; }
    g.ncells = (int)ncells;
    ctx->cell_hmax = hmax;
    return ensure_cells(ctx, g.ncells);
}

// distance the search stencil covers around any point of a cell in every
// dimension: reach cells (every pair within it is found by a build)
static double stencil_cover(const ndsph_ctx* ctx)
{
    double c = 1e300;
    for (int d = 0; d < ctx->o.ndim; d++) c = std::min(c, ctx->g.cs[d]);
    return c * (double)((ctx->g.sw - 1) / 2);
}

static float unord_bitsf(unsigned u)
{
    u = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    float f;
    memcpy(&f, &u, sizeof f);
    return f;
}

// A step may keep the last link when the check of k_reuse_check passes:
// h + dmax <= skin h_build for every particle (the rows hold every pair
// within 2 max(h_i, h_j)) and hmax + dmax <= cell/2 (the Newton-Raphson
// relink cap).  Returns true and sets the step's dmax if so; the positions
// in xs are refreshed either way.
static bool try_keep_link(ndsph_ctx* ctx, bool keep_hmax_ghost, int* rc)
{
    *rc = 0;
    if (!reuse_on(ctx) || !ctx->nl_valid || !ctx->linked || ctx->grid_cf <= 1.0 || !ctx->S.nl) return false;
    // where particles outrun the skin every step (a supersonic flow), the
    // check fails each time: after two, three and four or more failures in a
    // row it is tried again after one, three and seven steps (a single pair of
    // failures, e.g. while a learned predictor is still untrained, then costs
    // one forced relink, not seven)
    if (ctx->keep_skip > 0) {
        ctx->keep_skip--;
        return false;
    }
    cudaStream_t st = ctx->st;
    Reduce* r = ctx->red;
    const unsigned init[2] = {0u, 0xffffffffu};
    if (cudaMemsetAsync(&r->hmax, 0, sizeof(unsigned long long), st) != cudaSuccess ||
        cudaMemcpyAsync(&r->reuse_d2, init, sizeof init, cudaMemcpyHostToDevice, st) != cudaSuccess) {
        *rc = NDSPH_E_CUDA;
        return false;
    }
    launch_reuse_check(ctx->F, ctx->S, ctx->g, ctx->o, ctx->n, ctx->nl_skin, ctx->nl_grow, r, st);
    if (read_red(ctx, r, st) != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
        *rc = NDSPH_E_CUDA;
        return false;
    }
    const double hmax = bitsd(ctx->h_red->hmax);
    float d2;
    memcpy(&d2, &ctx->h_red->reuse_d2, sizeof d2);
    const float slack = unord_bitsf(ctx->h_red->reuse_slack);
    float csmax = 0.f;
    for (int d = 0; d < ctx->o.ndim; d++) csmax = std::max(csmax, ctx->g.csf[d]);
    // rounding of the FP32 coordinates: a relative and an absolute margin
    const float dmax = sqrtf(d2) * 1.001f + 2e-6f * csmax;
    if (!(hmax > 0.0) || !std::isfinite(hmax) || !(dmax <= slack) ||
        !(hmax * ctx->nl_grow + dmax <= 0.5 * stencil_cover(ctx) / (1.0 + 1.e-9))) {
        ctx->keep_fails = std::min(ctx->keep_fails + 1, 4);
        if (ctx->keep_fails >= 2) ctx->keep_skip = (1 << (ctx->keep_fails - 1)) - 1;   // 1, 3, 7
        return false;
    }
    ctx->keep_fails = 0;
    if (!keep_hmax_ghost) {
        ctx->h_red->hmax_ghost = dbits(hmax);
        if (cudaMemcpyAsync(&r->hmax_ghost, &ctx->h_red->hmax_ghost, sizeof(unsigned long long),
                            cudaMemcpyHostToDevice, st) != cudaSuccess) {
            *rc = NDSPH_E_CUDA;
            return false;
        }
        if (ctx->o.stacked) launch_sim_ghost_h(ctx->F, ctx->S.sim, ctx->o, ctx->n, 1, st);
    }
    // the check covers every particle's current h: no row is stale
    if (cudaMemsetAsync(&r->nl_stale, 0, sizeof(int), st) != cudaSuccess) {
        *rc = NDSPH_E_CUDA;
        return false;
    }
    ctx->cell_hmax = hmax;
    ctx->nl_dmax = dmax;
    ctx->nl_reused++;
    return true;
}

// link: hmax + bbox, grid, counting sort by cell, permutation of `fields`;
// with may_keep, a step whose rows still hold every pair keeps the last link
static int do_link(ndsph_ctx* ctx, const int* fields, int nfields, bool keep_hmax_ghost, bool may_keep = false)
{
    const int n = ctx->n;
    cudaStream_t st = ctx->st;
    if (may_keep) {
        int rc = 0;
        if (try_keep_link(ctx, keep_hmax_ghost, &rc)) return 0;
        if (rc) return rc;
    }
    // late inputs still on their way are laid out again after this link
    // (what the gather moves of them now is overwritten then)
    if (ctx->late_pending) ctx->late_relayout = true;
    ctx->nl_valid = false;
    ctx->nl_dmax = 0.f;
    launch_link_reset(ctx->red, st);
    launch_hmax_bbox(ctx->F, ctx->o.ndim, n, ctx->red, &ctx->red->hmax, st);
    CK(read_red(ctx, ctx->red, st));
    CK(cudaStreamSynchronize(st));
    double hmax = bitsd(ctx->h_red->hmax);
    if (!(hmax > 0.0) || !std::isfinite(hmax)) {
        ctx->err = "link: max h <= 0 or not finite";
        return NDSPH_E_H_NONPOS;
    }
    double lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
        lo[d] = (d < ctx->o.ndim) ? unord_bits(ctx->h_red->xlo[d]) : 0.0;
        hi[d] = (d < ctx->o.ndim) ? unord_bits(ctx->h_red->xhi[d]) : 0.0;
        if (d < ctx->o.ndim && (!std::isfinite(lo[d]) || !std::isfinite(hi[d]))) {
            ctx->err = "link: non-finite position";
            return NDSPH_E_NAN;
        }
    }
    int rc = build_grid(ctx, hmax, lo, hi);
    if (rc) return rc;
    if (!keep_hmax_ghost) {
        ctx->h_red->hmax_ghost = dbits(hmax);
        CK(cudaMemcpyAsync(&ctx->red->hmax_ghost, &ctx->h_red->hmax_ghost, sizeof(unsigned long long),
                           cudaMemcpyHostToDevice, st));
        // a periodic batch: each simulation's ghosts take its own max h
        if (ctx->o.stacked) launch_sim_ghost_h(ctx->F, ctx->S.sim, ctx->o, n, 1, st);
    }
    CK(cudaMemcpyAsync(ctx->d_fields, fields, sizeof(int) * (size_t)nfields, cudaMemcpyHostToDevice, st));
    link_sort_gather(ctx, ctx->d_fields, nfields, st);
    ctx->linked = true;
    CK(cudaGetLastError());
    return build_nlist(ctx);
}

// counting sort by cell on the current grid, then the permutation gather of
// `d_fields` into the other slab and the swap of the slabs and side arrays
static void link_sort_gather(ndsph_ctx* ctx, const int* d_fields, int nfields, cudaStream_t st)
{
    ctx->packs_valid = false;
    ctx->tubes_valid = false;
    const int n = ctx->n;
    launch_cell_key(ctx->F, ctx->g, ctx->o, n, ctx->S.sim, ctx->srt, ctx->red, st);
    launch_scan(ctx->srt, ctx->g.ncells, st);
    launch_scatter_sort(ctx->srt, n, ctx->g.ncells, st);
    FieldPtrs dst;
    double* other = ctx->slab[1 - ctx->cur];
    for (int f = 0; f < NF; f++) {
        // keep the HH/HNEXT swap state consistent across slabs
        size_t off = (size_t)(ctx->F.f[f] - ctx->slab[ctx->cur]);
        dst.f[f] = other + off;
    }
    launch_gather_fields(dst, ctx->F, d_fields, nfields, ctx->srt.perm, n, st);
    launch_gather_int(ctx->itype2, ctx->S.itype, ctx->srt.perm, n, st);
    launch_gather_int(ctx->id2, ctx->S.id, ctx->srt.perm, n, st);
    launch_gather_int(ctx->ireal2, ctx->S.ireal, ctx->srt.perm, n, st);
    if (ctx->o.batched) {
        launch_gather_int(ctx->sim2, ctx->S.sim, ctx->srt.perm, n, st);
        std::swap(ctx->sim2, ctx->S.sim);
    }
    std::swap(ctx->itype2, ctx->S.itype);
    std::swap(ctx->id2, ctx->S.id);
    std::swap(ctx->ireal2, ctx->S.ireal);
    ctx->cur = 1 - ctx->cur;
    ctx->F = dst;
    launch_post_sort(ctx->S, ctx->srt, n, ctx->g.ncells, ctx->g, ctx->F, ctx->o, st);
}

static int link_all(ndsph_ctx* ctx, bool keep_hmax_ghost)
{
    std::vector<int> all(NF);
    for (int f = 0; f < NF; f++) all[f] = f;
    return do_link(ctx, all.data(), NF, keep_hmax_ghost);
}

// neighbour rows split by particle type: two types (gas + dust) in the 3D
// FP32 form, whose density passes then read only the rows of their own type
static bool typed_rows_wanted(const ndsph_ctx* ctx)
{
    return ctx->o.idust != 0 && ctx->o.precision == NDSPH_PREC_FP32 && ctx->o.ndim == 3;
}

static SweepArgs sweep_args(ndsph_ctx* ctx)
{
    SweepArgs a;
    a.F = ctx->F;
    a.S = ctx->S;
    a.cell_start = ctx->srt.start;
    a.cell_h = ctx->srt.cell_h;
    a.g = ctx->g;
    a.o = ctx->o;
    a.t = ctx->t;
    a.red = ctx->red;
    a.n = ctx->n;
    a.its = 0;
    a.nlist = 0;
    a.ncalc_next = ctx->d_ncalc;
    a.nl_ld = ctx->cap;
    a.nl_stride = ctx->nl_stride;
    a.nl_skin = ctx->nl_skin;
    a.nl_dmax = ctx->nl_dmax;
    a.typed_rows = (typed_rows_wanted(ctx) && ctx->S.nl2) ? 1 : 0;
    a.mixed = 0;
    a.d_its = nullptr;
    a.d_nlist = nullptr;
    a.gate = nullptr;
    a.graph = 0;
    a.plist = nullptr;
    a.pi0 = a.pn = 0;
    a.tail_on = 0;
    memset(&a.tail, 0, sizeof a.tail);
    return a;
}

// (re)build the neighbour lists of the current link; grows the stride and
// rebuilds once if some particle had more candidates than the stride
static int build_nlist(ndsph_ctx* ctx)
{
    cudaStream_t st = ctx->st;
    ctx->nl_valid = false;
    const bool typed = typed_rows_wanted(ctx);
    if (ctx->nl_stride == 0) {
        int s0 = ctx->o.ndim == 1 ? 32 : (ctx->o.ndim == 2 ? 64 : 160);
        CK(cudaMalloc(&ctx->S.nl, sizeof(unsigned) * (size_t)s0 * ctx->cap));
        ctx->nl_stride = s0;
    }
    if (typed && !ctx->S.nl2) CK(cudaMalloc(&ctx->S.nl2, sizeof(unsigned) * (size_t)ctx->nl_stride * ctx->cap));
    for (int attempt = 0; attempt < 4; attempt++) {
        int z[3] = {0, 0, 0};
        CK(cudaMemcpyAsync(&ctx->red->nl_stale, z, sizeof(int) * 3, cudaMemcpyHostToDevice, st));
        SweepArgs a = sweep_args(ctx);
        launch_build_nlist(a, st);
        ctx->timing.nl_builds++;
        CK(cudaGetLastError());
        int h[3];
        CK(cudaMemcpyAsync(h, &ctx->red->nl_stale, sizeof(int) * 3, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (!h[1]) {
            ctx->nl_valid = reuse_on(ctx) && ctx->grid_cf > 1.0 && ctx->nl_dmax == 0.f;
            return 0;
        }
        // overflow: grow to the largest count seen (+50%, so a slowly
        // growing maximum does not reallocate every few steps) and rebuild
        int ns = (h[2] + h[2] / 2 + 8 + 3) & ~3;   // rows of whole 16-byte groups
        CK(cudaFree(ctx->S.nl));
        ctx->S.nl = nullptr;
        CK(cudaMalloc(&ctx->S.nl, sizeof(unsigned) * (size_t)ns * ctx->cap));
        if (ctx->S.nl2) {
            CK(cudaFree(ctx->S.nl2));
            ctx->S.nl2 = nullptr;
            CK(cudaMalloc(&ctx->S.nl2, sizeof(unsigned) * (size_t)ns * ctx->cap));
        }
        ctx->nl_stride = ns;
    }
    ctx->err = "neighbour list stride did not converge";
    return NDSPH_E_CAPACITY;
}

// iterate_density iterate_density.f90:43-360 on the linked device state
static int do_iterate_density(ndsph_ctx* ctx, int* its_out, int* ncalctotal_out, int* nrelink_out)
{
    const int n = ctx->n;
    cudaStream_t st = ctx->st;
    const int itsmax = ctx->o.maxdensits;
    launch_density_init(ctx->F, ctx->S, n, ctx->red, st);
    int zero = 0;
    CK(cudaMemcpyAsync(&ctx->red->redolink, &zero, sizeof(int), cudaMemcpyHostToDevice, st));
    int its = 0, ncalc = n, ncalctotal = 0, nrelink = 0;
    bool redolink = false, h1_stale = true, rows_stale = false, any_full = false;
    if (ctx->o.batched) launch_sim_nr_init(ctx->o, st);
    if (ctx->o.precision == NDSPH_PREC_FP32) {
        SweepArgs pa = sweep_args(ctx);
        launch_pack_v(pa, st);
    }
    // count fixed particles: a full pass is taken while ncalc == npart
    float dens_ms = 0.f, pass1_ms = 0.f;
    while (ncalc > 0 && its <= itsmax) {
        its++;
        // rows outgrown on a step that kept the last link: the cells no longer
        // bound the displacements, so the rows are rebuilt by a full relink
        const bool rows_relink = rows_stale && ctx->nl_dmax > 0.f;
        bool relinked = false;
        if (redolink || rows_relink) {
            // relink (iterate_density.f90:122-126): the ghosts' hhmax becomes the
            // current max h.  The cells and the neighbour lists only have to be
            // rebuilt if h outgrew them; otherwise refreshing hhmax is enough.
            CK(cudaMemsetAsync(&ctx->red->hmax, 0, sizeof(unsigned long long), st));
            launch_hmax_bbox(ctx->F, ctx->o.ndim, n, ctx->red, &ctx->red->hmax, st);
            unsigned long long hb = 0ull;
            CK(cudaMemcpyAsync(&hb, &ctx->red->hmax, sizeof(hb), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            const double hmax_now = bitsd(hb);
            const double cap = 0.5 * stencil_cover(ctx) / (1.0 + 1.e-9) - (double)ctx->nl_dmax;
            if (hmax_now <= cap && !rows_relink) {
                CK(cudaMemcpyAsync(&ctx->red->hmax_ghost, &hb, sizeof(hb), cudaMemcpyHostToDevice, st));
                // a periodic batch: the simulations that asked take their own max h
                if (ctx->o.stacked) launch_sim_ghost_h(ctx->F, ctx->S.sim, ctx->o, n, 0, st);
            } else {
                // active list -> ids
                std::vector<int> act(ncalc), ids(n);
                CK(cudaMemcpy(act.data(), ctx->S.active, sizeof(int) * (size_t)ncalc, cudaMemcpyDeviceToHost));
                CK(cudaMemcpy(ids.data(), ctx->S.id, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost));
                for (int k = 0; k < ncalc; k++) act[k] = ids[act[k]];
                // a relink asked for by the rows alone keeps the ghosts' hhmax;
                // in a periodic batch only the simulations that asked refresh it
                int rc = link_all(ctx, !redolink || ctx->o.stacked);
                if (rc) return rc;
                if (redolink && ctx->o.stacked) launch_sim_ghost_h(ctx->F, ctx->S.sim, ctx->o, n, 0, st);
                relinked = true;
                std::vector<int> pos(n);
                CK(cudaMemcpy(pos.data(), ctx->S.pos_of_id, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost));
                for (int k = 0; k < ncalc; k++) act[k] = pos[act[k]];
                CK(cudaMemcpy(ctx->S.active, act.data(), sizeof(int) * (size_t)ncalc, cudaMemcpyHostToDevice));
                if (ctx->o.precision == NDSPH_PREC_FP32) {
                    SweepArgs pa = sweep_args(ctx);
                    launch_pack_v(pa, st);
                }
                h1_stale = true;
            }
            if (redolink) nrelink++;
        }
        if (rows_stale && !relinked) {
            if (h1_stale) launch_h1(ctx->F, ctx->S, n, st);   // list radius from the current h
            h1_stale = false;
            int rc = build_nlist(ctx);
            if (rc) return rc;
        }
        rows_stale = false;
        const bool full = (ncalc == n);
        // a batch: a pass over the active list in which the simulations whose
        // every particle is still unconverged take the full pass's rule, as
        // each run alone would (the rest take the partial pass's)
        const bool mixed = ctx->o.batched && !full && any_full;
        const bool jacobi = full || mixed;
        // 1/h: after the start, a full pass (every h changed) or a relink; a
        // partial pass keeps it current for the particles it updates
        if (h1_stale) launch_h1(ctx->F, ctx->S, n, st);
        h1_stale = jacobi;
        if (jacobi && its > 1) launch_copy(ctx->F.f[HNEXT], ctx->F.f[HH], n, st);
        CK(cudaMemsetAsync(ctx->d_ncalc, 0, sizeof(int), st));
        CK(cudaMemsetAsync(&ctx->red->redolink, 0, sizeof(int), st));
        if (ctx->o.batched) CK(cudaMemsetAsync(&ctx->red->sim_any_full, 0, sizeof(int), st));
        SweepArgs a = sweep_args(ctx);
        a.its = its;
        a.nlist = ncalc;
        a.mixed = mixed ? 1 : 0;
        tmark(ctx, 2);
        launch_density(a, jacobi, st);
        tmark(ctx, 3);
        CK(cudaGetLastError());
        if (ctx->o.batched) launch_sim_full_update(ctx->o, ctx->red, st);
        if (jacobi) std::swap(ctx->F.f[HH], ctx->F.f[HNEXT]);
        if (ctx->o.has_fixed) launch_fixed_density_copy(ctx->F, ctx->S, n, st);
        ncalctotal += ncalc;
        // the next pass's count comes back with the reductions, one wait
        if (ctx->hd_ncalc) launch_read_words(ctx->hd_ncalc, ctx->d_ncalc, sizeof(int), st);
        else CK(cudaMemcpyAsync(ctx->h_ncalc, ctx->d_ncalc, sizeof(int), cudaMemcpyDeviceToHost, st));
        int rc = sync_red(ctx);
        if (rc) return rc;
        const int h_ncalc = *ctx->h_ncalc;
        if (ctx->profiling) {
            float ms = tdiff(ctx, 2, 3);
            dens_ms += ms;
            if (its == 1) pass1_ms = ms;
        }
        redolink = ctx->h_red->redolink != 0;
        any_full = ctx->o.batched && ctx->h_red->sim_any_full != 0;
        ncalc = h_ncalc;
        std::swap(ctx->S.active, ctx->S.active_next);
        // rows outgrown by some h: rebuilt before the next pass (a particle
        // that flags them is unconverged, so there is one)
        rows_stale = ctx->h_red->nl_stale != 0;
    }
    ctx->timing.density_ms = dens_ms;
    ctx->timing.density_pass1_ms = pass1_ms;
    ctx->timing.density_passes = its;
    if (its_out) *its_out = its;
    if (ncalctotal_out) *ncalctotal_out = ncalctotal;
    if (nrelink_out) *nrelink_out = nrelink;
    if (its > itsmax && itsmax > 0) {
        char buf[128];
        snprintf(buf, sizeof buf, "ERROR: DENSITY NOT CONVERGED ON %d PARTICLES", ncalc);
        ctx->err = buf;
        return NDSPH_E_NOT_CONVERGED;
    }
    return 0;
}

static int do_cons2prim(ndsph_ctx* ctx)
{
    launch_eos(ctx->F, ctx->S, ctx->o, ctx->n, ctx->red, ctx->st);
    launch_fixed_copy(ctx->F, ctx->S, ctx->o, ctx->n, ctx->st);
    CK(cudaGetLastError());
    return 0;
}

// ndsph_step without fixed particles: the rates sweep in pieces, piece c
// over the slots of host particles c*len .. (c+1)*len (in slot order, so a
// piece keeps the cells' locality).  Each particle's rates and corrected
// state (the corrector's arithmetic, read-only) go into the host-order
// staging from the sweep itself, and each chunk goes back to the host on the
// copy stream while the later pieces run; the corrector follows the whole
// sweep as before.
static int rates_streamed(ndsph_ctx* ctx, SweepArgs a)
{
    cudaStream_t st = ctx->st;
    ndsph_particles* p = ctx->dl_tail;
    const int n = ctx->n, nd = ctx->o.ndim, K = ctx->dl_pieces;
    const int len = (n + K - 1) / K;
    StepTail t;
    struct Out { double* host; double** stage; int stride; };
    // (the positions went back before the density passes when dl_x_done)
    Out outs[] = {{ctx->dl_x_done ? nullptr : p->x, &t.x, nd}, {p->vel, &t.v, 3}, {p->Bevol, &t.be, 3},
                  {p->en, &t.en, 1}, {p->hh, &t.hh, 1}, {p->alpha, &t.al, 3}, {p->drhodt, &t.drhodt, 1},
                  {p->dhdt, &t.dhdt, 1},
                  {p->force, &t.force, 3}, {p->dBevoldt, &t.db, 3}, {p->dudt, &t.dudt, 1},
                  {p->dendt, &t.dendt, 1}, {p->daldt, &t.dal, 3}, {p->divB, &t.divb, 1},
                  {p->curlB, &t.curlb, 3}, {p->del2u, &t.del2u, 1}, {p->graddivv, &t.gdv, 3}};
    size_t need = 0;
    for (const Out& o : outs) if (o.host) need += (size_t)o.stride * n;
    int rc = arena_reserve(ctx, need);
    if (rc) return rc;
    for (Out& o : outs) {
        *o.stage = nullptr;
        if (!o.host) continue;
        *o.stage = ctx->d_arena + ctx->arena_used;
        ctx->arena_used += (size_t)o.stride * n;
    }
    launch_piece_list(ctx->S.id, n, K, len, ctx->d_pcnt, ctx->d_plist, st);
    a.plist = ctx->d_plist;
    a.tail_on = 1;
    a.tail = t;
    // pieces alternate between the main and the upload stream (idle since
    // the late inputs arrived), so the next piece's blocks fill the SMs
    // while a piece drains; the pieces touch disjoint slots
    cudaStream_t ps[2] = {st, ctx->st_up};
    CK(cudaEventRecord(ctx->ev_pfork, st));
    CK(cudaStreamWaitEvent(ctx->st_up, ctx->ev_pfork, 0));
    for (int c = 0; c < K; c++) {
        const int h0 = c * len, cnt = std::min(len, n - h0);
        if (cnt <= 0) break;
        a.pi0 = h0;
        a.pn = cnt;
        // the sweep writes each particle's outputs and corrected state into
        // the staging; the chunk's copies follow the piece
        launch_rates(a, ps[c & 1]);
        CK(cudaEventRecord(ctx->ev_dl, ps[c & 1]));
        CK(cudaStreamWaitEvent(ctx->st_cp, ctx->ev_dl, 0));
        for (const Out& o : outs)
            if (o.host)
                CK(cudaMemcpyAsync(o.host + (size_t)h0 * o.stride, *o.stage + (size_t)h0 * o.stride,
                                   sizeof(double) * (size_t)cnt * o.stride, cudaMemcpyDeviceToHost, ctx->st_cp));
    }
    CK(cudaEventRecord(ctx->ev_pjoin, ctx->st_up));
    CK(cudaStreamWaitEvent(st, ctx->ev_pjoin, 0));
    CK(cudaGetLastError());
    ctx->dl_tail_done = true;
    return 0;
}

static int do_rates(ndsph_ctx* ctx)
{
    cudaStream_t st = ctx->st;
    launch_h1(ctx->F, ctx->S, ctx->n, st);
    SweepArgs a = sweep_args(ctx);
    if (ctx->o.precision == NDSPH_PREC_FP32) launch_pack_rates(a, st);
    tmark(ctx, 4);
    if (ctx->dl_tail) {
        int rc = rates_streamed(ctx, a);
        if (rc) return rc;
    } else {
        launch_rates(a, st);
    }
    tmark(ctx, 5);
    ctx->packs_valid = (ctx->o.precision == NDSPH_PREC_FP32);
    launch_finalize_dt(ctx->red, ctx->o, ctx->d_dtout, st);
    if (ctx->o.batched) launch_sim_finalize(ctx->o, ctx->d_sim_dtnext, ctx->d_sim_out, st);
    CK(cudaGetLastError());
    CK(read_dtout(ctx, st));
    int rc = sync_red(ctx);
    if (rc) return rc;
    ctx->timing.rates_ms = tdiff(ctx, 4, 5);
    ndsph_dt& d = ctx->last_dt;
    d.dtcourant = ctx->h_dtout[0];
    d.dtforce = ctx->h_dtout[1];
    d.dtav = ctx->h_dtout[2];
    d.dtdrag = ctx->h_dtout[3];
    d.dtvisc = 1.7976931348623157e308;
    d.vsigmax = ctx->h_dtout[4];
    d.stressmax = ctx->h_dtout[5];
    d.hhmax = bitsd(ctx->h_red->hmax_ghost);
    return 0;
}

// derivs: boundary, link, iterate_density, cons2prim, get_rates
static void mlp_train_async(ndsph_ctx* ctx);

static int do_derivs(ndsph_ctx* ctx, const int* fields, int nfields)
{
    cudaStream_t st = ctx->st;
    tmark(ctx, 0);
    bool anyb = false;
    for (int d = 0; d < ctx->o.ndim; d++) if (ctx->o.ibound[d] != 0) anyb = true;
    if (anyb) launch_boundary_wrap(ctx->F, ctx->o, ctx->n, st);
    int rc = do_link(ctx, fields, nfields, false, true);
    if (rc) return rc;
    // a streamed host-buffer step: the positions are final here (wrapped; the
    // corrector's wrap leaves them), so they go back while the density
    // passes run
    if (ctx->dl_tail && ctx->dl_tail->x) {
        rc = download_aos_ordered(ctx, ctx->dl_tail->x, X0, ctx->o.ndim, ctx->o.ndim, ctx->n);
        if (rc) return rc;
        ctx->dl_x_done = true;
    }
    tmark(ctx, 1);
    launch_reduce_reset(ctx->red, st);
    if (ctx->o.batched) launch_sim_reset(ctx->o, st);
    int its = 0, nct = 0, nrl = 0;
    rc = do_iterate_density(ctx, &its, &nct, &nrl);
    if (rc) return rc;
    if (ctx->mlp_train_here) {
        ctx->mlp_train_here = false;
        mlp_train_async(ctx);
    }
    if (ctx->dl_early) {
        rc = download_density_group(ctx, ctx->dl_early);
        if (rc) return rc;
        ctx->dl_density_done = true;
    }
    tmark(ctx, 6);
    rc = wait_late(ctx);
    if (rc) return rc;
    rc = do_cons2prim(ctx);
    if (rc) return rc;
    if (ctx->dl_early) {
        rc = download_prim_group(ctx, ctx->dl_early);
        if (rc) return rc;
        ctx->dl_prim_done = true;
    }
    tmark(ctx, 7);
    rc = do_rates(ctx);
    if (rc) return rc;
    ctx->last_dt.its = its;
    ctx->last_dt.ncalctotal = nct;
    ctx->last_dt.nrelink = nrl;
    if (ctx->profiling) {
        ctx->timing.link_ms = tdiff(ctx, 0, 1);
        ctx->timing.eos_ms = tdiff(ctx, 6, 7);
    }
    return 0;
}

// outputs final once the Newton-Raphson iteration ends (rates and the
// corrector leave them alone when no particle is fixed) and once the EOS ran
static int download_density_group(ndsph_ctx* ctx, ndsph_particles* p)
{
    const int n = ctx->n;
    int rc = 0;
    rc |= download_aos(ctx, p->rho, RHO, 1, 1, n);
    rc |= download_aos(ctx, p->rhoalt, RHOALT, 1, 1, n);
    rc |= download_aos(ctx, p->gradh, GRADH, 1, 1, n);
    rc |= download_aos(ctx, p->gradhn, GRADHN, 1, 1, n);
    rc |= download_aos(ctx, p->gradgradh, GRADGRADH, 1, 1, n);
    if (ctx->dl_early && p->numneigh) {
        int* dst = (int*)(ctx->d_arena + ctx->arena_used);   // int staging in the arena
        const size_t need = ((size_t)n * sizeof(int) + sizeof(double) - 1) / sizeof(double);
        if (ctx->arena_used + need <= ctx->arena_cap) {
            ctx->arena_used += need;
            CK(cudaEventRecord(ctx->ev_dl, ctx->st));
            CK(cudaStreamWaitEvent(ctx->st_g, ctx->ev_dl, 0));
            launch_slab_to_int(dst, ctx->S.numneigh, ctx->S.pos_of_id, n, ctx->st_g);
            CK(cudaEventRecord(ctx->ev_g, ctx->st_g));
            CK(cudaStreamWaitEvent(ctx->st_cp, ctx->ev_g, 0));
            CK(cudaMemcpyAsync(p->numneigh, dst, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, ctx->st_cp));
        } else {
            rc |= download_int(ctx, p->numneigh, ctx->S.numneigh, n, false);
        }
    }
    return rc;
}
static int download_prim_group(ndsph_ctx* ctx, ndsph_particles* p)
{
    const int n = ctx->n;
    int rc = 0;
    rc |= download_aos(ctx, p->dens, DENS, 1, 1, n);
    rc |= download_aos(ctx, p->uu, UU, 1, 1, n);
    rc |= download_aos(ctx, p->pr, PR, 1, 1, n);
    rc |= download_aos(ctx, p->spsound, CS, 1, 1, n);
    rc |= download_aos(ctx, p->Bfield, BF0, 3, 3, n);
    return rc;
}

static int download_all(ndsph_ctx* ctx, ndsph_particles* p)
{
    const int n = ctx->n, nd = ctx->o.ndim;
    int rc = 0;
    // streamed with the rates pieces; the density and EOS groups went before
    if (ctx->dl_tail_done) return download_end(ctx);
    rc |= download_aos(ctx, p->x, X0, nd, nd, n);
    rc |= download_aos(ctx, p->vel, V0, 3, 3, n);
    rc |= download_aos(ctx, p->Bevol, BE0, 3, 3, n);
    rc |= download_aos(ctx, p->en, EN, 1, 1, n);
    rc |= download_aos(ctx, p->hh, HH, 1, 1, n);
    if (!ctx->dl_early) rc |= download_aos(ctx, p->pmass, PM, 1, 1, n);   // ndsph_step: unchanged, not copied
    rc |= download_aos(ctx, p->alpha, AL0, 3, 3, n);
    rc |= download_aos(ctx, p->drhodt, DRHODT, 1, 1, n);
    rc |= download_aos(ctx, p->dhdt, DHDT, 1, 1, n);
    if (!ctx->dl_density_done) rc |= download_density_group(ctx, p);
    if (!ctx->dl_prim_done) rc |= download_prim_group(ctx, p);
    rc |= download_aos(ctx, p->force, F0, 3, 3, n);
    rc |= download_aos(ctx, p->dBevoldt, DB0, 3, 3, n);
    rc |= download_aos(ctx, p->dudt, DUDT, 1, 1, n);
    rc |= download_aos(ctx, p->dendt, DENDT, 1, 1, n);
    rc |= download_aos(ctx, p->daldt, DAL0, 3, 3, n);
    rc |= download_aos(ctx, p->divB, DIVB, 1, 1, n);
    rc |= download_aos(ctx, p->curlB, CB0, 3, 3, n);
    rc |= download_aos(ctx, p->del2u, DEL2U, 1, 1, n);
    rc |= download_aos(ctx, p->graddivv, GDV0, 3, 3, n);
    if (rc) return rc;
    if (ctx->dl_early) return download_end(ctx);   // numneigh went with the density group
    rc = download_int(ctx, p->numneigh, ctx->S.numneigh, n, false);
    return rc;
}

static void fill_dt(ndsph_ctx* ctx, ndsph_dt* d)
{
    if (!d) return;
    ctx->last_dt.dt = ctx->dt;
    ctx->last_dt.time = ctx->time;
    ctx->last_dt.nsteps = ctx->nsteps;
    *d = ctx->last_dt;
}

#define GUARD_CTX() do { if (!ctx) { g_err = "null context"; return NDSPH_E_ARG; } } while (0)
#define GUARD_N() do { if (npart < 0 || !p) { ctx->err = "bad npart or particles"; return NDSPH_E_ARG; } } while (0)

// ---------------------------------------------------------------------------
// drop-in entry points
// ---------------------------------------------------------------------------
extern "C" int ndsph_set_linklist(ndsph_ctx* ctx, ndsph_particles* p, int32_t npart, ndsph_dt* dts)
{
    GUARD_CTX(); GUARD_N();
    int rc = upload_inputs(ctx, p, npart, false, false);
    if (rc) return rc;
    rc = link_all(ctx, false);
    if (rc) return rc;
    CK(cudaStreamSynchronize(ctx->st));
    ctx->last_dt.hhmax = ctx->cell_hmax;
    fill_dt(ctx, dts);
    return 0;
}

extern "C" int ndsph_iterate_density(ndsph_ctx* ctx, ndsph_particles* p, int32_t npart, ndsph_dt* dts)
{
    GUARD_CTX(); GUARD_N();
    int rc = upload_inputs(ctx, p, npart, false, false);
    if (rc) return rc;
    rc = link_all(ctx, false);
    if (rc) return rc;
    launch_reduce_reset(ctx->red, ctx->st);
    int its = 0, nct = 0, nrl = 0;
    rc = do_iterate_density(ctx, &its, &nct, &nrl);
    ctx->last_dt.its = its; ctx->last_dt.ncalctotal = nct; ctx->last_dt.nrelink = nrl;
    ctx->last_dt.hhmax = bitsd(ctx->h_red->hmax_ghost);
    if (rc) return rc;
    const int n = ctx->n;
    rc |= download_aos(ctx, p->hh, HH, 1, 1, n);
    rc |= download_aos(ctx, p->rho, RHO, 1, 1, n);
    rc |= download_aos(ctx, p->rhoalt, RHOALT, 1, 1, n);
    rc |= download_aos(ctx, p->drhodt, DRHODT, 1, 1, n);
    rc |= download_aos(ctx, p->dhdt, DHDT, 1, 1, n);
    rc |= download_aos(ctx, p->gradh, GRADH, 1, 1, n);
    rc |= download_aos(ctx, p->gradhn, GRADHN, 1, 1, n);
    rc |= download_aos(ctx, p->gradgradh, GRADGRADH, 1, 1, n);
    if (rc) return rc;
    rc = download_int(ctx, p->numneigh, ctx->S.numneigh, n, false);
    fill_dt(ctx, dts);
    return rc;
}

extern "C" int ndsph_conservative2primitive(ndsph_ctx* ctx, ndsph_particles* p, int32_t npart)
{
    GUARD_CTX(); GUARD_N();
    int rc = upload_inputs(ctx, p, npart, true, false);
    if (rc) return rc;
    launch_iota(ctx->S.pos_of_id, npart, ctx->st);
    rc = do_cons2prim(ctx);
    if (rc) return rc;
    rc = sync_red(ctx);
    if (rc) return rc;
    const int n = ctx->n;
    // unsorted state: id = iota, so download maps identity
    rc |= download_aos(ctx, p->dens, DENS, 1, 1, n);
    rc |= download_aos(ctx, p->uu, UU, 1, 1, n);
    rc |= download_aos(ctx, p->pr, PR, 1, 1, n);
    rc |= download_aos(ctx, p->spsound, CS, 1, 1, n);
    rc |= download_aos(ctx, p->Bfield, BF0, 3, 3, n);
    if (rc) return rc;
    return download_end(ctx);
}

extern "C" int ndsph_get_rates(ndsph_ctx* ctx, ndsph_particles* p, int32_t npart, ndsph_dt* dts)
{
    GUARD_CTX(); GUARD_N();
    int rc = upload_inputs(ctx, p, npart, true, true);
    if (rc) return rc;
    rc = link_all(ctx, false);
    if (rc) return rc;
    launch_reduce_reset(ctx->red, ctx->st);
    // stressmax from the given B and P (the EOS pass recomputes them from
    // Bevol, rho, en exactly as conservative2primitive does)
    rc = do_cons2prim(ctx);
    if (rc) return rc;
    rc = do_rates(ctx);
    if (rc) return rc;
    const int n = ctx->n;
    rc |= download_aos(ctx, p->force, F0, 3, 3, n);
    rc |= download_aos(ctx, p->dBevoldt, DB0, 3, 3, n);
    rc |= download_aos(ctx, p->dudt, DUDT, 1, 1, n);
    rc |= download_aos(ctx, p->dendt, DENDT, 1, 1, n);
    rc |= download_aos(ctx, p->daldt, DAL0, 3, 3, n);
    rc |= download_aos(ctx, p->divB, DIVB, 1, 1, n);
    rc |= download_aos(ctx, p->curlB, CB0, 3, 3, n);
    rc |= download_aos(ctx, p->del2u, DEL2U, 1, 1, n);
    rc |= download_aos(ctx, p->graddivv, GDV0, 3, 3, n);
    rc |= download_aos(ctx, p->drhodt, DRHODT, 1, 1, n);
    rc |= download_aos(ctx, p->dhdt, DHDT, 1, 1, n);
    rc |= download_aos(ctx, p->pr, PR, 1, 1, n);
    rc |= download_aos(ctx, p->spsound, CS, 1, 1, n);
    rc |= download_aos(ctx, p->Bfield, BF0, 3, 3, n);
    rc |= download_aos(ctx, p->dens, DENS, 1, 1, n);
    rc |= download_aos(ctx, p->uu, UU, 1, 1, n);
    if (rc) return rc;
    rc = download_end(ctx);
    fill_dt(ctx, dts);
    return rc;
}

extern "C" int ndsph_derivs(ndsph_ctx* ctx, ndsph_particles* p, int32_t npart, ndsph_dt* dts)
{
    GUARD_CTX(); GUARD_N();
    int rc = upload_inputs(ctx, p, npart, false, false);
    if (rc) return rc;
    rc = do_derivs(ctx, STATE_FIELDS, (int)(sizeof(STATE_FIELDS) / sizeof(int)));
    if (rc) return rc;
    rc = download_all(ctx, p);
    fill_dt(ctx, dts);
    return rc;
}

extern "C" int ndsph_primitive2conservative(ndsph_ctx* ctx, ndsph_particles* p, int32_t npart, ndsph_dt* dts)
{
    GUARD_CTX(); GUARD_N();
    int rc = upload_inputs(ctx, p, npart, false, false);
    if (rc) return rc;
    const int n = ctx->n;
    rc |= upload_aos(ctx, p->dens, DENS, 1, 1, n);
    rc |= upload_aos(ctx, p->uu, UU, 1, 1, n);
    rc |= upload_aos(ctx, p->Bfield, BF0, 3, 3, n);
    if (rc) return rc;
    launch_p2c_init(ctx->F, ctx->S, ctx->o, n, ctx->st);
    // polyk from the first gas particle when iener = 0 (conservative2primitive.f90:511-528)
    if (ctx->o.iener == 0) {
        for (int i = 0; i < n; i++) {
            if (p->itype[i] != NDSPH_ITYPE_GAS) continue;
            double g1 = ctx->o.gamma - 1.;
            ctx->o.polyk = (ctx->o.gamma <= 1.0001) ? 2. / 3. * p->uu[i] : g1 * p->uu[i] / pow(p->dens[i], g1);
            ctx->opts.polyk = ctx->o.polyk;
            break;
        }
    }
    rc = link_all(ctx, false);
    if (rc) return rc;
    launch_reduce_reset(ctx->red, ctx->st);
    int its = 0;
    rc = do_iterate_density(ctx, &its, nullptr, nullptr);
    if (rc) return rc;
    launch_p2c_post(ctx->F, ctx->S, ctx->o, n, ctx->st);
    rc = do_derivs(ctx, STATE_FIELDS, (int)(sizeof(STATE_FIELDS) / sizeof(int)));
    if (rc) return rc;
    ctx->time = 0.0;
    ctx->dt = 0.0;
    ctx->nsteps = 0;
    rc = download_all(ctx, p);
    fill_dt(ctx, dts);
    return rc;
}

static const int MLP_FIELDS[] = {HPRED, HROOT, FT0, FT1, FT2};

// fields the link at the start of a step's derivs carries into the new slot
// order: the state and the step's saves, without position components beyond
// ndim, and without the density outputs when a density pass follows and no
// particle is fixed (the first pass then rewrites them for every particle;
// fixed particles carry some of theirs through; dh/dt stays, a particle left
// unconverged keeps it).  A relink inside the Newton-Raphson loop carries
// every field.
static std::vector<int> step_live_fields(const ndsph_ctx* ctx, bool learned)
{
    const int nd = ctx->o.ndim;
    const bool dens = ctx->o.maxdensits >= 1 && !ctx->o.has_fixed;
    std::vector<int> live;
    for (int f : STATE_FIELDS) {
        if ((f == X1 && nd < 2) || (f == X2 && nd < 3)) continue;
        if (dens && (f == RHO || f == RHOALT || f == DRHODT || f == GRADH || f == GRADHN || f == GRADGRADH))
            continue;
        live.push_back(f);
    }
    for (int f : INCOPY_FIELDS) {
        if ((f == XIN1 && nd < 2) || (f == XIN2 && nd < 3)) continue;
        live.push_back(f);
    }
    if (learned)
        for (int f : MLP_FIELDS) live.push_back(f);
    return live;
}

// learned h, before the link: features of the previous step, h_pred -> h_init
static void mlp_infer(ndsph_ctx* ctx)
{
    MlpInferArgs a;
    memset(&a, 0, sizeof a);
    a.n = ctx->n;
    a.ndim = ctx->o.ndim;
    a.dt = ctx->dt;
    a.hfact = ctx->o.hfact;
    const double pi = 3.141592653589793;
    const double r = 2.0 * ctx->o.hfact;
    a.nn_ref = (a.ndim == 3) ? 4.0 / 3.0 * pi * r * r * r : ((a.ndim == 2) ? pi * r * r : 2.0 * r);
    a.zclip = 2.0;             // |log(h_init/h_pred)| <= 0.02: a poor prediction costs
                               // NR passes, never a neighbour-list rebuild
    a.apply = 1;
    a.fixed = ctx->o.has_fixed;
    a.hin = ctx->F.f[HIN];
    a.rho = ctx->F.f[RHO];
    a.drhodt = ctx->F.f[DRHODT];
    a.cs = ctx->F.f[CS];
    a.pmass = ctx->F.f[PM];
    a.hroot = ctx->F.f[HROOT];
    // the packs hold the previous rates sweep's values of each slot (no link
    // since; FP32 form only)
    a.pk_v = (ctx->o.precision == NDSPH_PREC_FP32 && ctx->packs_valid) ? ctx->S.pk_v : nullptr;
    a.pk_t = a.pk_v ? ctx->S.pk_t : nullptr;
    a.numneigh = ctx->S.numneigh;
    a.itype = ctx->S.itype;
    a.hh = ctx->F.f[HH];
    a.hpred = ctx->F.f[HPRED];
    for (int k = 0; k < MLP_NFW; k++) a.feat[k] = reinterpret_cast<float2*>(ctx->F.f[FT0 + k]);
    launch_mlp_infer(ctx->mlp_frag, a, ctx->st);
}

// learned h, after the density iteration: train on (features, converged h)
static void mlp_train(ndsph_ctx* ctx, cudaStream_t st)
{
    const long long n = ctx->n;
    // the gradient starts at zero: set so at init, and the Adam kernel
    // clears it after every use
    for (int it = 0; it < ctx->mlp_iters; it++) {
        MlpTrainArgs a;
        memset(&a, 0, sizeof a);
        a.nbatch = (int)std::min<long long>(ctx->mlp_batch, n);
        a.n = n;
        // strided sample: stride coprime with n, offset varies per update
        long long stride = n / std::max(a.nbatch, 1);
        if (stride < 1) stride = 1;
        while (stride > 1 && std::__gcd(stride, n) != 1) stride--;
        a.stride = stride;
        a.offset = (long long)(ctx->mlp_step * 7919LL + it * 104729LL) % n;
        for (int k = 0; k < MLP_NFW; k++) a.feat[k] = reinterpret_cast<const float2*>(ctx->F.f[FT0 + k]);
        a.hconv = ctx->F.f[HROOT];
        a.hpred = ctx->F.f[HPRED];
        if (it == ctx->mlp_iters - 1) CK_VOID(cudaMemsetAsync(ctx->mlp_loss, 0, sizeof(float), st));
        launch_mlp_grad(ctx->mlp_p, a, ctx->mlp_g, ctx->mlp_loss, st);
        ctx->mlp_step++;
        launch_mlp_adam(ctx->mlp_p, ctx->mlp_m, ctx->mlp_v, ctx->mlp_g, ctx->mlp_step, ctx->mlp_lr, st);
    }
    launch_mlp_pack(ctx->mlp_p, ctx->mlp_frag, st);
}

// The training reads the features, h_pred and the converged h, which nothing
// between the end of the density iteration and the corrector writes, and
// updates the weights, which the next step's inference reads: it runs on its
// own stream over that stretch (the EOS and the rates sweep), and the main
// stream waits for it before the corrector.  Without the stream it runs in
// order on the main stream.
static void mlp_train_async(ndsph_ctx* ctx)
{
    if (!ctx->st_mlp) {
        if (cudaStreamCreateWithFlags(&ctx->st_mlp, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&ctx->ev_mfork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ctx->ev_mjoin, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            if (ctx->st_mlp) { cudaStreamDestroy(ctx->st_mlp); ctx->st_mlp = nullptr; }
            if (ctx->ev_mfork) { cudaEventDestroy(ctx->ev_mfork); ctx->ev_mfork = nullptr; }
            if (ctx->ev_mjoin) { cudaEventDestroy(ctx->ev_mjoin); ctx->ev_mjoin = nullptr; }
            mlp_train(ctx, ctx->st);
            return;
        }
    }
    if (cudaEventRecord(ctx->ev_mfork, ctx->st) != cudaSuccess ||
        cudaStreamWaitEvent(ctx->st_mlp, ctx->ev_mfork, 0) != cudaSuccess) {
        cudaGetLastError();
        mlp_train(ctx, ctx->st);
        return;
    }
    mlp_train(ctx, ctx->st_mlp);
    cudaEventRecord(ctx->ev_mjoin, ctx->st_mlp);
    ctx->mlp_pending = true;
}
static void mlp_join(ndsph_ctx* ctx)
{
    if (!ctx->mlp_pending) return;
    cudaStreamWaitEvent(ctx->st, ctx->ev_mjoin, 0);
    ctx->mlp_pending = false;
}

// one leapfrog step on the device state (stepND_leapfrog_mhd.f90:31-275)
// fuse_next: another device-resident step follows in the same call, so the
// corrector also runs that step's save and predictor
static int dev_step_once(ndsph_ctx* ctx, bool fuse_next = false)
{
    cudaStream_t st = ctx->st;
    mlp_join(ctx);   // a training left by a step that stopped with an error
    // dt lives in the Reduce block
    CK(cudaMemcpyAsync(&ctx->red->dt, &ctx->dt, sizeof(double), cudaMemcpyHostToDevice, st));
    if (ctx->predicted)
        ctx->predicted = false;
    else if (ctx->late_pending)
        launch_predictor_part(ctx->F, ctx->S, ctx->o, ctx->n, ctx->red, 1, st);   // the rest in wait_late
    else
        launch_predictor(ctx->F, ctx->S, ctx->o, ctx->n, ctx->red, st);
    const bool learned = ctx->opts.learned_h && ctx->mlp_p;
    if (learned) {
        tmark(ctx, 12);
        mlp_infer(ctx);
        tmark(ctx, 13);
    }
    const std::vector<int> live = step_live_fields(ctx, learned);
    // the training overlaps the EOS and the rates sweep; a profiled step
    // runs it in order so that its time can be taken
    ctx->mlp_train_here = learned && !ctx->profiling;
    int rc = do_derivs(ctx, live.data(), (int)live.size());
    ctx->mlp_train_here = false;
    if (rc) return rc;
    mlp_join(ctx);
    if (learned) {
        if (ctx->profiling) {
            tmark(ctx, 14);
            mlp_train(ctx, st);
            tmark(ctx, 15);
            float loss = 0.f;
            cudaMemcpyAsync(&loss, ctx->mlp_loss, sizeof(float), cudaMemcpyDeviceToHost, st);
            cudaStreamSynchronize(st);
            ctx->timing.mlp_loss = loss;
            ctx->timing.mlp_ms = tdiff(ctx, 12, 13) + tdiff(ctx, 14, 15);
        }
        ctx->timing.mlp_updates = ctx->mlp_step;
    }
    if (fuse_next)
        launch_corrector_predictor(ctx->F, ctx->S, ctx->o, ctx->n, ctx->red, ctx->d_dtout + 6, st);
    else
        launch_corrector(ctx->F, ctx->S, ctx->o, ctx->n, ctx->red, st);
    rc = sync_red(ctx);
    if (rc) return rc;
    ctx->time += ctx->dt;
    ctx->dt = ctx->h_dtout[6];
    ctx->nsteps++;
    ctx->predicted = fuse_next;
    return 0;
}

extern "C" int ndsph_set_learning(ndsph_ctx* ctx, float lr, int32_t iters_per_step, int32_t batch)
{
    GUARD_CTX();
    if (!(lr > 0.f) || iters_per_step < 0 || batch < 1) { ctx->err = "bad learning schedule"; return NDSPH_E_ARG; }
    ctx->mlp_lr = lr;
    ctx->mlp_iters = iters_per_step;
    ctx->mlp_batch = batch;
    return 0;
}

// standalone MLP entry points for the tests (host buffers)
extern "C" int ndsph_mlp_forward(const float* params, const float* feats, int32_t n, float* out)
{
    if (!params || n < 0 || (n > 0 && (!feats || !out))) return NDSPH_E_ARG;
    if (n == 0) return 0;
    float *dp = nullptr, *df = nullptr, *dout = nullptr;
    MlpFrag* fr = nullptr;
    int rc = 0;
    if (cudaMalloc(&dp, sizeof(float) * MLP_NPARAM) != cudaSuccess || cudaMalloc(&fr, sizeof(MlpFrag)) != cudaSuccess ||
        cudaMalloc(&df, sizeof(float) * (size_t)n * MLP_NIN) != cudaSuccess ||
        cudaMalloc(&dout, sizeof(float) * (size_t)n) != cudaSuccess) {
        rc = NDSPH_E_CUDA;
    } else {
        cudaMemcpy(dp, params, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice);
        cudaMemcpy(df, feats, sizeof(float) * (size_t)n * MLP_NIN, cudaMemcpyHostToDevice);
        launch_mlp_pack(dp, fr, 0);
        launch_mlp_forward(fr, df, n, dout, 0);
        if (cudaMemcpy(out, dout, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess) rc = NDSPH_E_CUDA;
    }
    cudaFree(dp); cudaFree(fr); cudaFree(df); cudaFree(dout);
    return rc;
}

extern "C" int ndsph_mlp_grad(const float* params, const float* feats, const float* targets, int32_t n,
                              float* grad, float* loss)
{
    if (!params || n <= 0 || !feats || !targets || !grad || !loss) return NDSPH_E_ARG;
    float *dp = nullptr, *df = nullptr, *dt = nullptr, *dg = nullptr, *dl = nullptr;
    int rc = 0;
    if (cudaMalloc(&dp, sizeof(float) * MLP_NPARAM) != cudaSuccess ||
        cudaMalloc(&df, sizeof(float) * (size_t)n * MLP_NIN) != cudaSuccess ||
        cudaMalloc(&dt, sizeof(float) * (size_t)n) != cudaSuccess ||
        cudaMalloc(&dg, sizeof(float) * MLP_NPARAM) != cudaSuccess || cudaMalloc(&dl, sizeof(float)) != cudaSuccess) {
        rc = NDSPH_E_CUDA;
    } else {
        cudaMemcpy(dp, params, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice);
        cudaMemcpy(df, feats, sizeof(float) * (size_t)n * MLP_NIN, cudaMemcpyHostToDevice);
        cudaMemcpy(dt, targets, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice);
        MlpTrainArgs a;
        memset(&a, 0, sizeof a);
        a.nbatch = n;
        a.feats = df;
        a.targets = dt;
        cudaMemset(dg, 0, sizeof(float) * MLP_NPARAM);
        cudaMemset(dl, 0, sizeof(float));
        launch_mlp_grad(dp, a, dg, dl, 0);
        if (cudaMemcpy(grad, dg, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(loss, dl, sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = NDSPH_E_CUDA;
    }
    cudaFree(dp); cudaFree(df); cudaFree(dt); cudaFree(dg); cudaFree(dl);
    return rc;
}

static int dev_upload_impl(ndsph_ctx* ctx, const ndsph_particles* p, int32_t npart, bool link)
{
    int rc = upload_inputs(ctx, p, npart, true, true);
    if (rc) return rc;
    const int n = ctx->n;
    rc |= upload_aos(ctx, p->force, F0, 3, 3, n);
    rc |= upload_aos(ctx, p->dBevoldt, DB0, 3, 3, n);
    rc |= upload_aos(ctx, p->dendt, DENDT, 1, 1, n);
    rc |= upload_aos(ctx, p->dudt, DUDT, 1, 1, n);
    rc |= upload_aos(ctx, p->daldt, DAL0, 3, 3, n);
    rc |= upload_aos(ctx, p->divB, DIVB, 1, 1, n);
    rc |= upload_aos(ctx, p->curlB, CB0, 3, 3, n);
    if (rc) return rc;
    if (const int* v = (const int*)host_view(ctx, p->numneigh)) {
        launch_int_to_slab(ctx->S.numneigh, v, nullptr, n, ctx->st);
    } else {
        CK(cudaMemcpyAsync(ctx->d_istage, p->numneigh, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, ctx->st));
        launch_int_to_slab(ctx->S.numneigh, ctx->d_istage, nullptr, n, ctx->st);
    }
    if (link) rc = link_all(ctx, false);
    CK(cudaStreamSynchronize(ctx->st));
    return rc;
}

extern "C" int ndsph_dev_upload(ndsph_ctx* ctx, const ndsph_particles* p, int32_t npart)
{
    GUARD_CTX();
    if (npart < 0 || !p) { ctx->err = "bad npart or particles"; return NDSPH_E_ARG; }
    return dev_upload_impl(ctx, p, npart, true);
}

extern "C" int ndsph_dev_download(ndsph_ctx* ctx, ndsph_particles* p, ndsph_dt* dts)
{
    GUARD_CTX();
    if (!p) return NDSPH_E_ARG;
    int rc = download_all(ctx, p);
    fill_dt(ctx, dts);
    return rc;
}

extern "C" int ndsph_dev_step(ndsph_ctx* ctx, int32_t nsteps, ndsph_dt* dts)
{
    GUARD_CTX();
    const long long l0 = ndsph_launch_counter().load();
    // the whole call is bracketed by events on the context's stream
    CK(cudaEventRecord(ctx->ev[10], ctx->st));
    float rates_sum = 0.f, dens_sum = 0.f, link_sum = 0.f;
    int passes = 0;
    // between two steps of the call the corrector and the next predictor run
    // as one pass (one simulation without fixed particles: the predictor
    // then reads only each particle's own fields); the call ends corrected
    const bool fusable = !ctx->o.has_fixed && !ctx->o.batched;
    for (int k = 0; k < nsteps; k++) {
        tmark(ctx, 8);
        int rc = dev_step_once(ctx, fusable && k + 1 < nsteps);
        tmark(ctx, 9);
        if (rc) {
            ctx->predicted = false;
            return rc;
        }
        if (ctx->profiling) {
            cudaEventSynchronize(ctx->ev[9]);
            ctx->timing.step_ms = tdiff(ctx, 8, 9);
            rates_sum += ctx->timing.rates_ms;
            dens_sum += ctx->timing.density_ms;
            link_sum += ctx->timing.link_ms;
            passes += ctx->timing.density_passes;
        }
    }
    CK(cudaEventRecord(ctx->ev[11], ctx->st));
    CK(cudaEventSynchronize(ctx->ev[11]));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev[10], ctx->ev[11]);
    ctx->timing.total_ms = ms;
    if (ctx->profiling && nsteps > 0) {
        // per-call sums of the per-step kernel times
        ctx->timing.rates_ms = rates_sum;
        ctx->timing.density_ms = dens_sum;
        ctx->timing.link_ms = link_sum;
        ctx->timing.density_passes = passes;
    }
    ctx->timing.launches = (int32_t)(ndsph_launch_counter().load() - l0);
    fill_dt(ctx, dts);
    return 0;
}

extern "C" int ndsph_dev_set_time(ndsph_ctx* ctx, double dt, double time, int32_t nsteps)
{
    GUARD_CTX();
    ctx->dt = dt;
    ctx->time = time;
    ctx->nsteps = nsteps;
    return 0;
}

extern "C" int ndsph_dev_derivs(ndsph_ctx* ctx, ndsph_dt* dts)
{
    GUARD_CTX();
    int rc = do_derivs(ctx, STATE_FIELDS, (int)(sizeof(STATE_FIELDS) / sizeof(int)));
    fill_dt(ctx, dts);
    return rc;
}

// inputs of one leapfrog step: the state and the previous rates the
// predictor reads (force, dBevol/dt, de/dt, dalpha/dt, dh/dt); rho only for
// the learned-h predictor, whose features include it.  Every other
// array the step returns is recomputed for every particle -- except with
// fixed particles (whose gradgradh and rates the reference carries through)
// or maxdensits = 0 (no density pass), where everything is uploaded.
static int step_upload(ndsph_ctx* ctx, const ndsph_particles* p, int32_t npart)
{
    ctx->packs_valid = false;
    if (ctx->o.has_fixed || ctx->o.maxdensits < 1) return dev_upload_impl(ctx, p, npart, false);
    // when the last step's link may be kept, the caller's arrays go straight
    // into that step's slot order (slot k <- particle id[k]); the link's
    // check then decides from the uploaded positions and h whether the rows
    // still hold every pair, so arrays the caller changed are safe
    const bool keep = ctx->nl_valid && ctx->linked && npart == ctx->n && reuse_on(ctx);
    int rc = 0;
    // the learned-h predictor's inputs from the previous step that are not
    // among the uploaded arrays follow each particle into this upload's order
    bool carry_mlp = false;
    if (!keep) {
        const int n_prev = ctx->n;
        rc = ensure_capacity(ctx, npart);
        if (rc) return rc;
        carry_mlp = ctx->opts.learned_h && ctx->linked && n_prev == npart;
        ctx->n = npart;
        ctx->nl_valid = false;
    }
    const int n = npart, nd = ctx->o.ndim;
    const int* idm = keep ? ctx->S.id : nullptr;
    // late inputs (Bevol, energy, alpha and their rates: the EOS and their
    // part of the predictor) on the upload stream, overlapping the link and
    // the density passes (and the learned-h inference, which reads none of them)
    // early inputs (the predictor of x, v, h; the link; the density passes).
    // rho is recomputed for every particle by the first density pass and
    // read before it only as the save of fixed particles (none here) and as
    // a feature of the learned-h predictor
    rc |= upload_aos(ctx, p->x, X0, nd, nd, n, idm);
    rc |= upload_aos(ctx, p->vel, V0, 3, 3, n, idm);
    rc |= upload_aos(ctx, p->hh, HH, 1, 1, n, idm);
    rc |= upload_aos(ctx, p->pmass, PM, 1, 1, n, idm);
    if (ctx->opts.learned_h) rc |= upload_aos(ctx, p->rho, RHO, 1, 1, n, idm);
    rc |= upload_aos(ctx, p->dhdt, DHDT, 1, 1, n, idm);
    rc |= upload_aos(ctx, p->force, F0, 3, 3, n, idm);
    if (rc) return rc;
    // behind the early copies, so they do not share the link's bandwidth
    CK(cudaEventRecord(ctx->ev_up0, ctx->st_cp));
    CK(cudaStreamWaitEvent(ctx->st_up, ctx->ev_up0, 0));
    ctx->late_nf = 0;
    ctx->late_used = 0;
    ctx->late_relayout = false;
    rc |= upload_aos_late(ctx, p->Bevol, BE0, 3, 3, n, idm);
    rc |= upload_aos_late(ctx, p->en, EN, 1, 1, n, idm);
    rc |= upload_aos_late(ctx, p->alpha, AL0, 3, 3, n, idm);
    rc |= upload_aos_late(ctx, p->dBevoldt, DB0, 3, 3, n, idm);
    rc |= upload_aos_late(ctx, p->dendt, DENDT, 1, 1, n, idm);
    rc |= upload_aos_late(ctx, p->daldt, DAL0, 3, 3, n, idm);
    if (rc) return rc;
    CK(cudaEventRecord(ctx->ev_late, ctx->st_up));
    ctx->late_pending = true;
    if (keep) {
        const int* v = (const int*)host_view(ctx, p->itype);
        if (!v) {
            CK(cudaMemcpyAsync(ctx->d_istage, p->itype, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, ctx->st));
            v = ctx->d_istage;
        }
        launch_int_to_slab(ctx->S.itype, v, ctx->S.id, n, ctx->st);
    } else {
        if (const int* v = (const int*)host_view(ctx, p->itype))
            launch_int_shift(ctx->S.itype, v, n, 0, ctx->st);
        else
            CK(cudaMemcpyAsync(ctx->S.itype, p->itype, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, ctx->st));
        if (carry_mlp) {
            // slot k takes particle k: gather the previous step's values the
            // predictor reads (its h_pred and root estimate, drho/dt, c_s,
            // numneigh, and rho when the caller passes none) from the old
            // slot pos_of_id[k] into the other slab, then copy back
            static const int mf[5] = {HPRED, HROOT, DRHODT, CS, RHO};
            const int nmf = p->rho ? 4 : 5;
            CK(cudaMemcpyAsync(ctx->d_fields, mf, sizeof(int) * nmf, cudaMemcpyHostToDevice, ctx->st));
            FieldPtrs tmp;
            double* other = ctx->slab[1 - ctx->cur];
            for (int f = 0; f < NF; f++) tmp.f[f] = other + (size_t)(ctx->F.f[f] - ctx->slab[ctx->cur]);
            launch_gather_fields(tmp, ctx->F, ctx->d_fields, nmf, ctx->S.pos_of_id, n, ctx->st);
            for (int k = 0; k < nmf; k++) launch_copy(ctx->F.f[mf[k]], tmp.f[mf[k]], n, ctx->st);
            launch_gather_int(ctx->d_istage, ctx->S.numneigh, ctx->S.pos_of_id, n, ctx->st);
            CK(cudaMemcpyAsync(ctx->S.numneigh, ctx->d_istage, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice,
                               ctx->st));
        }
        launch_iota(ctx->S.id, n, ctx->st);
        launch_iota(ctx->S.pos_of_id, n, ctx->st);
        ctx->linked = false;
    }
    CK(cudaMemsetAsync(ctx->S.ireal, 0xff, sizeof(int) * (size_t)n, ctx->st));   // no fixed particles
    return 0;
}

extern "C" int ndsph_step(ndsph_ctx* ctx, ndsph_particles* p, int32_t npart, ndsph_dt* dts)
{
    GUARD_CTX(); GUARD_N();
    // the predictor is per particle, so the state need not be cell-sorted
    // before the step: derivs links after the predictor
    const long long l0 = ndsph_launch_counter().load();
    int rc = step_upload(ctx, p, npart);
    if (rc) return rc;
    if (dts) { ctx->dt = dts->dt; ctx->time = dts->time; ctx->nsteps = dts->nsteps; }
    // without fixed particles the density outputs and the primitives are
    // final before the rates sweep: copy them back while it runs
    const bool early = !ctx->o.has_fixed;
    ctx->dl_early = early ? p : nullptr;
    // the rest streams with the rates pieces when the copies are staged and
    // the arrays are large enough for the pieces to pay
    const bool streamed = early && !ctx->host_access && !ctx->o.batched && ctx->dl_pieces > 1 &&
                          npart >= (1 << 16);
    ctx->dl_tail = streamed ? p : nullptr;
    ctx->dl_density_done = ctx->dl_prim_done = ctx->dl_tail_done = ctx->dl_x_done = false;
    ctx->arena_used = 0;
    rc = dev_step_once(ctx);
    if (rc) {
        cudaStreamSynchronize(ctx->st_g);
        cudaStreamSynchronize(ctx->st_cp);
        cudaStreamSynchronize(ctx->st_up);
        ctx->late_pending = false;
        ctx->dl_early = nullptr;
        ctx->dl_tail = nullptr;
        ctx->dl_density_done = ctx->dl_prim_done = ctx->dl_tail_done = ctx->dl_x_done = false;
        return rc;
    }
    ctx->dl_early = p;   // also: pmass is not copied back (the step never writes it)
    rc = download_all(ctx, p);
    ctx->dl_early = nullptr;
    ctx->dl_tail = nullptr;
    ctx->dl_density_done = ctx->dl_prim_done = ctx->dl_tail_done = ctx->dl_x_done = false;
    ctx->timing.launches = (int32_t)(ndsph_launch_counter().load() - l0);
    fill_dt(ctx, dts);
    return rc;
}

// ---------------------------------------------------------------------------
// batched form: nsim independent simulations in one device state with
// per-simulation dt, clock, reductions and drag constant.  Open/fixed
// boundaries: the simulations lie side by side along x.  Periodic in every
// dimension: each simulation keeps its own box and a cell grid of its own,
// the grids stacked (cell = sim * cells per grid + local cell), so the
// periodic wrap of the search stays inside each simulation.
// ---------------------------------------------------------------------------
extern "C" int ndsph_batch_upload(ndsph_ctx* ctx, const ndsph_particles* p, int32_t npart, const int32_t* sim,
                                  int32_t nsim, int32_t initialise)
{
    GUARD_CTX();
    if (!p || !sim || npart <= 0 || nsim <= 0) { ctx->err = "bad batch arguments"; return NDSPH_E_ARG; }
    int nper = 0;
    for (int d = 0; d < ctx->o.ndim; d++) {
        if (ctx->o.ibound[d] == 2) { ctx->err = "batched form: reflective boundaries are not supported"; return NDSPH_E_ARG; }
        nper += ctx->o.periodic[d];
    }
    if (nper != 0 && nper != ctx->o.ndim) {
        ctx->err = "batched form needs open or fixed boundaries, or periodic ones in every dimension";
        return NDSPH_E_ARG;
    }
    const bool stacked = (nper == ctx->o.ndim);
    for (int i = 0; i < npart; i++)
        if (sim[i] < 0 || sim[i] >= nsim) { ctx->err = "simulation index out of range"; return NDSPH_E_ARG; }
    int rc = upload_inputs(ctx, p, npart, true, !initialise);
    if (rc) return rc;
    const int n = ctx->n;
    if (initialise) {
        rc |= upload_aos(ctx, p->dens, DENS, 1, 1, n);
        rc |= upload_aos(ctx, p->uu, UU, 1, 1, n);
        rc |= upload_aos(ctx, p->Bfield, BF0, 3, 3, n);
    } else {
        rc |= upload_aos(ctx, p->force, F0, 3, 3, n);
        rc |= upload_aos(ctx, p->dBevoldt, DB0, 3, 3, n);
        rc |= upload_aos(ctx, p->dendt, DENDT, 1, 1, n);
        rc |= upload_aos(ctx, p->daldt, DAL0, 3, 3, n);
    }
    if (rc) return rc;
    // per-simulation arrays
    if (nsim != ctx->nsim) {
        void* old[] = {ctx->d_sim_red, ctx->d_sim_dt, ctx->d_sim_dtnext, ctx->d_sim_out, ctx->d_sim_off,
                       ctx->d_sim_aux};
        for (void* q : old) if (q) cudaFree(q);
        if (ctx->h_sim_out) cudaFreeHost(ctx->h_sim_out);
        CK(cudaMalloc(&ctx->d_sim_red, sizeof(unsigned long long) * SIMRED * (size_t)nsim));
        CK(cudaMalloc(&ctx->d_sim_dt, sizeof(double) * (size_t)nsim));
        CK(cudaMalloc(&ctx->d_sim_dtnext, sizeof(double) * (size_t)nsim));
        CK(cudaMalloc(&ctx->d_sim_out, sizeof(double) * 4 * (size_t)nsim));
        CK(cudaMalloc(&ctx->d_sim_off, sizeof(double) * (size_t)nsim));
        CK(cudaMalloc(&ctx->d_sim_aux, sizeof(unsigned long long) * SIMAUX * (size_t)nsim));
        CK(cudaMallocHost(&ctx->h_sim_out, sizeof(double) * 4 * (size_t)nsim));
        ctx->nsim = nsim;
    }
    CK(cudaMemsetAsync(ctx->d_sim_dt, 0, sizeof(double) * (size_t)nsim, ctx->st));
    CK(cudaMemsetAsync(ctx->d_sim_out, 0, sizeof(double) * 4 * (size_t)nsim, ctx->st));
    std::vector<double> off(nsim, 0.0);
    const double span = 2.0 * (ctx->o.xmax[0] - ctx->o.xmin[0]) + 1.0;
    if (!stacked)
        for (int s2 = 0; s2 < nsim; s2++) off[s2] = span * s2;
    // drag constants: the caller's per-simulation values, else the options'
    const bool own_k = ctx->h_kdrag.size() == (size_t)nsim;
    std::vector<unsigned long long> aux((size_t)SIMAUX * nsim, 0ull);
    for (int s2 = 0; s2 < nsim; s2++)
        aux[(size_t)s2 * SIMAUX + SA_KDRAG] = dbits(own_k ? ctx->h_kdrag[s2] : ctx->o.Kdrag);
    CK(cudaMemcpyAsync(ctx->d_sim_aux, aux.data(), sizeof(unsigned long long) * aux.size(), cudaMemcpyHostToDevice,
                       ctx->st));
    CK(cudaMemcpyAsync(ctx->d_sim_off, off.data(), sizeof(double) * (size_t)nsim, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->S.sim, sim, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, ctx->st));
    ctx->o.batched = 1;
    ctx->o.nsim = nsim;
    ctx->o.sim_red = ctx->d_sim_red;
    ctx->o.sim_dt = ctx->d_sim_dt;
    ctx->o.sim_aux = ctx->d_sim_aux;
    ctx->o.stacked = stacked ? 1 : 0;
    ctx->nl_valid = false;
    ctx->linked = false;
    ctx->predicted = false;          // a new state: no step has predicted it
    ctx->tubes_predicted = false;
    launch_add_offset(ctx->F, ctx->S.sim, ctx->d_sim_off, n, +1, ctx->st);
    if (initialise) {
        launch_p2c_init(ctx->F, ctx->S, ctx->o, n, ctx->st);
        rc = link_all(ctx, false);
        if (rc) return rc;
        launch_reduce_reset(ctx->red, ctx->st);
        launch_sim_reset(ctx->o, ctx->st);
        rc = do_iterate_density(ctx, nullptr, nullptr, nullptr);
        if (rc) return rc;
        launch_p2c_post(ctx->F, ctx->S, ctx->o, n, ctx->st);
        rc = do_derivs(ctx, STATE_FIELDS, (int)(sizeof(STATE_FIELDS) / sizeof(int)));
        if (rc) return rc;
    } else {
        rc = link_all(ctx, false);
        if (rc) return rc;
    }
    CK(cudaMemsetAsync(ctx->d_sim_dt, 0, sizeof(double) * (size_t)nsim, ctx->st));
    CK(cudaMemsetAsync(ctx->d_sim_out, 0, sizeof(double) * 4 * (size_t)nsim, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return 0;
}

// one eager batched step: predictor, derivs, corrector, next dt per simulation
// fuse_next (no fixed particles): another eager step follows in the same
// call, so the corrector also runs that step's save and predictor with each
// simulation's next dt (k_corrector_predictor); every call ends corrected
static int batch_step_eager(ndsph_ctx* ctx, bool fuse_next)
{
    cudaStream_t st = ctx->st;
    if (ctx->predicted) ctx->predicted = false;
    else launch_predictor(ctx->F, ctx->S, ctx->o, ctx->n, ctx->red, st);
    const std::vector<int> live = step_live_fields(ctx, false);
    int rc = do_derivs(ctx, live.data(), (int)live.size());
    if (rc) return rc;
    fuse_next = fuse_next && !ctx->o.has_fixed;
    if (fuse_next) launch_corrector_predictor(ctx->F, ctx->S, ctx->o, ctx->n, ctx->red, ctx->d_sim_dtnext, st);
    else launch_corrector(ctx->F, ctx->S, ctx->o, ctx->n, ctx->red, st);
    ctx->predicted = fuse_next;
    // next dt of every simulation
    CK(cudaMemcpyAsync(ctx->d_sim_dt, ctx->d_sim_dtnext, sizeof(double) * (size_t)ctx->nsim,
                       cudaMemcpyDeviceToDevice, st));
    rc = sync_red(ctx);
    if (rc) ctx->predicted = false;
    return rc;
}

// ---------------------------------------------------------------------------
// captured batched step (CUDA graph).  One graph launch runs the whole step:
// predictor, boundary, link on the cells fixed at capture, the neighbour-row
// build, the Newton-Raphson passes (the first full pass, then a WHILE
// conditional node over the partial passes whose condition a kernel sets from
// the device-side counts), EOS, rates, corrector and the next dt.  The host
// reads the reduction block once per step.  Cases the eager host loop handles
// by reallocation or relinking set `gfail` on the device instead; the step is
// then redone from the predicted state on the eager path (h back to its value
// at the start of the iteration) and the graphs are captured again.
// ---------------------------------------------------------------------------
static ndsph_ctx::PtrState save_ptrs(const ndsph_ctx* c)
{
    ndsph_ctx::PtrState p;
    memset(&p, 0, sizeof(p));   // padding too: states are compared bytewise
    p.cur = c->cur; p.F = c->F; p.S = c->S;
    p.itype2 = c->itype2; p.id2 = c->id2; p.ireal2 = c->ireal2; p.sim2 = c->sim2;
    return p;
}
static void load_ptrs(ndsph_ctx* c, const ndsph_ctx::PtrState& p)
{
    c->cur = p.cur; c->F = p.F; c->S = p.S;
    c->itype2 = p.itype2; c->id2 = p.id2; c->ireal2 = p.ireal2; c->sim2 = p.sim2;
}
static bool same_ptrs(const ndsph_ctx::PtrState& a, const ndsph_ctx::PtrState& b)
{
    return memcmp(&a, &b, sizeof(a)) == 0;
}

static void graph_drop(ndsph_ctx* ctx)
{
    for (int k = 0; k < 2; k++) {
        if (ctx->gexec[k]) cudaGraphExecDestroy(ctx->gexec[k]);
        ctx->gexec[k] = nullptr;
    }
    ctx->gvalid = false;
}

static bool graph_usable(const ndsph_ctx* ctx)
{
    return ctx->graph_mode >= 1 && ctx->o.batched && !ctx->o.stacked && !ctx->opts.learned_h && !ctx->profiling &&
           ctx->o.maxdensits >= 1 && ctx->n > 0;
}

// h cap of the captured cells (the cheap relink's test)
static double cell_cap(const ndsph_ctx* ctx)
{
    double cap = 1e300;
    const double reach = (double)((ctx->g.sw - 1) / 2);
    for (int d = 0; d < ctx->o.ndim; d++) cap = std::min(cap, 0.5 * reach * ctx->g.cs[d] / (1.0 + 1.e-9));
    return cap;
}

// one Newton-Raphson pass on stream s (full: the first pass of the step)
static void capture_nr_pass(ndsph_ctx* ctx, bool full, cudaGraphConditionalHandle hc, int its_cap,
                            cudaStream_t s)
{
    const int n = ctx->n;
    launch_nr_pre(ctx->red, ctx->d_ncalc, s);
    if (!full) {
        // the relink check of iterate_density.f90:122-126 (the first pass never relinks)
        launch_hmax_bbox(ctx->F, ctx->o.ndim, n, ctx->red, &ctx->red->hmax, s, &ctx->red->g_gate);
        launch_nr_relink_apply(ctx->red, cell_cap(ctx), s);
    }
    SweepArgs a = sweep_args(ctx);
    a.d_its = &ctx->red->g_its;
    if (!full) a.d_nlist = &ctx->red->g_nlist;
    launch_density(a, full, s);
    if (full) std::swap(ctx->F.f[HH], ctx->F.f[HNEXT]);
    if (ctx->o.has_fixed) launch_fixed_density_copy(ctx->F, ctx->S, n, s);
    launch_nr_post(ctx->red, ctx->d_ncalc, n, its_cap, hc, s);
    launch_copy_active(ctx->S.active, ctx->S.active_next, &ctx->red->g_nlist, n, s);
    // after the full pass every h changed; partial passes keep 1/h current themselves
    if (full) launch_h1(ctx->F, ctx->S, n, s);
    SweepArgs b = sweep_args(ctx);
    b.gate = &ctx->red->g_rebuild;
    b.graph = 1;
    launch_build_nlist(b, s);
}

#define GCK(call)                                                                          \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess && err == cudaSuccess) { err = e_; what = #call; }           \
    } while (0)

// capture one step from the current pointer state; leaves the pointers in the
// state after the step
static int capture_one(ndsph_ctx* ctx, cudaGraphExec_t* out, long long* nmain, long long* nbody)
{
    const long long c0 = ndsph_launch_counter().load();
    long long b0 = 0, b1 = 0;
    cudaStream_t st = ctx->st;
    const int n = ctx->n;
    cudaError_t err = cudaSuccess;
    const char* what = "";
    cudaGraph_t graph = nullptr;
    bool anyb = false;
    for (int d = 0; d < ctx->o.ndim; d++) if (ctx->o.ibound[d] != 0) anyb = true;
    const int its_cap = std::min(ctx->o.maxdensits, 30);
    GCK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    if (err) { ctx->err = std::string("graph capture: ") + cudaGetErrorString(err); return NDSPH_E_CUDA; }
    launch_graph_begin(ctx->red, st);
    launch_predictor(ctx->F, ctx->S, ctx->o, n, ctx->red, st);
    if (anyb) launch_boundary_wrap(ctx->F, ctx->o, n, st);
    // link on the captured cells
    launch_link_reset(ctx->red, st);
    launch_hmax_bbox(ctx->F, ctx->o.ndim, n, ctx->red, &ctx->red->hmax, st);
    launch_grid_check(ctx->red, ctx->g, ctx->o, st);
    link_sort_gather(ctx, ctx->d_live, ctx->nlive, st);
    GCK(cudaMemsetAsync(&ctx->red->nl_stale, 0, sizeof(int) * 3, st));
    {
        SweepArgs a = sweep_args(ctx);
        a.graph = 1;
        launch_build_nlist(a, st);
    }
    launch_reduce_reset(ctx->red, st);
    launch_sim_reset(ctx->o, st);
    // iterate_density
    launch_density_init(ctx->F, ctx->S, n, ctx->red, st);
    GCK(cudaMemsetAsync(&ctx->red->redolink, 0, sizeof(int), st));
    launch_h1(ctx->F, ctx->S, n, st);
    if (ctx->o.precision == NDSPH_PREC_FP32) {
        SweepArgs pa = sweep_args(ctx);
        launch_pack_v(pa, st);
    }
    cudaStreamCaptureStatus cs;
    cudaGraph_t cgraph = nullptr;
    GCK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &cgraph, nullptr, nullptr, nullptr));
    cudaGraphConditionalHandle hc = 0;
    GCK(cudaGraphConditionalHandleCreate(&hc, cgraph, 0, cudaGraphCondAssignDefault));
    capture_nr_pass(ctx, true, hc, its_cap, st);
    // the partial passes: WHILE node
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    GCK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &cgraph, &deps, nullptr, &ndeps));
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = hc;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t wnode = nullptr;
    GCK(cudaGraphAddNode(&wnode, cgraph, deps, nullptr, ndeps, &cp));
    if (err == cudaSuccess) {
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        GCK(cudaStreamUpdateCaptureDependencies(st, &wnode, nullptr, 1, cudaStreamSetCaptureDependencies));
        GCK(cudaStreamBeginCaptureToGraph(ctx->st2, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        b0 = ndsph_launch_counter().load();
        capture_nr_pass(ctx, false, hc, its_cap, ctx->st2);
        b1 = ndsph_launch_counter().load();
        GCK(cudaStreamEndCapture(ctx->st2, &body));
    }
    // cons2prim, rates, corrector, next dt
    launch_eos(ctx->F, ctx->S, ctx->o, n, ctx->red, st);
    launch_fixed_copy(ctx->F, ctx->S, ctx->o, n, st);
    launch_h1(ctx->F, ctx->S, n, st);
    {
        SweepArgs a = sweep_args(ctx);
        if (ctx->o.precision == NDSPH_PREC_FP32) launch_pack_rates(a, st);
        launch_rates(a, st);
    }
    launch_finalize_dt(ctx->red, ctx->o, ctx->d_dtout, st);
    launch_sim_finalize(ctx->o, ctx->d_sim_dtnext, ctx->d_sim_out, st);
    launch_corrector(ctx->F, ctx->S, ctx->o, n, ctx->red, st);
    launch_sim_dt_advance(ctx->d_sim_dt, ctx->d_sim_dtnext, ctx->nsim, ctx->red, st);
    GCK(cudaMemcpyAsync(ctx->h_red, ctx->red, sizeof(Reduce), cudaMemcpyDeviceToHost, st));
    GCK(cudaGetLastError());
    cudaError_t e2 = cudaStreamEndCapture(st, &graph);
    if (err == cudaSuccess && e2 != cudaSuccess) { err = e2; what = "cudaStreamEndCapture"; }
    if (err == cudaSuccess) GCK(cudaGraphInstantiate(out, graph, 0));
    if (graph) cudaGraphDestroy(graph);
    // capturing launches nothing: the launches are counted when the graph runs
    const long long c1 = ndsph_launch_counter().load();
    ndsph_launch_counter().fetch_sub(c1 - c0);
    *nbody = b1 - b0;
    *nmain = (c1 - c0) - *nbody;
    if (err != cudaSuccess) {
        cudaGetLastError();
        ctx->err = std::string("graph capture: ") + what + ": " + cudaGetErrorString(err);
        return NDSPH_E_CUDA;
    }
    return 0;
}
#undef GCK

static int capture_graphs(ndsph_ctx* ctx)
{
    cudaStream_t st = ctx->st;
    graph_drop(ctx);
    if (!ctx->st2) CK(cudaStreamCreateWithFlags(&ctx->st2, cudaStreamNonBlocking));
    if (!ctx->d_live) CK(cudaMalloc(&ctx->d_live, sizeof(int) * NF));
    const std::vector<int> live = step_live_fields(ctx, false);
    ctx->nlive = (int)live.size();
    CK(cudaMemcpyAsync(ctx->d_live, live.data(), sizeof(int) * live.size(), cudaMemcpyHostToDevice, st));
    // cells of the captured link: 2 hmax gmargin wide, 3 spare layers on open sides
    launch_link_reset(ctx->red, st);
    launch_hmax_bbox(ctx->F, ctx->o.ndim, ctx->n, ctx->red, &ctx->red->hmax, st);
    CK(cudaMemcpyAsync(ctx->h_red, ctx->red, sizeof(Reduce), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const double hmax = bitsd(ctx->h_red->hmax);
    if (!(hmax > 0.0) || !std::isfinite(hmax)) { ctx->err = "link: max h <= 0 or not finite"; return NDSPH_E_H_NONPOS; }
    const double hc = hmax * ctx->gmargin;
    const double c = 2.0 * hc * (1.0 + 1.e-9);
    double lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
        lo[d] = (d < ctx->o.ndim) ? unord_bits(ctx->h_red->xlo[d]) - 2.0 * c : 0.0;
        hi[d] = (d < ctx->o.ndim) ? unord_bits(ctx->h_red->xhi[d]) + 2.0 * c : 0.0;
        if (d < ctx->o.ndim && (!std::isfinite(lo[d]) || !std::isfinite(hi[d]))) {
            ctx->err = "link: non-finite position";
            return NDSPH_E_NAN;
        }
    }
    int rc = build_grid(ctx, hc, lo, hi);
    if (rc) return rc;
    ctx->g_hmax = hmax;
    const ndsph_ctx::PtrState s0 = save_ptrs(ctx);
    ctx->gptr[0] = s0;
    rc = capture_one(ctx, &ctx->gexec[0], &ctx->gl_main[0], &ctx->gl_body[0]);
    if (rc) { load_ptrs(ctx, s0); graph_drop(ctx); return rc; }
    ctx->gptr[1] = save_ptrs(ctx);
    rc = capture_one(ctx, &ctx->gexec[1], &ctx->gl_main[1], &ctx->gl_body[1]);
    const bool back = same_ptrs(save_ptrs(ctx), s0);
    load_ptrs(ctx, s0);
    if (rc) { graph_drop(ctx); return rc; }
    if (!back) { graph_drop(ctx); ctx->err = "graph capture: pointer state did not return"; return NDSPH_E_CUDA; }
    ctx->gparity = 0;
    ctx->gvalid = true;
    return 0;
}

// redo a step whose captured form set gfail: from the predicted state, with h
// back to its value at the start of the iteration
static int graph_redo(ndsph_ctx* ctx)
{
    cudaStream_t st = ctx->st;
    launch_copy(ctx->F.f[HH], ctx->F.f[HDEN0], ctx->n, st);
    CK(cudaMemsetAsync(&ctx->red->gfail, 0, sizeof(int), st));
    const std::vector<int> live = step_live_fields(ctx, false);
    int rc = do_derivs(ctx, live.data(), (int)live.size());
    if (rc) return rc;
    launch_corrector(ctx->F, ctx->S, ctx->o, ctx->n, ctx->red, st);
    CK(cudaMemcpyAsync(ctx->d_sim_dt, ctx->d_sim_dtnext, sizeof(double) * (size_t)ctx->nsim,
                       cudaMemcpyDeviceToDevice, st));
    return sync_red(ctx);
}

static int batch_step_graph(ndsph_ctx* ctx)
{
    if (!ctx->gvalid) {
        int rc = capture_graphs(ctx);
        if (rc) return rc;
    }
    const int p = ctx->gparity;
    CK(cudaGraphLaunch(ctx->gexec[p], ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    load_ptrs(ctx, ctx->gptr[1 - p]);
    ctx->gparity = 1 - p;
    ctx->gsteps++;
    ndsph_launch_counter().fetch_add(ctx->gl_main[p] + (long long)std::max(ctx->h_red->g_its - 1, 0) * ctx->gl_body[p]);
    if (ctx->h_red->err && !ctx->h_red->gfail) {
        ctx->err = device_err_msg(ctx->h_red->err, ctx->h_red->err_index);
        return ctx->h_red->err;
    }
    if (ctx->h_red->gfail) {
        // the captured step left its cells, rows or pass budget: what it
        // computed (a status it raised included) is redone on the eager path
        // from the step's predicted state, which raises any real error again
        if (ctx->h_red->err) {
            CK(cudaMemsetAsync(&ctx->red->err, 0, 2 * sizeof(int), ctx->st));
            ctx->h_red->err = 0;
        }
        ctx->gredo++;
        graph_drop(ctx);
        int rc = graph_redo(ctx);
        if (rc) return rc;
        if (ctx->gredo > 8 && ctx->gredo * 4 > ctx->gsteps) ctx->graph_mode = 0;   // mostly redone: stay eager
        return 0;
    }
    // cells much larger than h needs: capture again on the next step
    if (bitsd(ctx->h_red->hmax_ghost) < 0.8 * ctx->g_hmax) graph_drop(ctx);
    return 0;
}

// The fused per-tube step needs every simulation's particles in one run of
// slots, simulations in order (as the link leaves a 1D batch: simulation s
// sits at x offset s (2 L + 1)), and each tube small enough for one block's
// shared memory.  Ranges and a largest-first launch order are set up after
// every link.
static int tubes_prepare(ndsph_ctx* ctx)
{
    if (ctx->tubes_valid) return 0;
    ctx->tube_maxm = 0;
    ctx->tubes_valid = true;
    const int n = ctx->n, ns = ctx->nsim;
    if (n <= 0 || ns <= 0) return 0;
    std::vector<int> sim(n);
    CK(cudaStreamSynchronize(ctx->st));
    CK(cudaMemcpy(sim.data(), ctx->S.sim, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost));
    std::vector<int> start(ns + 1, 0), cnt(ns, 0);
    for (int k = 0; k < n; k++) {
        if (sim[k] < 0 || sim[k] >= ns || (k > 0 && sim[k] < sim[k - 1])) return 0;   // not in order
        cnt[sim[k]]++;
    }
    int maxm = 0;
    for (int q = 0; q < ns; q++) {
        if (cnt[q] == 0) return 0;
        start[q + 1] = start[q] + cnt[q];
        maxm = std::max(maxm, cnt[q]);
    }
    if (maxm > TUBE_MAX) return 0;
    std::vector<int> order(ns);
    for (int q = 0; q < ns; q++) order[q] = q;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cnt[x] > cnt[y]; });
    if (!ctx->d_tube_start) {
        CK(cudaMalloc(&ctx->d_tube_start, sizeof(int) * (size_t)(ns + 1)));
        CK(cudaMalloc(&ctx->d_tube_order, sizeof(int) * (size_t)ns));
        ctx->tube_cap = ns;
    } else if (ns > ctx->tube_cap) {
        cudaFree(ctx->d_tube_start);
        cudaFree(ctx->d_tube_order);
        ctx->d_tube_start = ctx->d_tube_order = nullptr;
        CK(cudaMalloc(&ctx->d_tube_start, sizeof(int) * (size_t)(ns + 1)));
        CK(cudaMalloc(&ctx->d_tube_order, sizeof(int) * (size_t)ns));
        ctx->tube_cap = ns;
    }
    CK(cudaMemcpy(ctx->d_tube_start, start.data(), sizeof(int) * (size_t)(ns + 1), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_tube_order, order.data(), sizeof(int) * (size_t)ns, cudaMemcpyHostToDevice));
    ctx->tube_maxm = maxm;
    return 0;
}

static bool fused_usable(const ndsph_ctx* ctx)
{
    return ctx->graph_mode == 1 && ctx->o.batched && !ctx->o.stacked && ctx->o.ndim == 1 && !ctx->opts.learned_h &&
           !ctx->profiling && ctx->o.maxdensits >= 1 && ctx->n > 0 && ctx->linked;
}

// one leapfrog step of every tube in one launch (k_tube_step); false in
// *done when the batch does not qualify
// predict_next: another fused step follows in the same call, so this
// launch's corrector also runs that step's save and predictor; the state
// between two such launches is the predicted one, and every call ends
// corrected.  The host reads the status block every 16 steps and at the end.
static int batch_step_fused(ndsph_ctx* ctx, bool* done, bool predict_next, bool check)
{
    *done = false;
    int rc = tubes_prepare(ctx);
    if (rc) return rc;
    if (ctx->tube_maxm <= 0) {
        if (ctx->tubes_predicted) { ctx->err = "batched step: predicted state without the fused step"; return NDSPH_E_ARG; }
        return 0;
    }
    SweepArgs a = sweep_args(ctx);
    launch_tube_step(a, ctx->d_tube_start, ctx->d_tube_order, ctx->nsim, ctx->d_sim_dtnext, ctx->d_sim_out,
                     ctx->tube_maxm, ctx->tubes_predicted, predict_next, ctx->st);
    CK(cudaGetLastError());
    ctx->tubes_predicted = predict_next;
    *done = true;
    ctx->fsteps++;
    if (!check) return 0;
    rc = sync_red(ctx);
    if (rc) ctx->tubes_predicted = false;
    return rc;
}

extern "C" int ndsph_batch_step(ndsph_ctx* ctx, int32_t nsteps, double* dt_out, double* time_out)
{
    GUARD_CTX();
    if (!ctx->o.batched) { ctx->err = "call ndsph_batch_upload first"; return NDSPH_E_ARG; }
    cudaStream_t st = ctx->st;
    const long long l0 = ndsph_launch_counter().load();
    CK(cudaEventRecord(ctx->ev[10], st));
    for (int k = 0; k < nsteps; k++) {
        bool done = false;
        if (fused_usable(ctx)) {
            const bool last = (k + 1 == nsteps);
            const int rc = batch_step_fused(ctx, &done, !last, last || (k % 16) == 15);
            if (rc) return rc;
        }
        if (!done) {
            const int rc = graph_usable(ctx) ? batch_step_graph(ctx) : batch_step_eager(ctx, k + 1 < nsteps);
            if (rc) return rc;
        }
        ctx->nsteps++;
    }
    CK(cudaEventRecord(ctx->ev[11], st));
    CK(cudaMemcpyAsync(ctx->h_sim_out, ctx->d_sim_out, sizeof(double) * 4 * (size_t)ctx->nsim,
                       cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev[10], ctx->ev[11]);
    ctx->timing.total_ms = ms;
    ctx->timing.launches = (int32_t)(ndsph_launch_counter().load() - l0);
    ctx->timing.graph_steps = ctx->gsteps;
    ctx->timing.graph_redos = ctx->gredo;
    ctx->timing.fused_steps = ctx->fsteps;
    for (int s2 = 0; s2 < ctx->nsim; s2++) {
        if (dt_out) dt_out[s2] = ctx->h_sim_out[s2 * 4 + 2];
        if (time_out) time_out[s2] = ctx->h_sim_out[s2 * 4 + 3];
    }
    return 0;
}

extern "C" int ndsph_set_host_access(ndsph_ctx* ctx, int32_t mode)
{
    GUARD_CTX();
    if (mode != 0 && mode != 1) { ctx->err = "host access mode must be 0 or 1"; return NDSPH_E_ARG; }
    CK(cudaStreamSynchronize(ctx->st));
    ctx->host_access = mode;
    return 0;
}

extern "C" int ndsph_batch_set_kdrag(ndsph_ctx* ctx, int32_t nsim, const double* kdrag)
{
    GUARD_CTX();
    if (nsim <= 0 || !kdrag) { ctx->err = "bad drag constants"; return NDSPH_E_ARG; }
    for (int s2 = 0; s2 < nsim; s2++)
        if (!(kdrag[s2] >= 0.0) || !std::isfinite(kdrag[s2])) { ctx->err = "drag constant negative or not finite"; return NDSPH_E_ARG; }
    ctx->h_kdrag.assign(kdrag, kdrag + nsim);
    if (ctx->o.batched && ctx->nsim == nsim) {
        CK(cudaStreamSynchronize(ctx->st));
        std::vector<unsigned long long> aux((size_t)SIMAUX * nsim);
        CK(cudaMemcpy(aux.data(), ctx->d_sim_aux, sizeof(unsigned long long) * aux.size(), cudaMemcpyDeviceToHost));
        for (int s2 = 0; s2 < nsim; s2++) aux[(size_t)s2 * SIMAUX + SA_KDRAG] = dbits(kdrag[s2]);
        CK(cudaMemcpy(ctx->d_sim_aux, aux.data(), sizeof(unsigned long long) * aux.size(), cudaMemcpyHostToDevice));
    }
    return 0;
}

extern "C" int ndsph_batch_set_graph(ndsph_ctx* ctx, int32_t mode)
{
    GUARD_CTX();
    if (mode < 0 || mode > 2) { ctx->err = "batched step mode must be 0, 1 or 2"; return NDSPH_E_ARG; }
    graph_drop(ctx);
    ctx->graph_mode = mode;
    return 0;
}

extern "C" int ndsph_batch_download(ndsph_ctx* ctx, ndsph_particles* p)
{
    GUARD_CTX();
    if (!ctx->o.batched || !p) { ctx->err = "call ndsph_batch_upload first"; return NDSPH_E_ARG; }
    launch_add_offset(ctx->F, ctx->S.sim, ctx->d_sim_off, ctx->n, -1, ctx->st);
    int rc = download_all(ctx, p);
    launch_add_offset(ctx->F, ctx->S.sim, ctx->d_sim_off, ctx->n, +1, ctx->st);
    CK(cudaStreamSynchronize(ctx->st));
    return rc;
}

extern "C" int ndsph_neighbour_csr(ndsph_ctx* ctx, int32_t mode, int64_t* offsets, int32_t* neigh, int64_t cap)
{
    GUARD_CTX();
    if (!ctx->linked || !offsets) { ctx->err = "call ndsph_set_linklist first"; return NDSPH_E_ARG; }
    const int n = ctx->n;
    cudaStream_t st = ctx->st;
    launch_h1(ctx->F, ctx->S, n, st);
    SweepArgs a = sweep_args(ctx);
    long long* d_cnt = nullptr;
    CK(cudaMalloc(&d_cnt, sizeof(long long) * (size_t)(n + 1)));
    launch_neigh_count(a, mode, d_cnt, st);
    std::vector<long long> cnt(n);
    CK(cudaMemcpyAsync(cnt.data(), d_cnt, sizeof(long long) * (size_t)n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    int64_t tot = 0;
    for (int i = 0; i < n; i++) { offsets[i] = tot; tot += cnt[i]; }
    offsets[n] = tot;
    if (tot > cap || !neigh) { cudaFree(d_cnt); ctx->err = "neighbour buffer too small"; return NDSPH_E_CAPACITY; }
    CK(cudaMemcpyAsync(d_cnt, offsets, sizeof(long long) * (size_t)n, cudaMemcpyHostToDevice, st));
    int* d_out = nullptr;
    CK(cudaMalloc(&d_out, sizeof(int) * (size_t)std::max<int64_t>(tot, 1)));
    launch_neigh_fill(a, mode, d_cnt, d_out, st);
    CK(cudaMemcpyAsync(neigh, d_out, sizeof(int) * (size_t)tot, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    cudaFree(d_out);
    cudaFree(d_cnt);
    for (int64_t k = 0; k < tot; k++) neigh[k] += 1;
    return 0;
}

extern "C" int ndsph_set_tuning(ndsph_ctx* ctx, const ndsph_tuning* t)
{
    GUARD_CTX();
    if (!t || !(t->nl_skin >= 1.0f && t->nl_skin <= 2.0f) || !(t->nl_grow >= 1.0f && t->nl_grow <= 1.5f) ||
        !(t->graph_cell_margin >= 1.0f && t->graph_cell_margin <= 2.0f) || (t->nl_reuse != 0 && t->nl_reuse != 1) ||
        (t->stencil != 3 && t->stencil != 5) || t->step_pieces < 1 || t->step_pieces > 8) {
        ctx->err = "tuning out of range (nl_skin in [1,2], nl_grow in [1,1.5], graph_cell_margin in [1,2], "
                   "stencil 3 or 5, step_pieces in [1,8])";
        return NDSPH_E_ARG;
    }
    ctx->nl_skin = t->nl_skin;
    ctx->nl_reuse = t->nl_reuse;
    ctx->nl_grow = t->nl_grow;
    ctx->nl_sw5 = (t->stencil == 5) ? 1 : 0;
    ctx->dl_pieces = t->step_pieces;
    // captured batched steps hold the old settings: capture afresh
    graph_drop(ctx);
    ctx->gmargin = t->graph_cell_margin;
    // rows built with the old radius: the next step links afresh
    ctx->nl_valid = false;
    ctx->keep_fails = ctx->keep_skip = 0;
    return 0;
}

extern "C" int ndsph_get_tuning(ndsph_ctx* ctx, ndsph_tuning* t)
{
    GUARD_CTX();
    if (!t) return NDSPH_E_ARG;
    t->nl_skin = ctx->nl_skin;
    t->nl_reuse = ctx->nl_reuse;
    t->nl_grow = ctx->nl_grow;
    t->graph_cell_margin = (float)ctx->gmargin;
    t->stencil = ctx->nl_sw5 ? 5 : 3;
    t->step_pieces = ctx->dl_pieces;
    return 0;
}

extern "C" int ndsph_get_timing(ndsph_ctx* ctx, ndsph_timing* t)
{
    GUARD_CTX();
    ctx->timing.nl_reused = ctx->nl_reused;
    if (t) *t = ctx->timing;
    return 0;
}

extern "C" int ndsph_set_profiling(ndsph_ctx* ctx, int32_t on)
{
    GUARD_CTX();
    ctx->profiling = on != 0;
    return 0;
}
