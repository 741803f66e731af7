/*
 * ndsph.h -- C-ABI of the GB300-native NDSPMHD hot path (libndsph_gpu.so).
 *
 * The reference (danieljprice/ndspmhd, serial Fortran 90) runs its per-step
 * SPH hot path through argument-less subroutines that talk through Fortran
 * module globals.  This header is the drop-in boundary: a Fortran shim
 * (ndspmhd_gb300/fortran/gpu_sph.f90) keeps the subroutine names and forwards
 * c_loc() of the module arrays to the entry points below.
 *
 * Conventions (identical to the Fortran side):
 *   - real     == double, integer == int32_t
 *   - x(ndim,n) is AoS per particle: x[i*ndim + d]
 *   - vel, Bevol, Bfield, force, dBevoldt, daldt, curlB, graddivv, alpha are
 *     (3,n) arrays: v[i*3 + d]   (ndimV = ndimB = 3 in every dimension)
 *   - particle indices passed across the boundary (ireal) are 1-based
 *   - every entry point returns 0 on success or an NDSPH_E* code; the shim
 *     maps a non-zero code to the reference's `call quit`.
 *   - one host thread calls the library; each handle owns one CUDA stream.
 */
#ifndef NDSPH_H
#define NDSPH_H

#include <stdint.h>

#if defined(__GNUC__)
#define NDSPH_API __attribute__((visibility("default")))
#else
#define NDSPH_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (mirror the reference's quit/stop sites) ---------------- */
#define NDSPH_OK               0
#define NDSPH_E_ARG            1   /* bad argument / option out of scope         */
#define NDSPH_E_CUDA           2   /* CUDA runtime error                         */
#define NDSPH_E_H_NONPOS       3   /* h <= 0       iterate_density.f90:99-102    */
#define NDSPH_E_RHO_NONPOS     4   /* rho <= 0     iterate_density.f90:168-170   */
#define NDSPH_E_NOT_CONVERGED  5   /* NR budget    iterate_density.f90:349-351   */
#define NDSPH_E_VSIG_DET       6   /* MHD det < 0  ratesND_mhd.f90:1422-1429     */
#define NDSPH_E_NAN            7   /* non-finite result                          */
#define NDSPH_E_CELLS          8   /* cell grid invalid (box < 3 cells, h > box) */
#define NDSPH_E_CLUMP          9   /* dx = 0 pair  ratesND_mhd.f90:419-424       */
#define NDSPH_E_CAPACITY      10   /* size above a fixed maximum                 */
#define NDSPH_E_U_NEG         11   /* u_therm < 0  eos.f90:66-72 (iener /= 0)    */

/* ---- particle types (variablesND.f90:165-171) ------------------------------ */
#define NDSPH_ITYPE_GAS      0
#define NDSPH_ITYPE_BND      1
#define NDSPH_ITYPE_DUST     2
#define NDSPH_ITYPE_BNDDUST 12

/* ---- pair-sum precision forms ---------------------------------------------- */
#define NDSPH_PREC_FP64  0   /* plain FP64, table-exact kernel (parity form)      */
#define NDSPH_PREC_FP32  1   /* FP32 pair terms, FP64 separations/accumulation    */

/*
 * Runtime options: the subset of the reference's `options`, `artvi`, `eos`,
 * `bound`, `setup_params` and `timestep` modules that the hot path reads
 * (defaults.f90:29-120).  Options outside the supported subset (ikernel != 0,
 * ikernav != 3, icty != 0, igravity != 0, iresist != 0, idivbzero != 0, ...)
 * have no field here: the library implements the reference's defaults for them.
 */
typedef struct ndsph_opts {
    int32_t ndim;            /* 1, 2 or 3 (dimen?D.f90)                           */
    int32_t ibound[3];       /* 0 none, 1 fixed particles, 3 periodic             */
    double  xmin[3];         /* bound module                                      */
    double  xmax[3];
    double  hfact;           /* 1.2                                               */
    double  tolh;            /* 1e-3                                              */
    double  psep;            /* setup particle spacing (h bump when numneigh<=1)  */
    int32_t maxdensits;      /* 250                                               */
    int32_t imhd;            /* 0, 1 (evolve B/rho) or 11 (evolve B)              */
    int32_t imagforce;       /* 2 (tensor form, stressmax correction)             */
    int32_t iener;           /* 2 (thermal energy) or 0 (polytropic/isothermal)   */
    int32_t iav;             /* 2                                                 */
    int32_t iavlim[3];       /* (2,1,0)                                           */
    double  alphamin;        /* 0.1                                               */
    double  alphaumin;       /* 0.0                                               */
    double  alphaBmin;       /* 1.0                                               */
    double  beta;            /* 2.0                                               */
    double  avdecayconst;    /* 0.1                                               */
    double  gamma;           /* 5/3                                               */
    double  polyk;           /* 1.0 (iener=0)                                     */
    int32_t idust;           /* 0 or 2 (two-fluid)                                */
    int32_t idrag_nature;    /* 1 (constant K)                                    */
    double  Kdrag;
    double  C_cour;          /* 0.3                                               */
    double  C_force;         /* 0.25                                              */
    int32_t precision;       /* NDSPH_PREC_*                                      */
    int32_t learned_h;       /* 1: MLP h predictor in front of NR (device forms)  */
} ndsph_opts;

/* Fill `o` with the reference defaults (defaults.f90:29-120) for `ndim`. */
NDSPH_API void ndsph_default_opts(ndsph_opts* o, int32_t ndim);

/*
 * Host particle arrays, Fortran module layout.  `n` below is the number of
 * real particles (npart); arrays must hold at least n entries (times the
 * per-particle stride).  Inputs are read, outputs are written; a caller may
 * pass the same pointers on every call.
 */
typedef struct ndsph_particles {
    /* part module: state (inputs) */
    double*  x;          /* (ndim,n)                                            */
    double*  vel;        /* (3,n)                                               */
    double*  Bevol;      /* (3,n)  B/rho (imhd 1..9) or B (imhd 11..)            */
    double*  en;         /* (n)    thermal energy (iener=2)                      */
    double*  hh;         /* (n)    smoothing length: in, updated by NR (inout)   */
    double*  pmass;      /* (n)                                                 */
    double*  alpha;      /* (3,n)  AV / conductivity / resistivity parameters   */
    int32_t* itype;      /* (n)                                                 */
    int32_t* ireal;      /* (n)    1-based source of fixed particles, 0 = none  */
    /* density / hterms outputs */
    double*  rho;        /* (n)                                                 */
    double*  rhoalt;     /* (n)    number-density sum (densn)                   */
    double*  drhodt;     /* (n)                                                 */
    double*  dhdt;       /* (n)                                                 */
    double*  gradh;      /* (n)    1/omega                                      */
    double*  gradhn;     /* (n)                                                 */
    double*  gradgradh;  /* (n)    zeta term                                    */
    int32_t* numneigh;   /* (n)                                                 */
    /* conservative2primitive outputs */
    double*  dens;       /* (n)                                                 */
    double*  uu;         /* (n)                                                 */
    double*  pr;         /* (n)                                                 */
    double*  spsound;    /* (n)                                                 */
    double*  Bfield;     /* (3,n)                                               */
    /* rates module outputs */
    double*  force;      /* (3,n)                                               */
    double*  dBevoldt;   /* (3,n)                                               */
    double*  dudt;       /* (n)                                                 */
    double*  dendt;      /* (n)                                                 */
    double*  daldt;      /* (3,n)                                               */
    double*  divB;       /* (n)                                                 */
    double*  curlB;      /* (3,n)                                               */
    double*  del2u;      /* (n)    conductivity-switch source                   */
    double*  graddivv;   /* (3,n)  curl-v estimate (iavlim(1) /= 3)             */
} ndsph_particles;

/* Timestep scalars of the `timestep` module plus diagnostics. */
typedef struct ndsph_dt {
    double  dtcourant;   /* ratesND_mhd.f90:1481                                */
    double  dtforce;     /* ratesND_mhd.f90:938-943                             */
    double  dtav;
    double  dtdrag;      /* ratesND_mhd.f90:545 (min t_s)                       */
    double  dtvisc;
    double  vsigmax;
    double  stressmax;   /* ratesND_mhd.f90:232-245                             */
    double  hhmax;       /* bound module                                        */
    double  dt;          /* next leapfrog dt (stepND_leapfrog_mhd.f90:252)      */
    double  time;
    int32_t its;         /* NR passes of the last iterate_density (itsdensity)  */
    int32_t ncalctotal;  /* particles summed over all passes                    */
    int32_t nsteps;
    int32_t nrelink;     /* cell-grid rebuilds inside the NR loop               */
} ndsph_dt;

typedef struct ndsph_ctx ndsph_ctx;   /* opaque: device mirrors, stream, tables */

/* ---- life cycle -------------------------------------------------------------
 * ndsph_init mirrors setkernels(ikernel=0,...) + setkerndrag(41) + init_drag
 * (initialiseND_mhd.f90:188-223, kernelND.f90:102-117): it builds the 4001-point
 * cubic-spline and double-hump tables in FP64 on the host, uploads them, and
 * reserves device capacity for `nmax` particles (grown on demand).            */
NDSPH_API int ndsph_init(ndsph_ctx** ctx, const ndsph_opts* opts, int32_t nmax);
NDSPH_API int ndsph_finalize(ndsph_ctx* ctx);
NDSPH_API const char* ndsph_last_error(ndsph_ctx* ctx);

/* ---- drop-in entry points (host arrays, one H2D/D2H per call) ---------------
 * ndsph_set_linklist  replaces set_linklist        linkND.f90:45-161
 *                     (+ periodic wrap boundaryND.f90:30-90; ghosts are not
 *                     built: periodic images are taken inside the sweeps the
 *                     way ghostND_mhd.f90:224-225 places them)
 * ndsph_iterate_density replaces iterate_density   iterate_density.f90:43-360
 *                     with density   density_sums.f90:38-379 (first pass) and
 *                     density_partial density_sums.f90:396-658 (later passes)
 * ndsph_conservative2primitive replaces the in-scope part of
 *                     conservative2primitive.f90:42-470 and eos.f90:40-106
 * ndsph_get_rates     replaces get_rates           ratesND_mhd.f90:29-979
 *                     (rates_core :1175-1690, artificial_dissipation
 *                     :1700-1894, mhd_terms :2377-2720, drag_forces
 *                     :1074-1169, get_tstop dust.f90:77-101)
 * ndsph_derivs        replaces derivs              derivs.f90:27-287
 *                     (boundary, link, iterate_density, cons2prim, get_rates)
 *                     in one H2D + one D2H.
 * ndsph_step          replaces step               stepND_leapfrog_mhd.f90:31-275
 *                     (predictor, derivs, corrector, boundary, dt) with the
 *                     leapfrog on the device; state in host arrays.  Outputs
 *                     are copied back while the step runs, so after a
 *                     non-zero status the arrays hold a mix of old and new
 *                     values (the reference stops there too).                  */
NDSPH_API int ndsph_set_linklist(ndsph_ctx* ctx, ndsph_particles* p, int32_t npart, ndsph_dt* dts);
NDSPH_API int ndsph_iterate_density(ndsph_ctx* ctx, ndsph_particles* p, int32_t npart, ndsph_dt* dts);
NDSPH_API int ndsph_conservative2primitive(ndsph_ctx* ctx, ndsph_particles* p, int32_t npart);
NDSPH_API int ndsph_get_rates(ndsph_ctx* ctx, ndsph_particles* p, int32_t npart, ndsph_dt* dts);
NDSPH_API int ndsph_derivs(ndsph_ctx* ctx, ndsph_particles* p, int32_t npart, ndsph_dt* dts);
NDSPH_API int ndsph_step(ndsph_ctx* ctx, ndsph_particles* p, int32_t npart, ndsph_dt* dts);

/* primitive2conservative (conservative2primitive.f90:478-799): initial h from
 * hfact*(m/rho)^(1/ndim) with rho = dens on input, density iteration,
 * Bevol and en from Bfield and uu, then one derivs.  Inputs: x, vel, pmass,
 * itype, ireal, dens (as initial rho), uu, Bfield, alpha.                     */
NDSPH_API int ndsph_primitive2conservative(ndsph_ctx* ctx, ndsph_particles* p, int32_t npart, ndsph_dt* dts);

/* ---- device-resident form ----------------------------------------------------
 * State lives in HBM between steps (sorted by cell); upload/download convert
 * to and from the host layout.  ndsph_dev_step runs one full leapfrog step on
 * the device with no host synchronisation except the NR pass count.           */
NDSPH_API int ndsph_dev_upload(ndsph_ctx* ctx, const ndsph_particles* p, int32_t npart);
NDSPH_API int ndsph_dev_download(ndsph_ctx* ctx, ndsph_particles* p, ndsph_dt* dts);
NDSPH_API int ndsph_dev_step(ndsph_ctx* ctx, int32_t nsteps, ndsph_dt* dts);
NDSPH_API int ndsph_dev_derivs(ndsph_ctx* ctx, ndsph_dt* dts);
/* set the leapfrog clock of the device-resident state (evolve.f90:50-56 starts
 * with dt = 0; later steps use the dt returned by the previous step)          */
NDSPH_API int ndsph_dev_set_time(ndsph_ctx* ctx, double dt, double time, int32_t nsteps);

/* ---- batched form --------------------------------------------------------------
 * `nsim` independent simulations with the same options (open or fixed
 * boundaries, or periodic in every dimension: each simulation then keeps its
 * own periodic box, the same xmin/xmax for all), in one device state: the
 * batched counterpart of running the reference once per input file
 * (ndspmhd.f90:312-359, multi/multirun.f90).  Batched steps predict h as
 * the reference does (the learned-h option applies to one simulation).
 * sim[i] (0-based) names the simulation of particle i; ireal stays 1-based
 * over the whole array.  Each simulation keeps its own dt and clock (first
 * step dt = 0 as evolve.f90:50-56); reductions (dtcourant, dtforce,
 * stressmax, ...) are per simulation, so each one evolves as it would alone.
 * initialise = 1 runs primitive2conservative on the inputs (dens, uu,
 * Bfield), 0 takes a full state.  dt_out/time_out hold nsim doubles.       */
NDSPH_API int ndsph_batch_upload(ndsph_ctx* ctx, const ndsph_particles* p, int32_t npart, const int32_t* sim,
                                 int32_t nsim, int32_t initialise);
NDSPH_API int ndsph_batch_step(ndsph_ctx* ctx, int32_t nsteps, double* dt_out, double* time_out);
NDSPH_API int ndsph_batch_download(ndsph_ctx* ctx, ndsph_particles* p);
/* how the host-buffer entry points move the caller's arrays: 1 (default) the
 * layout kernels read and write them in place when the device can address
 * them (pinned memory, or pageable memory on systems where the device reads
 * it, as Grace over NVLink-C2C does), else through staging copies; 0 always
 * staging copies.  The results are the same either way.                      */
NDSPH_API int ndsph_set_host_access(ndsph_ctx* ctx, int32_t mode);
/* per-simulation drag constants K (dust.f90:91, idrag_nature = 1: the
 * stopping time rho_i rho_j / (K (rho_i + rho_j))) of a batch whose runs
 * differ in K, as their input files would: kdrag holds nsim values >= 0.
 * Call it before ndsph_batch_upload so that the initialising derivs use them
 * (they are kept for every later upload of nsim simulations); called on an
 * uploaded batch of nsim simulations it also changes the next steps.
 * Without it every simulation takes the options' Kdrag.                     */
NDSPH_API int ndsph_batch_set_kdrag(ndsph_ctx* ctx, int32_t nsim, const double* kdrag);
/* how ndsph_batch_step runs a step: 1 (default) one launch per step -- for a
 * 1D batch whose simulations hold at most 4096 particles each, a fused kernel
 * with one block per simulation that runs its whole leapfrog step (predictor,
 * order by x, every Newton-Raphson pass, EOS, rates, its dt, corrector) with
 * no global sort or neighbour rows; otherwise as 2; 2 one captured CUDA graph
 * per step -- link, neighbour rows, the Newton-Raphson passes under a
 * device-driven WHILE node, EOS, rates, leapfrog and the per-simulation dt,
 * with steps the graph cannot finish (cells or rows outgrown, a relink, the
 * pass limit) redone on the eager path; 0 the eager host loop (one host
 * synchronisation per Newton-Raphson pass).  Replaces the one-run-per-input
 * loop of multi/multirun.f90; no reference counterpart for the mode itself.  */
NDSPH_API int ndsph_batch_set_graph(ndsph_ctx* ctx, int32_t mode);

/* ---- parity / debug helpers (never on a timed path) -------------------------
 * ndsph_neighbour_csr: after ndsph_set_linklist, the 1-based neighbour set of
 * every real particle under the criterion `mode` (0: q_i<2 gather as
 * density_partial, 1: q_i<2 or q_j<2 as density/get_rates), as CSR.  The
 * replacement of check_neighbourlist.f90:27-182.  `offsets` has npart+1
 * entries; `neigh` capacity `cap`; returns NDSPH_E_CAPACITY if too small.     */
NDSPH_API int ndsph_neighbour_csr(ndsph_ctx* ctx, int32_t mode, int64_t* offsets, int32_t* neigh, int64_t cap);

/* kernel tables as built on the host (for the table parity test): 5*4001
 * doubles: wij, grwij, grgrwij, wijdrag, grwijdrag.                            */
NDSPH_API int ndsph_kernel_tables(int32_t ndim, double* out);

/* ---- allocation-free entry point -------------------------------------------
 * No counterpart in the reference: an added entry point for callers that may
 * not allocate device memory when they call (device memory owned by another
 * runtime's pool, e.g. an OpenACC/OpenMP-offload host that maps the module
 * arrays itself; real-time loops that must not take cudaMalloc's implicit
 * synchronisation; applications that reserve all device memory up front).
 * It runs the first density pass of iterate_density with every particle
 * treated as converged (the maxdensits = 0 case): rho, gradh (= 1/omega) and
 * drhodt (normalised by gradh) for particles that are not fixed (the outputs
 * of fixed particles are left as they are: the caller copies them from their
 * sources as set_fixedbound does), numneigh for every particle.
 * All pointers are DEVICE pointers in the host layout of ndsph_particles
 * (x(ndim,n), vel(3,n)); `stream` is a cudaStream_t (NULL = legacy stream);
 * the call returns after the stream has finished its work.  Options: ndim,
 * ibound (0, 1 or 3, as ndsph_init), xmin/xmax; the rest take no part.
 * Scratch: one file-scope __device__ array of about 6 MB plus the kernel
 * tables (576 KB), held by every GPU that loads the library until exit;
 * npart <= 262144 and cells <= 262144 (cells of 2 hmax over the bounding box
 * or periodic box), larger sizes return NDSPH_E_CAPACITY.  Errors (also h <= 0
 * -> NDSPH_E_H_NONPOS, rho <= 0 -> NDSPH_E_RHO_NONPOS, a non-finite position
 * -> NDSPH_E_NAN) leave their message in ndsph_last_error(NULL).  Calls share
 * the scratch, so calls that overlap on the GPU race; each call clears what
 * must start at zero.  The first call on a device takes the scratch's device
 * address (cudaGetSymbolAddress) and uploads the kernel tables of the three
 * dimensions: make it before any stream capture.  No cudaMalloc, cudaFree or
 * allocating library call.                                                   */
NDSPH_API int ndsph_density_noalloc(const ndsph_opts* opts, const double* d_x, const double* d_hh,
                                    const double* d_pmass, const double* d_vel, const int32_t* d_itype,
                                    int32_t npart, double* d_rho, double* d_drhodt, double* d_gradh,
                                    int32_t* d_numneigh, void* stream);

/* per-kernel device timings of the last call (ms), for the bench's roofline. */
typedef struct ndsph_timing {
    float link_ms, density_ms, density_pass1_ms, eos_ms, rates_ms, post_ms, step_ms, total_ms;
    int32_t density_passes;
    int32_t launches;        /* kernel launches issued by the last step call   */
    int64_t pairs_density;   /* accepted (i,j) pairs summed in pass 1          */
    int64_t pairs_rates;     /* accepted (i,j) pairs in the rates sweep        */
    float   mlp_loss;        /* learned h: last minibatch loss (z units^2)     */
    float   mlp_ms;          /* learned h: inference + training time per step  */
    int32_t mlp_updates;     /* learned h: optimiser steps taken so far        */
    int32_t nl_builds;       /* neighbour-list builds so far (link + rebuilds)  */
    int32_t graph_steps;     /* batched steps run as a captured CUDA graph      */
    int32_t graph_redos;     /* of those, steps redone on the eager path        */
    int32_t nl_reused;       /* steps that kept the previous link and rows      */
    int32_t fused_steps;     /* batched steps run by the fused per-tube kernel   */
} ndsph_timing;
NDSPH_API int ndsph_get_timing(ndsph_ctx* ctx, ndsph_timing* t);

/* ---- search tuning ----------------------------------------------------------
 * Knobs of the neighbour search; none changes which pairs are summed.  No
 * reference counterpart: the reference rebuilds its cell link list every step
 * (derivs.f90:82-92 calling set_linklist, linkND.f90:45-161) with cells of
 * 2 hmax and no neighbour rows.  ndspmhd_gb300/autotune.py times candidate
 * settings on a workload and picks one.
 *   nl_skin   rows hold every pair within 2 max(h_i, h_j) nl_skin     (1.1)
 *   nl_reuse  FP32 form, one simulation: a step keeps the slot order, cells
 *             (sized 2 hmax nl_skin) and rows of the previous link while
 *             h + dmax <= nl_skin h_build holds for every particle, dmax
 *             being the largest displacement since the rows were built  (1)
 *   nl_grow   room for Newton-Raphson growth of h in that check      (1.005)
 *   graph_cell_margin  batched captured steps: cells of 2 hmax margin, so
 *             h may grow by the margin before a step leaves the graph (1.05)
 *   stencil   5 (wide): the FP32 form of one 3D simulation searches 5^3
 *             stencils of cells of hmax (x skin), about half the candidates
 *             of 3^3 stencils of 2 hmax cells, its rows packing 25-bit
 *             particle indices (npart < 2^25, else 3^3); 1D contexts (every
 *             form, batches included) search runs of 17 cells of hmax/4 and
 *             skip each cell farther than 2 skin max(h_i, the cell's largest
 *             h).  3 (narrow): 3^ndim stencils of 2 hmax cells everywhere.
 *             2D, the 3D FP64 form and 3D batches always use 3^ndim.     (5)
 *   step_pieces  ndsph_step on staged host arrays of >= 65536 particles and
 *             no fixed particles: the rates sweep runs in this many pieces,
 *             piece c over the particles of the c-th chunk of the host
 *             arrays, and each chunk's rates and corrected state go back
 *             while the later pieces run; 1: all after the corrector.  The
 *             values returned are the same either way.                   (8)
 * ndsph_set_tuning rejects values outside nl_skin in [1, 2], nl_grow in
 * [1, 1.5], graph_cell_margin in [1, 2], stencil in {3, 5}, step_pieces in
 * [1, 8]; the next step links afresh.                                        */
typedef struct ndsph_tuning {
    float   nl_skin;
    int32_t nl_reuse;
    float   nl_grow;
    float   graph_cell_margin;
    int32_t stencil;
    int32_t step_pieces;
} ndsph_tuning;
NDSPH_API int ndsph_set_tuning(ndsph_ctx* ctx, const ndsph_tuning* t);
NDSPH_API int ndsph_get_tuning(ndsph_ctx* ctx, ndsph_tuning* t);

/* ---- learned-h predictor: standalone forward / gradient (tests) ------------
 * params: the 1313 FP32 master weights (W1[32][6], b1[32], W2[32][32], b2[32],
 * W3[32], b3); feats[n][6]; host buffers.  ndsph_mlp_forward runs the
 * tensor-core inference (BF16 operands, FP32 accumulation); ndsph_mlp_grad
 * the training kernel: grad of mean((out - target)^2) and that loss.  No
 * reference counterpart (the learned part is new).                           */
NDSPH_API int ndsph_mlp_forward(const float* params, const float* feats, int32_t n, float* out);
/* training schedule of the learned-h predictor of a context (opts.learned_h):
 * Adam learning rate, optimiser steps per leapfrog step, minibatch size.     */
NDSPH_API int ndsph_set_learning(ndsph_ctx* ctx, float lr, int32_t iters_per_step, int32_t batch);
NDSPH_API int ndsph_mlp_grad(const float* params, const float* feats, const float* targets, int32_t n,
                             float* grad, float* loss);
NDSPH_API int ndsph_set_profiling(ndsph_ctx* ctx, int32_t on);

#ifdef __cplusplus
}
#endif
#endif /* NDSPH_H */
