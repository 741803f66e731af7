// ndsph_mlp.h -- the learned smoothing-length predictor (see ndsph_mlp.cu).
#pragma once
#include <cuda_runtime.h>
#include <vector>

namespace ndsph {

constexpr int MLP_NIN = 6;
constexpr int MLP_OFF_W1 = 0;
constexpr int MLP_OFF_B1 = MLP_OFF_W1 + 32 * MLP_NIN;
constexpr int MLP_OFF_W2 = MLP_OFF_B1 + 32;
constexpr int MLP_OFF_B2 = MLP_OFF_W2 + 32 * 32;
constexpr int MLP_OFF_W3 = MLP_OFF_B2 + 32;
constexpr int MLP_OFF_B3 = MLP_OFF_W3 + 32;
constexpr int MLP_NPARAM = MLP_OFF_B3 + 1;   // 1313

// tensor-core operands in per-lane fragment order + FP32 biases / last layer
struct MlpFrag {
    uint2 w1[4][32];
    uint2 w2[2][4][32];
    float b1[32], b2[32], w3[32];
    float b3, pad[3];
};

// inputs of one inference pass over the slots (SoA pointers of the slab)
//   features (FP32, O(1)):
//   f0 = 100 log(h_pred / h_prev)       leapfrog predictor step (ihvar = 2)
//   f1 = 100 dt div v,  div v = -drho/dt / rho of the previous step
//   f2 = 10 (numneigh / n_ref - 1)      previous neighbour count
//   f3 = 10 dt c_s / h_prev             Courant number
//   f4 = 100 log(rho h^ndim / (m hfact^ndim)) / ndim   h-rho consistency
//   f5 = z of the previous step         100 log(h_root / h_pred) (builder's choice),
//        h_root the Newton-Raphson estimate of the root at convergence
// The features of slot i are stored as FP32 pairs (f0,f1), (f2,f3), (f4,f5)
// in three double-sized words (feat[k][i]) for the training after the
// density iteration; the link in between permutes them with the slab.
constexpr int MLP_NFW = 3;
struct MlpInferArgs {
    int n, ndim;
    double dt, hfact, nn_ref, zclip;
    int apply, fixed;
    const double *hin, *rho, *drhodt, *cs, *pmass;
    const double* hroot;   // the previous step's root estimate (0 before any)
    // FP32 form: the previous rates sweep's FP32 packs (v, m) and (rho, P,
    // c_s, u) of each slot, read instead of converting the FP64 fields (the
    // conversions ran this kernel on the FP64 pipe); nullptr in the FP64 form
    const float4 *pk_v, *pk_t;
    const int *numneigh, *itype;
    double* hh;        // in: h_pred; out: h_pred exp(z/100)
    double* hpred;     // in: the previous step's h_pred; out: this step's
    float2* feat[MLP_NFW];
};

struct MlpTrainArgs {
    int nbatch;
    long long n, stride, offset;
    const float2* feat[MLP_NFW];
    const double *hconv, *hpred;
    const float *feats, *targets;   // explicit arrays (tests) instead of slots
};

void mlp_init_params(std::vector<float>& p, unsigned seed);
void launch_mlp_pack(const float* p, MlpFrag* fr, cudaStream_t st);
void launch_mlp_forward(const MlpFrag* fr, const float* feats, int n, float* out, cudaStream_t st);
void launch_mlp_infer(const MlpFrag* fr, const MlpInferArgs& a, cudaStream_t st);
void launch_mlp_grad(const float* p, const MlpTrainArgs& a, float* grad, float* loss, cudaStream_t st);
void launch_mlp_adam(float* p, float* m, float* v, float* g, int step, float lr, cudaStream_t st);

}  // namespace ndsph
