// ndsph_mlp.cu -- the learned smoothing-length predictor.
//
// A 6 -> 32 -> 32 -> 1 MLP (tanh hidden layers) predicts, per particle, the
// correction z = 100 log(h_conv / h_pred) between the Newton-Raphson
// converged h and the leapfrog predictor's h_pred = hhin + dt dhdt
// (stepND_leapfrog_mhd.f90:152-153, ihvar = 2), as the previous step's
// correction y_prev plus the network's output: y_prev passes in FP32, so the
// BF16 activations only carry the (smaller) change of the correction from
// one step to the next.  The prediction only moves
// the starting point of iterate_density: NR keeps the same tolerance and
// decides convergence, so a wrong prediction costs extra passes, never accuracy.
//
//  * inference: BF16 weights and activations, FP32 accumulation, on the
//    tensor cores with mma.sync.m16n8k16 (one warp = 16 particles per tile);
//  * training: online, after every step, on minibatches of the particles'
//    own features and the Newton-Raphson estimate of the root of f(h) at
//    convergence (the Newton step from the converged h: the converged h
//    itself only lies within ~tolh of the root, which put a floor of ~tolh
//    under the prediction error); forward/backward in FP32 with the
//    BF16-rounded weights the inference uses; Adam on FP32 master weights.
//
// Parameter vector (FP32, NPARAM = 1313): W1[32][6], b1[32], W2[32][32],
// b2[32], W3[32], b3.
#include <cuda_bf16.h>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>
#include "ndsph_common.cuh"
#include "ndsph_mlp.h"

namespace ndsph {

__device__ __forceinline__ unsigned pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<unsigned*>(&v);
}
__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
// hardware tanh (special-function unit, max abs error ~5e-4): inference only,
// where every activation is rounded to BF16 (relative step 4e-3) anyway
__device__ __forceinline__ float tanh_fast(float x)
{
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3,
                                         unsigned b0, unsigned b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// B fragments of W1 (4 n-tiles) and W2 (2 k-steps x 4 n-tiles) in the
// per-lane register order of mma.m16n8k16 (B[k][n] = W[n][k]); biases and W3
// as FP32 (bias adds and the last layer run on the CUDA cores)
__global__ void k_mlp_pack(const float* __restrict__ p, MlpFrag* fr)
{
    const int lane = threadIdx.x;   // 32 threads
    const int g = lane >> 2, t = lane & 3;
    const float* W1 = p + MLP_OFF_W1;
    const float* W2 = p + MLP_OFF_W2;
    for (int j = 0; j < 4; j++) {
        const int n = 8 * j + g;
        float k0 = (2 * t < MLP_NIN) ? W1[n * MLP_NIN + 2 * t] : 0.f;
        float k1 = (2 * t + 1 < MLP_NIN) ? W1[n * MLP_NIN + 2 * t + 1] : 0.f;
        fr->w1[j][lane] = make_uint2(pack_bf16(k0, k1), 0u);   // k >= 8 rows are zero
    }
    for (int s = 0; s < 2; s++)
        for (int j = 0; j < 4; j++) {
            const int n = 8 * j + g;
            const int k = 16 * s + 2 * t;
            fr->w2[s][j][lane] = make_uint2(pack_bf16(W2[n * 32 + k], W2[n * 32 + k + 1]),
                                            pack_bf16(W2[n * 32 + k + 8], W2[n * 32 + k + 9]));
        }
    if (lane == 0) {
        for (int k = 0; k < 32; k++) {
            fr->b1[k] = p[MLP_OFF_B1 + k];
            fr->b2[k] = p[MLP_OFF_B2 + k];
            fr->w3[k] = bf16r(p[MLP_OFF_W3 + k]);
        }
        fr->b3 = p[MLP_OFF_B3];
    }
}

// one 16-row tile through the network on the tensor cores; x[r][k] for the
// lane's rows g and g+8 come in as packed BF16 pairs; returns z for rows g, g+8
__device__ __forceinline__ void mlp_tile(const MlpFrag& fr, unsigned xa0, unsigned xa1, float& zg, float& zg8)
{
    const int lane = threadIdx.x & 31;
    const int t = lane & 3;
    // layer 1: [16 x 16(6 used)] x [16 x 32]
    float c1[4][4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        c1[j][0] = c1[j][1] = c1[j][2] = c1[j][3] = 0.f;
        const uint2 b = fr.w1[j][lane];
        mma_bf16(c1[j], xa0, xa1, 0u, 0u, b.x, b.y);
    }
    unsigned a2[2][4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int col = 8 * j + 2 * t;
        const float h0 = tanh_fast(c1[j][0] + fr.b1[col]);
        const float h1 = tanh_fast(c1[j][1] + fr.b1[col + 1]);
        const float h2 = tanh_fast(c1[j][2] + fr.b1[col]);
        const float h3 = tanh_fast(c1[j][3] + fr.b1[col + 1]);
        const int s = j >> 1, hiHalf = j & 1;
        a2[s][hiHalf * 2 + 0] = pack_bf16(h0, h1);   // row g
        a2[s][hiHalf * 2 + 1] = pack_bf16(h2, h3);   // row g+8
    }
    // layer 2: [16 x 32] x [32 x 32]
    float c2[4][4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        c2[j][0] = c2[j][1] = c2[j][2] = c2[j][3] = 0.f;
#pragma unroll
        for (int s = 0; s < 2; s++) {
            const uint2 b = fr.w2[s][j][lane];
            mma_bf16(c2[j], a2[s][0], a2[s][1], a2[s][2], a2[s][3], b.x, b.y);
        }
    }
    // layer 3 on the CUDA cores: z = W3 . tanh(c2 + b2) + b3
    float pg = 0.f, pg8 = 0.f;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int col = 8 * j + 2 * t;
        pg += fr.w3[col] * bf16r(tanh_fast(c2[j][0] + fr.b2[col])) + fr.w3[col + 1] * bf16r(tanh_fast(c2[j][1] + fr.b2[col + 1]));
        pg8 += fr.w3[col] * bf16r(tanh_fast(c2[j][2] + fr.b2[col])) + fr.w3[col + 1] * bf16r(tanh_fast(c2[j][3] + fr.b2[col + 1]));
    }
    pg += __shfl_xor_sync(0xffffffffu, pg, 1);
    pg += __shfl_xor_sync(0xffffffffu, pg, 2);
    pg8 += __shfl_xor_sync(0xffffffffu, pg8, 1);
    pg8 += __shfl_xor_sync(0xffffffffu, pg8, 2);
    zg = pg + fr.b3;
    zg8 = pg8 + fr.b3;
}

// forward of an explicit feature array (tests): feats[n][6] -> out[n]
__global__ void k_mlp_forward(const MlpFrag* __restrict__ frp, const float* __restrict__ feats, int n,
                              float* __restrict__ out)
{
    __shared__ MlpFrag fr;
    for (int k = threadIdx.x; k < (int)(sizeof(MlpFrag) / 4); k += blockDim.x)
        reinterpret_cast<unsigned*>(&fr)[k] = reinterpret_cast<const unsigned*>(frp)[k];
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int tile = warp; tile * 16 < n; tile += nwarps) {
        const int r0 = tile * 16 + g, r1 = r0 + 8;
        float f00 = 0.f, f01 = 0.f, f10 = 0.f, f11 = 0.f;
        if (2 * t < MLP_NIN) {
            if (r0 < n) { f00 = feats[r0 * MLP_NIN + 2 * t]; f01 = feats[r0 * MLP_NIN + 2 * t + 1]; }
            if (r1 < n) { f10 = feats[r1 * MLP_NIN + 2 * t]; f11 = feats[r1 * MLP_NIN + 2 * t + 1]; }
        }
        float z0, z1;
        mlp_tile(fr, pack_bf16(f00, f01), pack_bf16(f10, f11), z0, z1);
        if (t == 0) {
            if (r0 < n) out[r0] = z0;
            if (r1 < n) out[r1] = z1;
        }
    }
}

// features of one slot (all FP32, scaled to O(1)) -- see ndsph_mlp.h;
// false when one is not finite (a slot without a density yet: rho = 0 before
// the first density pass of a context whose caller passed none)
__device__ __forceinline__ bool slot_features(const MlpInferArgs& a, int i, float f[MLP_NIN])
{
    // FP32 throughout: the features are rounded to BF16 anyway, and FP64
    // transcendentals are expensive on this part
    // FP32 arithmetic from FP32 inputs where the FP32 form has them (FP64
    // conversions and divisions run on this part's narrow FP64 pipe)
    const float hprev = (float)a.hin[i], hpred = (float)a.hh[i];
    float rho, cs, m;
    if (a.pk_t) {
        const float4 t = a.pk_t[i];
        rho = t.x;
        cs = t.z;
        m = a.pk_v[i].w;
    } else {
        rho = (float)a.rho[i];
        cs = (float)a.cs[i];
        m = (float)a.pmass[i];
    }
    const float divv = -(float)a.drhodt[i] / rho;
    float hf = 1.f;
    const float hb = hprev / (float)a.hfact;
    for (int d = 0; d < a.ndim; d++) hf *= hb;
    f[0] = 100.f * __logf(hpred / hprev);
    f[1] = 100.f * (float)a.dt * divv;
    f[2] = 10.f * ((float)a.numneigh[i] / (float)a.nn_ref - 1.f);
    f[3] = 10.f * (float)a.dt * cs / hprev;
    f[4] = 100.f * __logf(rho * hf / m) / (float)a.ndim;
    // the previous step's correction, from its h_pred and root estimate
    // (none before the first learned step: both are 0 then)
    const float hp0 = (float)a.hpred[i], hr0 = (float)a.hroot[i];
    f[5] = (hp0 > 0.f && hr0 > 0.f) ? 100.f * __logf(hr0 / hp0) : 0.f;
    bool ok = true;
#pragma unroll
    for (int k = 0; k < MLP_NIN; k++) ok = ok && isfinite(f[k]);
    return ok;
}

// per step, before the link: h <- h_pred exp(z/100), features and h_pred kept
// for the training after the density iteration.  A warp takes 32 slots at a
// time: each lane loads and computes its own slot's features (coalesced), the
// two 16-row tiles go through the network on the tensor cores, and each lane
// stores its own slot's results.
__global__ void k_mlp_infer(const MlpFrag* __restrict__ frp, MlpInferArgs a)
{
    __shared__ MlpFrag fr;
    for (int k = threadIdx.x; k < (int)(sizeof(MlpFrag) / 4); k += blockDim.x)
        reinterpret_cast<unsigned*>(&fr)[k] = reinterpret_cast<const unsigned*>(frp)[k];
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int base = warp * 32; base < a.n; base += nwarps * 32) {
        const int i = base + lane;
        float fa[MLP_NIN] = {0, 0, 0, 0, 0, 0};
        bool ok = true;
        if (i < a.n) ok = slot_features(a, i, fa);
        if (!ok)
            for (int k = 0; k < MLP_NIN; k++) fa[k] = 0.f;   // the slot keeps h_pred (below)
        // A fragments of the two tiles: lane (g, t) holds columns 2t, 2t+1 of
        // rows g and g+8 (tile 0: slots base..base+15, tile 1: the next 16);
        // column pair (2k, 2k+1) comes by shuffle from the rows' lanes
        float x[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll
        for (int k = 0; k < 3; k++) {
#pragma unroll
            for (int tl = 0; tl < 2; tl++) {
                const float r00 = __shfl_sync(0xffffffffu, fa[2 * k], 16 * tl + g);
                const float r01 = __shfl_sync(0xffffffffu, fa[2 * k + 1], 16 * tl + g);
                const float r10 = __shfl_sync(0xffffffffu, fa[2 * k], 16 * tl + g + 8);
                const float r11 = __shfl_sync(0xffffffffu, fa[2 * k + 1], 16 * tl + g + 8);
                if (t == k) { x[tl][0] = r00; x[tl][1] = r01; x[tl][2] = r10; x[tl][3] = r11; }
            }
        }
        float z00, z08, z10, z18;
        mlp_tile(fr, pack_bf16(x[0][0], x[0][1]), pack_bf16(x[0][2], x[0][3]), z00, z08);
        mlp_tile(fr, pack_bf16(x[1][0], x[1][1]), pack_bf16(x[1][2], x[1][3]), z10, z18);
        // every lane of quad q holds z of rows q and q+8 of both tiles: lane
        // L takes its own slot's value from lane 4 (L mod 8)
        const int src = 4 * (lane & 7);
        const float a00 = __shfl_sync(0xffffffffu, z00, src);
        const float a08 = __shfl_sync(0xffffffffu, z08, src);
        const float a10 = __shfl_sync(0xffffffffu, z10, src);
        const float a18 = __shfl_sync(0xffffffffu, z18, src);
        const float zz = (lane < 8) ? a00 : (lane < 16) ? a08 : (lane < 24) ? a10 : a18;
        if (i < a.n) {
            for (int k = 0; k < MLP_NFW; k++) a.feat[k][i] = make_float2(fa[2 * k], fa[2 * k + 1]);
            // a slot without valid features is left out of the training
            if (!ok) a.feat[0][i] = make_float2(__int_as_float(0x7fc00000), 0.f);
            const double hpred = a.hh[i];
            a.hpred[i] = hpred;
            if (ok && !(a.fixed && a.itype[i] == 1)) {
                // the network predicts the change of the correction
                const float z = fminf(fmaxf(fa[5] + zz, -(float)a.zclip), (float)a.zclip);
                if (a.apply) a.hh[i] = hpred * (double)__expf(0.01f * z);
            }
        }
    }
}

// training: each thread one sample of a 64-sample tile; forward/backward in
// FP32 with the BF16-rounded weights.  A block walks several tiles and keeps
// its share of the parameter gradient in registers (thread q owns parameters
// q, q+64, ...), so each block adds to a parameter once per launch: the
// same-address atomics of the gradient, not the arithmetic, bounded a
// one-tile-per-block launch.
constexpr int TRAIN_BS = 64;
constexpr int TRAIN_PPT = (MLP_NPARAM + TRAIN_BS - 1) / TRAIN_BS;   // parameters per thread
constexpr int TRAIN_MAXBLOCKS = 1024;
__global__ void __launch_bounds__(TRAIN_BS) k_mlp_grad(const float* __restrict__ p, MlpTrainArgs a,
                                                       float* __restrict__ grad, float* __restrict__ loss)
{
    __shared__ float W1[32 * MLP_NIN], B1[32], W2[32 * 32], B2[32], W3[32];
    __shared__ float sx[TRAIN_BS][MLP_NIN + 1];
    __shared__ float sh1[TRAIN_BS][33], sd1[TRAIN_BS][33], sd2[TRAIN_BS][33], sh2[TRAIN_BS][33];
    __shared__ float sdz3[TRAIN_BS];
    for (int k = threadIdx.x; k < 32 * MLP_NIN; k += blockDim.x) W1[k] = bf16r(p[MLP_OFF_W1 + k]);
    for (int k = threadIdx.x; k < 32 * 32; k += blockDim.x) W2[k] = bf16r(p[MLP_OFF_W2 + k]);
    for (int k = threadIdx.x; k < 32; k += blockDim.x) {
        B1[k] = p[MLP_OFF_B1 + k];
        B2[k] = p[MLP_OFF_B2 + k];
        W3[k] = bf16r(p[MLP_OFF_W3 + k]);
    }
    const float b3 = p[MLP_OFF_B3];
    __syncthreads();
    const int tid = threadIdx.x;
    const float inv = 1.0f / (float)a.nbatch;
    float gacc[TRAIN_PPT];
#pragma unroll
    for (int u = 0; u < TRAIN_PPT; u++) gacc[u] = 0.f;
    float lacc = 0.f;
    const int ntiles = (a.nbatch + TRAIN_BS - 1) / TRAIN_BS;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int s = tile * TRAIN_BS + tid;
        const bool valid = s < a.nbatch;
        float x[MLP_NIN], y = 0.f;
        if (valid) {
            if (a.feats) {      // explicit arrays (tests)
                for (int k = 0; k < MLP_NIN; k++) x[k] = a.feats[(size_t)s * MLP_NIN + k];
                y = a.targets[s];
            } else {            // strided sample of the slots
                const long long i = ((long long)s * a.stride + a.offset) % a.n;
                for (int k = 0; k < MLP_NFW; k++) {
                    const float2 v = a.feat[k][i];
                    x[2 * k] = v.x;
                    x[2 * k + 1] = v.y;
                }
                // target: the change of the correction from the previous step
                // (feature 5, y_prev, unrounded), as the inference applies it
                y = 100.f * logf((float)a.hconv[i] / (float)a.hpred[i]) - x[5];
            }
            for (int k = 0; k < MLP_NIN; k++) x[k] = bf16r(x[k]);
        } else {
            for (int k = 0; k < MLP_NIN; k++) x[k] = 0.f;
        }
        // samples without valid features or target (a slot the inference
        // marked, or one without a converged h) add nothing
        bool good = valid && isfinite(y);
        for (int k = 0; k < MLP_NIN; k++) good = good && isfinite(x[k]);
        if (!good) {
            for (int k = 0; k < MLP_NIN; k++) x[k] = 0.f;
            y = 0.f;
        }
        float h1[32], h2[32];
        for (int n = 0; n < 32; n++) {
            float z = B1[n];
            for (int k = 0; k < MLP_NIN; k++) z += W1[n * MLP_NIN + k] * x[k];
            h1[n] = tanhf(z);
        }
        for (int n = 0; n < 32; n++) {
            float z = B2[n];
            for (int k = 0; k < 32; k++) z += W2[n * 32 + k] * h1[k];
            h2[n] = tanhf(z);
        }
        float out = b3;
        for (int k = 0; k < 32; k++) out += W3[k] * h2[k];
        const float r = good ? (out - y) : 0.f;
        const float dz3 = 2.f * r * inv;
        lacc += r * r * inv;
        float dz2[32];
        for (int n = 0; n < 32; n++) dz2[n] = dz3 * W3[n] * (1.f - h2[n] * h2[n]);
        float dz1[32];
        for (int k = 0; k < 32; k++) {
            float acc = 0.f;
            for (int n = 0; n < 32; n++) acc += dz2[n] * W2[n * 32 + k];
            dz1[k] = acc * (1.f - h1[k] * h1[k]);
        }
        for (int k = 0; k < MLP_NIN; k++) sx[tid][k] = x[k];
        for (int k = 0; k < 32; k++) { sh1[tid][k] = h1[k]; sh2[tid][k] = h2[k]; sd1[tid][k] = dz1[k]; sd2[tid][k] = dz2[k]; }
        sdz3[tid] = dz3;
        __syncthreads();
        // this tile's contribution to the parameters the thread owns
#pragma unroll
        for (int u = 0; u < TRAIN_PPT; u++) {
            const int q = tid + u * TRAIN_BS;
            if (q >= MLP_NPARAM) break;
            float acc = 0.f;
            if (q < MLP_OFF_B1) {                              // W1[n][k]
                const int n = q / MLP_NIN, k = q % MLP_NIN;
                for (int m = 0; m < TRAIN_BS; m++) acc += sd1[m][n] * sx[m][k];
            } else if (q < MLP_OFF_W2) {                       // b1[n]
                const int n = q - MLP_OFF_B1;
                for (int m = 0; m < TRAIN_BS; m++) acc += sd1[m][n];
            } else if (q < MLP_OFF_B2) {                       // W2[n][k]
                const int n = (q - MLP_OFF_W2) / 32, k = (q - MLP_OFF_W2) % 32;
                for (int m = 0; m < TRAIN_BS; m++) acc += sd2[m][n] * sh1[m][k];
            } else if (q < MLP_OFF_W3) {                       // b2[n]
                const int n = q - MLP_OFF_B2;
                for (int m = 0; m < TRAIN_BS; m++) acc += sd2[m][n];
            } else if (q < MLP_OFF_B3) {                       // W3[k]
                const int k = q - MLP_OFF_W3;
                for (int m = 0; m < TRAIN_BS; m++) acc += sdz3[m] * sh2[m][k];
            } else {                                           // b3
                for (int m = 0; m < TRAIN_BS; m++) acc += sdz3[m];
            }
            gacc[u] += acc;
        }
        __syncthreads();   // the next tile overwrites the shared arrays
    }
#pragma unroll
    for (int u = 0; u < TRAIN_PPT; u++) {
        const int q = tid + u * TRAIN_BS;
        if (q < MLP_NPARAM) atomicAdd(&grad[q], gacc[u]);
    }
    for (int off = 16; off > 0; off >>= 1) lacc += __shfl_down_sync(0xffffffffu, lacc, off);
    if ((tid & 31) == 0) atomicAdd(loss, lacc);
}

// Adam (Kingma & Ba 2015) on the FP32 master weights
__global__ void k_mlp_adam(float* p, float* m, float* v, float* g, int step, float lr)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= MLP_NPARAM) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float gq = g[q];
    g[q] = 0.f;   // ready for the next minibatch without a memset
    if (!isfinite(gq)) return;   // never let a non-finite gradient into the weights
    const float mq = b1 * m[q] + (1.f - b1) * gq;
    const float vq = b2 * v[q] + (1.f - b2) * gq * gq;
    m[q] = mq;
    v[q] = vq;
    const float mh = mq / (1.f - powf(b1, (float)step));
    const float vh = vq / (1.f - powf(b2, (float)step));
    p[q] -= lr * mh / (sqrtf(vh) + eps);
}

// ---------------------------------------------------------------------------
void mlp_init_params(std::vector<float>& p, unsigned seed)
{
    // deterministic small uniform init (xorshift), last layer zero so the
    // first prediction is the leapfrog predictor itself
    p.assign(MLP_NPARAM, 0.f);
    unsigned s = seed ? seed : 1u;
    auto rnd = [&s]() {
        s ^= s << 13; s ^= s >> 17; s ^= s << 5;
        return (float)(s & 0xffffff) / (float)0x1000000 * 2.f - 1.f;
    };
    const float a1 = sqrtf(6.f / (MLP_NIN + 32)), a2 = sqrtf(6.f / 64.f);
    for (int k = 0; k < 32 * MLP_NIN; k++) p[MLP_OFF_W1 + k] = a1 * rnd();
    for (int k = 0; k < 32 * 32; k++) p[MLP_OFF_W2 + k] = a2 * rnd();
    for (int k = 0; k < 32; k++) p[MLP_OFF_W3 + k] = 0.f;
}

void launch_mlp_pack(const float* p, MlpFrag* fr, cudaStream_t st) { NDSPH_COUNT_LAUNCH, k_mlp_pack<<<1, 32, 0, st>>>(p, fr); }
void launch_mlp_forward(const MlpFrag* fr, const float* feats, int n, float* out, cudaStream_t st)
{
    if (n <= 0) return;
    const int tiles = (n + 15) / 16;
    const int blocks = (tiles + 7) / 8;
    NDSPH_COUNT_LAUNCH, k_mlp_forward<<<blocks, 256, 0, st>>>(fr, feats, n, out);
}
void launch_mlp_infer(const MlpFrag* fr, const MlpInferArgs& a, cudaStream_t st)
{
    if (a.n <= 0) return;
    const int groups = (a.n + 31) / 32;   // 32 slots per warp and pass
    int blocks = (groups + 7) / 8;
    if (blocks > 152 * 16) blocks = 152 * 16;
    NDSPH_COUNT_LAUNCH, k_mlp_infer<<<blocks, 256, 0, st>>>(fr, a);
}
void launch_mlp_grad(const float* p, const MlpTrainArgs& a, float* grad, float* loss, cudaStream_t st)
{
    // grad must be zero on entry (the Adam kernel leaves it so); loss accumulates
    int blocks = (a.nbatch + TRAIN_BS - 1) / TRAIN_BS;
    if (blocks > TRAIN_MAXBLOCKS) blocks = TRAIN_MAXBLOCKS;
    if (blocks < 1) blocks = 1;
    NDSPH_COUNT_LAUNCH, k_mlp_grad<<<blocks, TRAIN_BS, 0, st>>>(p, a, grad, loss);
}
void launch_mlp_adam(float* p, float* m, float* v, float* g, int step, float lr, cudaStream_t st)
{
    NDSPH_COUNT_LAUNCH, k_mlp_adam<<<(MLP_NPARAM + 255) / 256, 256, 0, st>>>(p, m, v, g, step, lr);
}

}  // namespace ndsph
