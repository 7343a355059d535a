// oxg_mlp.cu - the HB + cross-stacking surrogate: training-data sampling from the plain
// evaluator, hand-written training kernels (forward, loss, backward to the weights on
// BF16 tensor cores with FP32 accumulation, Adam) and the inference image the force
// kernels use.
//
// FP32 master parameters of one class (flat, kMlpParams floats): W1[64][16] (input
// columns 7..15 stay zero), b1[64], W2[64][64], b2[64], W3[64][64], b3[64], w4[64], b4.
// Weight matrices are [out][in]. The device image (MlpDev) holds BF16 copies in per-lane
// mma fragment order, rebuilt from the masters after every optimiser step.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/oxdna_gb300.h"
#include "oxg_internal.h"
#include "oxg_mlp.cuh"

using namespace oxg;

namespace {

constexpr int P_W1 = 0, P_B1 = 1024, P_W2 = 1088, P_B2 = 5184, P_W3 = 5248, P_B3 = 9344,
              P_W4 = 9408, P_B4 = 9472;
constexpr int kMlpParams = 9480;  // per class (9473 used, padded)
static_assert(kMlpParams == OXG_MLP_PARAMS, "header and kernels disagree on the parameter count");

#define MCUDA(call)                                                                       \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return internal_set_error(OXG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// ------------------------------------------------------------------ packing
// frag[cls][tile][lane] from the FP32 masters (one thread per (cls, tile, lane)).
__global__ void k_mlp_pack(const float* P, MlpDev* M)
{
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= kMlpClasses * kFragTiles * 32) return;
    const int lane = id & 31, tile = (id >> 5) % kFragTiles, cls = id / (kFragTiles * 32);
    const float* W = P + (size_t)cls * kMlpParams;
    const int g = lane >> 2, t = lane & 3;
    // B[k][n] element for a tile: forward B[k = in][n = out] = W[out][in];
    // backward B[k = out][n = in] = W[out][in]
    float e[4];
    int kt, nt;
    const float* Wm;
    int in_dim;
    bool fwd;
    if (tile < kFragF2) { kt = 0; nt = tile; Wm = W + P_W1; in_dim = 16; fwd = true; }
    else if (tile < kFragF3) { kt = (tile - kFragF2) / 8; nt = (tile - kFragF2) % 8; Wm = W + P_W2; in_dim = 64; fwd = true; }
    else if (tile < kFragG3) { kt = (tile - kFragF3) / 8; nt = (tile - kFragF3) % 8; Wm = W + P_W3; in_dim = 64; fwd = true; }
    else if (tile < kFragG2) { kt = (tile - kFragG3) / 8; nt = (tile - kFragG3) % 8; Wm = W + P_W3; in_dim = 64; fwd = false; }
    else if (tile < kFragG1) { kt = (tile - kFragG2) / 8; nt = (tile - kFragG2) % 8; Wm = W + P_W2; in_dim = 64; fwd = false; }
    else { kt = (tile - kFragG1) / 2; nt = (tile - kFragG1) % 2; Wm = W + P_W1; in_dim = 16; fwd = false; }
    const int n = nt * 8 + g;
    const int ks[4] = {kt * 16 + 2 * t, kt * 16 + 2 * t + 1, kt * 16 + 2 * t + 8, kt * 16 + 2 * t + 9};
    for (int q = 0; q < 4; ++q) e[q] = fwd ? Wm[n * in_dim + ks[q]] : Wm[ks[q] * in_dim + n];
    M->frag[cls][tile][lane] = make_uint2(pack_bf16(e[0], e[1]), pack_bf16(e[2], e[3]));
}

// vectors (biases, w4, b4) of both classes; the normalisation is set separately
__global__ void k_mlp_pack_vec(const float* P, MlpDev* M)
{
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= kMlpClasses * kMlpHid) return;
    const int cls = id / kMlpHid, j = id % kMlpHid;
    const float* W = P + (size_t)cls * kMlpParams;
    MlpVec& V = M->vec[cls];
    V.b1[j] = W[P_B1 + j];
    V.b2[j] = W[P_B2 + j];
    V.b3[j] = W[P_B3 + j];
    V.w4[j] = W[P_W4 + j];
    if (j == 0) V.b4 = W[P_B4];
}

// ------------------------------------------------------------------ training
struct TrainArgs {
    const MlpDev* M;
    int cls;
    const float* feats;   // n x 8 (7 raw features, class)
    const float* target;  // n energies
    const int* idx;       // minibatch sample indices
    int nb;               // minibatch size
    float* grad;          // kMlpParams (this class), accumulated
    double* loss;         // sum of squared errors in normalised units, accumulated
};

constexpr int kTrainWarps = 4;
// per-warp transposed activations [unit][sample] (BF16) used as the weight-gradient
// GEMM operands, and the block's gradient accumulators
struct TrainSmem {
    __nv_bfloat16 xT[kTrainWarps][16][16];
    __nv_bfloat16 h1T[kTrainWarps][64][16];
    __nv_bfloat16 h2T[kTrainWarps][64][16];
    __nv_bfloat16 dzT[kTrainWarps][64][16];
    float g[kMlpParams];
};

__device__ __forceinline__ void store_T(__nv_bfloat16 (*T)[16], const float (*c)[4], int lane)
{
    const int g = lane >> 2;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int e = 0; e < 4; ++e) T[frag_col(nt, e, lane)][g + (e >> 1) * 8] = __float2bfloat16_rn(c[nt][e]);
}

__device__ __forceinline__ uint32_t ld2(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// dW[j][k] += sum_s dz[s][j] * h[s][k] for j < 64, k < 16 * NK (A = dz^T, B from h^T)
template <int NT>
__device__ __forceinline__ void weight_grad(const __nv_bfloat16 (*dzT)[16], const __nv_bfloat16 (*hT)[16],
                                            float* gW, int in_dim, int lane)
{
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int mt = 0; mt < 4; ++mt) {
        const int j = mt * 16 + g;
        const uint32_t a0 = ld2(&dzT[j][2 * t]), a1 = ld2(&dzT[j + 8][2 * t]);
        const uint32_t a2 = ld2(&dzT[j][2 * t + 8]), a3 = ld2(&dzT[j + 8][2 * t + 8]);
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const int k = nt * 8 + g;
            const uint2 b = make_uint2(ld2(&hT[k][2 * t]), ld2(&hT[k][2 * t + 8]));
            float d[4] = {0.f, 0.f, 0.f, 0.f};
            mma_bf16(d, a0, a1, a2, a3, b);
            const int c0 = nt * 8 + 2 * t;
            atomicAdd(&gW[j * in_dim + c0], d[0]);
            atomicAdd(&gW[j * in_dim + c0 + 1], d[1]);
            atomicAdd(&gW[(j + 8) * in_dim + c0], d[2]);
            atomicAdd(&gW[(j + 8) * in_dim + c0 + 1], d[3]);
        }
    }
}

// db[j] += sum over the 16 rows of the C fragments c
__device__ __forceinline__ void bias_grad(const float (*c)[4], float* gb, int lane)
{
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        float v0 = c[nt][0] + c[nt][2], v1 = c[nt][1] + c[nt][3];
#pragma unroll
        for (int o = 4; o < 32; o <<= 1) {
            v0 += __shfl_xor_sync(0xffffffffu, v0, o);
            v1 += __shfl_xor_sync(0xffffffffu, v1, o);
        }
        if (lane < 4) {
            atomicAdd(&gb[frag_col(nt, 0, lane)], v0);
            atomicAdd(&gb[frag_col(nt, 1, lane)], v1);
        }
    }
}

// One minibatch: loss L = sum_s (y_s - y*_s)^2 / nb in normalised energy units and its
// gradient with respect to every parameter of the class, accumulated into a.grad.
__global__ void __launch_bounds__(kTrainWarps * 32) k_mlp_train(TrainArgs a)
{
    extern __shared__ float4 smem_train[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>(smem_train);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    for (int k = threadIdx.x; k < kMlpParams; k += blockDim.x) S.g[k] = 0.f;
    const MlpDev& M = *a.M;
    const MlpVec& V = M.vec[a.cls];
    const uint2* F = &M.frag[a.cls][0][0];
    double sse = 0.0;
    __syncthreads();
    const int chunks = (a.nb + 15) / 16;
    for (int ch = blockIdx.x * kTrainWarps + w; ch < chunks; ch += gridDim.x * kTrainWarps) {
        // row r = lane & 15: its sample, normalised features and target
        const int r = lane & 15;
        const int sidx = ch * 16 + r;
        const bool valid = sidx < a.nb;
        float x[kMlpIn], yt = 0.f;
        if (valid) {
            const int s = a.idx[sidx];
#pragma unroll
            for (int f = 0; f < kMlpIn; ++f) x[f] = (a.feats[(size_t)s * 8 + f] - V.mu[f]) * V.inv_sd[f];
            yt = (a.target[s] - V.e_shift) / V.e_scale;
        } else {
#pragma unroll
            for (int f = 0; f < kMlpIn; ++f) x[f] = 0.f;
        }
        // x^T for the first layer's weight gradient (rows 7..15 zero)
        if (lane < 16) {
#pragma unroll
            for (int f = 0; f < 16; ++f) S.xT[w][f][r] = __float2bfloat16_rn(f < kMlpIn ? x[f] : 0.f);
        }
        // forward (as mlp_rows16)
        float xg[kMlpIn], xg8[kMlpIn];
#pragma unroll
        for (int f = 0; f < kMlpIn; ++f) {
            xg[f] = __shfl_sync(0xffffffffu, x[f], g);
            xg8[f] = __shfl_sync(0xffffffffu, x[f], g + 8);
        }
        auto pick = [&](const float* v, int f) {
            float q = 0.f;
#pragma unroll
            for (int k = 0; k < kMlpIn; ++k) q = (k == f) ? v[k] : q;
            return q;
        };
        uint32_t A0[1][4];
        A0[0][0] = pack_bf16(pick(xg, 2 * t), pick(xg, 2 * t + 1));
        A0[0][1] = pack_bf16(pick(xg8, 2 * t), pick(xg8, 2 * t + 1));
        A0[0][2] = 0u;
        A0[0][3] = 0u;
        float z1[8][4], s1[8][4], z2[8][4], s2[8][4], z3[8][4];
        uint32_t A[4][4];
        mlp_layer<1>(F + kFragF1 * 32, A0, z1, lane);
        bias_silu(z1, s1, V.b1, lane);
        store_T(S.h1T[w], z1, lane);
        c_to_a(z1, A);
        mlp_layer<4>(F + kFragF2 * 32, A, z2, lane);
        bias_silu(z2, s2, V.b2, lane);
        store_T(S.h2T[w], z2, lane);
        c_to_a(z2, A);
        mlp_layer<4>(F + kFragF3 * 32, A, z3, lane);
        float s3[8][4];
        bias_silu(z3, s3, V.b3, lane);
        float yg = 0.f, yg8 = 0.f;
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const float w0 = V.w4[frag_col(nt, 0, lane)], w1 = V.w4[frag_col(nt, 1, lane)];
            yg += z3[nt][0] * w0 + z3[nt][1] * w1;
            yg8 += z3[nt][2] * w0 + z3[nt][3] * w1;
        }
        yg += __shfl_xor_sync(0xffffffffu, yg, 1);
        yg += __shfl_xor_sync(0xffffffffu, yg, 2);
        yg8 += __shfl_xor_sync(0xffffffffu, yg8, 1);
        yg8 += __shfl_xor_sync(0xffffffffu, yg8, 2);
        yg += V.b4;
        yg8 += V.b4;
        // dL/dy of rows g and g + 8
        const float tg = __shfl_sync(0xffffffffu, yt, g), tg8 = __shfl_sync(0xffffffffu, yt, g + 8);
        const bool vg = __shfl_sync(0xffffffffu, valid, g), vg8 = __shfl_sync(0xffffffffu, valid, g + 8);
        const float dg = vg ? 2.f * (yg - tg) / (float)a.nb : 0.f;
        const float dg8 = vg8 ? 2.f * (yg8 - tg8) / (float)a.nb : 0.f;
        {
            // squared error: lanes with t == 0 hold rows g and g + 8
            const float e0 = vg ? (yg - tg) : 0.f, e1 = vg8 ? (yg8 - tg8) : 0.f;
            if (t == 0) sse += (double)e0 * e0 + (double)e1 * e1;
        }
        // output layer: dw4[j] = sum_s dL/dy_s h3[s][j]; db4 = sum_s dL/dy_s
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            float v0 = dg * z3[nt][0] + dg8 * z3[nt][2], v1 = dg * z3[nt][1] + dg8 * z3[nt][3];
#pragma unroll
            for (int o = 4; o < 32; o <<= 1) {
                v0 += __shfl_xor_sync(0xffffffffu, v0, o);
                v1 += __shfl_xor_sync(0xffffffffu, v1, o);
            }
            if (lane < 4) {
                atomicAdd(&S.g[P_W4 + frag_col(nt, 0, lane)], v0);
                atomicAdd(&S.g[P_W4 + frag_col(nt, 1, lane)], v1);
            }
        }
        {
            float v = (t == 0) ? dg + dg8 : 0.f;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) atomicAdd(&S.g[P_B4], v);
        }
        // dz3 = dL/dy * w4 * silu'(z3)
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const float w0 = V.w4[frag_col(nt, 0, lane)], w1 = V.w4[frag_col(nt, 1, lane)];
            s3[nt][0] *= dg * w0;
            s3[nt][1] *= dg * w1;
            s3[nt][2] *= dg8 * w0;
            s3[nt][3] *= dg8 * w1;
        }
        bias_grad(s3, S.g + P_B3, lane);
        store_T(S.dzT[w], s3, lane);
        __syncwarp();
        weight_grad<8>(S.dzT[w], S.h2T[w], S.g + P_W3, 64, lane);
        c_to_a(s3, A);
        mlp_layer<4>(F + kFragG3 * 32, A, z2, lane);  // dL/dh2
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e) s2[nt][e] *= z2[nt][e];
        bias_grad(s2, S.g + P_B2, lane);
        __syncwarp();
        store_T(S.dzT[w], s2, lane);
        __syncwarp();
        weight_grad<8>(S.dzT[w], S.h1T[w], S.g + P_W2, 64, lane);
        c_to_a(s2, A);
        mlp_layer<4>(F + kFragG2 * 32, A, z1, lane);  // dL/dh1
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e) s1[nt][e] *= z1[nt][e];
        bias_grad(s1, S.g + P_B1, lane);
        __syncwarp();
        store_T(S.dzT[w], s1, lane);
        __syncwarp();
        weight_grad<2>(S.dzT[w], S.xT[w], S.g + P_W1, 16, lane);
        __syncwarp();
    }
    // loss and the block's gradient into the global accumulators
    for (int o = 16; o > 0; o >>= 1) sse += __shfl_xor_sync(0xffffffffu, sse, o);
    if (lane == 0 && sse != 0.0) atomicAdd(a.loss, sse);
    __syncthreads();
    for (int k = threadIdx.x; k < kMlpParams; k += blockDim.x)
        if (S.g[k] != 0.f) atomicAdd(a.grad + k, S.g[k]);
}

// Adam on the masters of one class; zeroes the gradient. Input columns 7..15 of W1 stay 0.
__global__ void k_mlp_adam(float* P, float* G, float* m1, float* m2, int n, float lr, float b1,
                           float b2, float eps, float c1, float c2)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float gk = G[k];
    G[k] = 0.f;
    if (k < P_B1 && (k & 15) >= kMlpIn) return;
    const float mk = b1 * m1[k] + (1.f - b1) * gk;
    const float vk = b2 * m2[k] + (1.f - b2) * gk * gk;
    m1[k] = mk;
    m2[k] = vk;
    P[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + eps);
}

// Network outputs for contiguous samples of one class (tests, audits): y and dy/dx' in
// normalised units, one warp per 16 samples.
__global__ void k_mlp_predict(const MlpDev* M, int cls, const float* feats, int n, float* y,
                              float* dydx)
{
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    const MlpVec& V = M->vec[cls];
    for (int base = gw * 16; base < n; base += nw * 16) {
        const int s = base + (lane & 15);
        float x[kMlpIn];
#pragma unroll
        for (int f = 0; f < kMlpIn; ++f) x[f] = s < n ? (feats[(size_t)s * 8 + f] - V.mu[f]) * V.inv_sd[f] : 0.f;
        float yy, d[kMlpIn];
        mlp_rows16(*M, cls, x, yy, d);
        if (lane < 16 && s < n) {
            y[s] = yy;
#pragma unroll
            for (int f = 0; f < kMlpIn; ++f) dydx[(size_t)s * kMlpIn + f] = d[f];
        }
    }
}

}  // namespace

struct oxg_mlp {
    MlpDev* dev = nullptr;
    float* P = nullptr;   // masters, kMlpClasses * kMlpParams
    float* G = nullptr;   // gradients
    float* m1 = nullptr;  // Adam moments
    float* m2 = nullptr;
    double* loss = nullptr;
    int adam_t[kMlpClasses] = {0, 0};
    MlpVec vec_host[kMlpClasses];
};

namespace {

int mlp_repack(oxg_mlp* m, cudaStream_t st)
{
    const int n = kMlpClasses * kFragTiles * 32;
    k_mlp_pack<<<(n + 255) / 256, 256, 0, st>>>(m->P, m->dev);
    k_mlp_pack_vec<<<1, kMlpClasses * kMlpHid, 0, st>>>(m->P, m->dev);
    MCUDA(cudaGetLastError());
    return OXG_OK;
}

}  // namespace

namespace oxg {
const void* internal_mlp_device(const oxg_mlp* m) { return m ? m->dev : nullptr; }
}  // namespace oxg

extern "C" {

int oxg_mlp_create(oxg_mlp** out)
{
    if (!out) return internal_set_error(OXG_ERR_INVALID_ARG, "null output");
    oxg_mlp* m = new oxg_mlp();
    const size_t np = (size_t)kMlpClasses * kMlpParams;
    if (cudaMalloc(&m->dev, sizeof(MlpDev)) != cudaSuccess || cudaMalloc(&m->P, np * 4) != cudaSuccess ||
        cudaMalloc(&m->G, np * 4) != cudaSuccess || cudaMalloc(&m->m1, np * 4) != cudaSuccess ||
        cudaMalloc(&m->m2, np * 4) != cudaSuccess || cudaMalloc(&m->loss, sizeof(double)) != cudaSuccess) {
        oxg_mlp_destroy(m);
        return internal_set_error(OXG_ERR_CUDA, "cudaMalloc failed");
    }
    cudaMemset(m->dev, 0, sizeof(MlpDev));
    cudaMemset(m->P, 0, np * 4);
    cudaMemset(m->G, 0, np * 4);
    cudaMemset(m->m1, 0, np * 4);
    cudaMemset(m->m2, 0, np * 4);
    for (int c = 0; c < kMlpClasses; ++c) {
        std::memset(&m->vec_host[c], 0, sizeof(MlpVec));
        for (int f = 0; f < kMlpIn; ++f) m->vec_host[c].inv_sd[f] = 1.f;
        m->vec_host[c].e_scale = 1.f;
    }
    for (int c = 0; c < kMlpClasses; ++c) {
        const int rc = oxg_mlp_set_normalization(m, c, m->vec_host[c].mu, m->vec_host[c].inv_sd, 1.f, 0.f);
        if (rc) {
            oxg_mlp_destroy(m);
            return rc;
        }
    }
    *out = m;
    return OXG_OK;
}

int oxg_mlp_destroy(oxg_mlp* m)
{
    if (!m) return OXG_OK;
    cudaFree(m->dev);
    cudaFree(m->P);
    cudaFree(m->G);
    cudaFree(m->m1);
    cudaFree(m->m2);
    cudaFree(m->loss);
    delete m;
    return OXG_OK;
}

int oxg_mlp_set_params(oxg_mlp* m, const float* params)
{
    if (!m || !params) return internal_set_error(OXG_ERR_INVALID_ARG, "bad arguments");
    std::vector<float> p(params, params + (size_t)kMlpClasses * kMlpParams);
    for (int c = 0; c < kMlpClasses; ++c)
        for (int j = 0; j < 64; ++j)
            for (int f = kMlpIn; f < 16; ++f) p[(size_t)c * kMlpParams + P_W1 + j * 16 + f] = 0.f;
    MCUDA(cudaMemcpy(m->P, p.data(), p.size() * 4, cudaMemcpyHostToDevice));
    const size_t np = (size_t)kMlpClasses * kMlpParams * 4;
    MCUDA(cudaMemset(m->m1, 0, np));
    MCUDA(cudaMemset(m->m2, 0, np));
    m->adam_t[0] = m->adam_t[1] = 0;
    int rc = mlp_repack(m, nullptr);
    if (rc) return rc;
    MCUDA(cudaDeviceSynchronize());
    return OXG_OK;
}

int oxg_mlp_get_params(oxg_mlp* m, float* params)
{
    if (!m || !params) return internal_set_error(OXG_ERR_INVALID_ARG, "bad arguments");
    MCUDA(cudaMemcpy(params, m->P, (size_t)kMlpClasses * kMlpParams * 4, cudaMemcpyDeviceToHost));
    return OXG_OK;
}

int oxg_mlp_set_normalization(oxg_mlp* m, int cls, const float* mu, const float* inv_sd,
                              float e_scale, float e_shift)
{
    if (!m || cls < 0 || cls >= kMlpClasses || !mu || !inv_sd || !(e_scale != 0.f))
        return internal_set_error(OXG_ERR_INVALID_ARG, "bad arguments");
    MlpVec& v = m->vec_host[cls];
    for (int f = 0; f < kMlpIn; ++f) {
        v.mu[f] = mu[f];
        v.inv_sd[f] = inv_sd[f];
    }
    v.e_scale = e_scale;
    v.e_shift = e_shift;
    // only the normalisation fields: the biases and w4 come from the masters
    MlpVec* d = &m->dev->vec[cls];
    MCUDA(cudaMemcpy(d->mu, v.mu, sizeof(v.mu), cudaMemcpyHostToDevice));
    MCUDA(cudaMemcpy(d->inv_sd, v.inv_sd, sizeof(v.inv_sd), cudaMemcpyHostToDevice));
    MCUDA(cudaMemcpy(&d->e_scale, &v.e_scale, sizeof(float), cudaMemcpyHostToDevice));
    MCUDA(cudaMemcpy(&d->e_shift, &v.e_shift, sizeof(float), cudaMemcpyHostToDevice));
    return OXG_OK;
}

int oxg_mlp_gradient(oxg_mlp* m, int cls, const float* feats, const float* target, const int* idx,
                     int nb, float* grad_host, double* loss_host, void* stream)
{
    if (!m || cls < 0 || cls >= kMlpClasses || !feats || !target || !idx || nb <= 0)
        return internal_set_error(OXG_ERR_INVALID_ARG, "bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    TrainArgs a;
    a.M = m->dev;
    a.cls = cls;
    a.feats = feats;
    a.target = target;
    a.idx = idx;
    a.nb = nb;
    a.grad = m->G + (size_t)cls * kMlpParams;
    a.loss = m->loss;
    MCUDA(cudaMemsetAsync(m->loss, 0, sizeof(double), st));
    const int smem = (int)sizeof(TrainSmem);
    MCUDA(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    const int chunks = (nb + 15) / 16;
    const int blocks = std::max(1, std::min((chunks + kTrainWarps - 1) / kTrainWarps, 2 * internal_num_sms()));
    k_mlp_train<<<blocks, kTrainWarps * 32, smem, st>>>(a);
    MCUDA(cudaGetLastError());
    if (grad_host) {
        MCUDA(cudaMemcpyAsync(grad_host, a.grad, kMlpParams * 4, cudaMemcpyDeviceToHost, st));
        MCUDA(cudaMemsetAsync(a.grad, 0, kMlpParams * 4, st));
    }
    if (loss_host) MCUDA(cudaMemcpyAsync(loss_host, m->loss, sizeof(double), cudaMemcpyDeviceToHost, st));
    if (grad_host || loss_host) MCUDA(cudaStreamSynchronize(st));
    return OXG_OK;
}

int oxg_mlp_train_step(oxg_mlp* m, int cls, const float* feats, const float* target, const int* idx,
                       int nb, float lr, double* loss_host, void* stream)
{
    int rc = oxg_mlp_gradient(m, cls, feats, target, idx, nb, nullptr, loss_host, stream);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int t = ++m->adam_t[cls];
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)t), c2 = 1.f - std::pow(b2, (float)t);
    const size_t off = (size_t)cls * kMlpParams;
    k_mlp_adam<<<(kMlpParams + 255) / 256, 256, 0, st>>>(m->P + off, m->G + off, m->m1 + off, m->m2 + off,
                                                         kMlpParams, lr, b1, b2, 1e-8f, c1, c2);
    MCUDA(cudaGetLastError());
    return mlp_repack(m, st);
}

int oxg_mlp_predict(oxg_mlp* m, int cls, const float* feats, int n, float* y, float* dydx, void* stream)
{
    if (!m || cls < 0 || cls >= kMlpClasses || !feats || n < 0 || !y || !dydx)
        return internal_set_error(OXG_ERR_INVALID_ARG, "bad arguments");
    if (n == 0) return OXG_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int warps = (n + 15) / 16;
    const int blocks = std::min((warps + 7) / 8, 8 * internal_num_sms());
    k_mlp_predict<<<blocks, 256, 0, st>>>(m->dev, cls, feats, n, y, dydx);
    MCUDA(cudaGetLastError());
    MCUDA(cudaStreamSynchronize(st));
    return OXG_OK;
}

}  // extern "C"
