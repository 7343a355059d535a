// oxg_mlp.cu - the HB + cross-stacking surrogate: hand-written training kernels (forward,
// loss, backward to the weights with every GEMM on the tcgen05 tensor cores, BF16
// operands and FP32 accumulation in tensor memory; Adam), batch inference, and the
// device image the force kernels use.
//
// FP32 master parameters of one class (flat, kMlpParams floats): W1[64][16] (input
// columns 7..15 stay zero), b1[64], W2[64][64], b2[64], W3[64][64], b3[64], w4[64], b4.
// Weight matrices are [out][in]. The device image (MlpDev) holds BF16 copies as the six
// GEMMs' B operands in the canonical K-major layout, rebuilt from the masters after
// every optimiser step.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/oxdna_gb300.h"
#include "oxg_internal.h"
#include "oxg_mlp.cuh"
#include "oxg_tc.cuh"

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

// ------------------------------------------------------------------ tcgen05 images
// The B operands of one class in the canonical K-major layout (oxg_tc.cuh), one thread
// per element: forward F (n = output, k = input): W[n][k]; backward G (n = input, k =
// output): W[k][n]; each as hi = bf16(w) and lo = bf16(w - hi) images (F1 also carries
// W1_hi in input columns 7..13 for the inputs' low parts, G1 carries W1_lo in rows 7..13).
constexpr int kPackPerClass = 3 * 1024 + 8 * 4096;

__device__ __forceinline__ float bf16_hi(float w) { return __bfloat162float(__float2bfloat16_rn(w)); }

__global__ void k_mlp_pack_tc(const float* P, MlpDev* M)
{
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= kMlpClasses * kPackPerClass) return;
    const int cls = id / kPackPerClass;
    int e = id % kPackPerClass;
    const float* W = P + (size_t)cls * kMlpParams;
    unsigned char* img = M->tcw[cls];
    float v = 0.f;
    uint32_t off;
    if (e < 2048) {  // F1 (hi) and F1L: 64 x 16
        const bool lo = e >= 1024;
        const int n = (e & 1023) >> 4, k = e & 15;
        if (k < kMlpIn) {
            const float w = W[P_W1 + n * 16 + k];
            v = lo ? w - bf16_hi(w) : w;
        } else if (!lo && k < 2 * kMlpIn) {
            v = W[P_W1 + n * 16 + k - kMlpIn];
        }
        off = (lo ? tc::kImgF1L : tc::kImgF1) + tc::kmaj_off(64, n, k);
    } else if ((e -= 2048) < 8 * 4096) {  // F2, F3, G3, G2, then their lo images: 64 x 64
        const bool lo = e >= 4 * 4096;
        const int m = (e >> 12) & 3, n = (e >> 6) & 63, k = e & 63;
        const float* Wm = W + ((m == 0 || m == 3) ? P_W2 : P_W3);
        const float w = m < 2 ? Wm[n * 64 + k] : Wm[k * 64 + n];
        v = lo ? w - bf16_hi(w) : w;
        const uint32_t base = lo ? (m == 0 ? tc::kImgF2L : m == 1 ? tc::kImgF3L : m == 2 ? tc::kImgG3L : tc::kImgG2L)
                                 : (m == 0 ? tc::kImgF2 : m == 1 ? tc::kImgF3 : m == 2 ? tc::kImgG3 : tc::kImgG2);
        off = base + tc::kmaj_off(64, n, k);
    } else {  // G1: 16 (inputs: hi rows, then lo rows) x 64 (outputs)
        e -= 8 * 4096;
        const int n = e >> 6, k = e & 63;
        if (n < kMlpIn) {
            v = W[P_W1 + k * 16 + n];
        } else if (n < 2 * kMlpIn) {
            const float w = W[P_W1 + k * 16 + n - kMlpIn];
            v = w - bf16_hi(w);
        }
        off = tc::kImgG1 + tc::kmaj_off(16, n, k);
    }
    *reinterpret_cast<__nv_bfloat16*>(img + off) = __float2bfloat16_rn(v);
}

// ------------------------------------------------------------------ training (tcgen05)
struct TrainArgs {
    const MlpDev* M;
    int cls;
    const float* feats;   // n x 8 (7 raw features, class)
    const float* target;  // n energies
    const int* idx;       // minibatch sample indices
    int nb;               // minibatch size
    float* grad;          // kMlpParams (this class), accumulated
    double* loss;         // sum of squared errors in normalised units, accumulated
    uint32_t* err;        // set when an MMA wait gave up
};

// Shared-memory plan of the training kernel (bytes). Weight-gradient GEMMs contract over
// the 128 samples of a tile: A = dZ^T (128 rows: the 64 units, then zeros), B = H^T (80
// rows: the 64 inputs, a row of ones that yields the bias gradient, zeros) or X^T (32
// rows: 16 inputs, ones, zeros). 32 KB of slack follow the last operand.
constexpr uint32_t kTrW = 0, kTrX = tc::kImgBytes, kTrP = kTrX + kTcX, kTrQ = kTrP + kTcAct, kTrXT = kTrQ + kTcAct,
                   kTrH1T = kTrXT + 32 * 128 * 2, kTrH2T = kTrH1T + 80 * 128 * 2, kTrDZT = kTrH2T + 80 * 128 * 2,
                   kTrRed = kTrDZT + 128 * 128 * 2, kTrBytes = kTrRed + 4 * 65 * 4 + 32768;
static_assert(kTrBytes + 1024 <= 227 * 1024, "training kernel exceeds the shared memory of a block");
// tensor-memory columns of the weight gradients (after D1..D4)
constexpr uint32_t kColDW3 = 256, kColDW2 = 336, kColDW1 = 416;

// One minibatch: L = sum_s (y_s - y*_s)^2 / nb (normalised units) and its gradient with
// respect to every parameter of the class, accumulated into a.grad. A block of 128
// threads takes tiles of 128 samples; the weight gradients accumulate in tensor memory
// over the block's tiles and are added to a.grad once at the end.
__global__ void __launch_bounds__(128, 1) k_mlp_train(TrainArgs a)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const MlpVec& V = a.M->vec[a.cls];
    tc_load_weights(sm + kTrW, a.M->tcw[a.cls]);
    // constant rows of the weight-gradient operands: ones (bias gradients) and zeros
    st_bf16(sm + kTrXT, tc::kmaj_off(32, 16, tid), 1.f);
    for (int r = 17; r < 32; ++r) st_bf16(sm + kTrXT, tc::kmaj_off(32, r, tid), 0.f);
    st_bf16(sm + kTrH1T, tc::kmaj_off(80, 64, tid), 1.f);
    st_bf16(sm + kTrH2T, tc::kmaj_off(80, 64, tid), 1.f);
    for (int r = 65; r < 80; ++r) {
        st_bf16(sm + kTrH1T, tc::kmaj_off(80, r, tid), 0.f);
        st_bf16(sm + kTrH2T, tc::kmaj_off(80, r, tid), 0.f);
    }
    for (int r = 64; r < 128; ++r) st_bf16(sm + kTrDZT, tc::kmaj_off(128, r, tid), 0.f);
    float* red = reinterpret_cast<float*>(sm + kTrRed);
    for (int k = tid; k < 4 * 65; k += 128) red[k] = 0.f;
    if (warp == 0) tc::tmem_alloc(tc::smem_addr(&tmem_base), 512);
    if (tid == 0) tc::mbar_init(tc::smem_addr(&mbar), 1);
    tc::fence_smem_async();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    TcTile t;
    t.w = sm + kTrW;
    t.x = sm + kTrX;
    t.p = sm + kTrP;
    t.q = sm + kTrQ;
    t.mbar = tc::smem_addr(&mbar);
    t.tmem = tmem_base;
    t.bar_id = 1;
    const uint32_t lane_t = t.tmem + ((uint32_t)(warp * 32) << 16);
    uint32_t phase = 0;
    bool ok = true;
    double sse = 0.0;
    float gb4 = 0.f;
    bool first = true;
    const int tiles = (a.nb + kTcRows - 1) / kTcRows;
    for (int tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
        const int sidx = tile * kTcRows + tid;
        const bool valid = sidx < a.nb;
        float x[16], yt = 0.f;
#pragma unroll
        for (int f = 0; f < 16; ++f) x[f] = 0.f;
        if (valid) {
            const int sI = a.idx[sidx];
#pragma unroll
            for (int f = 0; f < kMlpIn; ++f) x[f] = (a.feats[(size_t)sI * 8 + f] - V.mu[f]) * V.inv_sd[f];
            yt = (a.target[sI] - V.e_shift) / V.e_scale;
        }
        float xr[16];
        split_inputs(x, xr);
        tc::st_row8(t.x, tc::kmaj_off(128, tid, 0), xr);
        tc::st_row8(t.x, tc::kmaj_off(128, tid, 8), xr + 8);
        // (the W1 gradient takes input rows 0..6 of X^T: the inputs' BF16 parts)
#pragma unroll
        for (int f = 0; f < 16; ++f) st_bf16(sm + kTrXT, tc::kmaj_off(32, f, tid), xr[f]);
        // forward (weights as hi + lo, as in inference), keeping the activations'
        // transposes for the weight gradients
        tc_publish(t);
        ok &= tc_gemm_split(t, phase, 0, t.x, 128, t.w + tc::kImgF1, t.w + tc::kImgF1L, 64, 64, 1);
        tc_forward_row(lane_t, 0, V.b1, t.p, tid, sm + kTrH1T, 80);
        tc_publish(t);
        ok &= tc_gemm_split(t, phase, 64, t.p, 128, t.w + tc::kImgF2, t.w + tc::kImgF2L, 64, 64, 4);
        tc_forward_row(lane_t, 64, V.b2, t.q, tid, sm + kTrH2T, 80);
        tc_publish(t);
        ok &= tc_gemm_split(t, phase, 128, t.q, 128, t.w + tc::kImgF3, t.w + tc::kImgF3L, 64, 64, 4);
        // output, loss, dL/dy (first pass over z3); dz3 = dL/dy * w4 * silu'(z3) and the
        // w4 gradient dL/dy * h3 (second pass; warp sums into the block's accumulators)
        {
            float y = V.b4;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                float z[16];
                tc::ld16(lane_t + 128 + 16 * c, z);
#pragma unroll
                for (int e = 0; e < 16; ++e) {
                    float h;
                    (void)tc::silu_and_grad(z[e] + V.b3[16 * c + e], h);
                    y += h * V.w4[16 * c + e];
                }
            }
            const float err = valid ? y - yt : 0.f;
            sse += (double)err * err;
            const float dy = 2.f * err / (float)a.nb;
            gb4 += dy;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                float z[16], dz[16];
                tc::ld16(lane_t + 128 + 16 * c, z);
#pragma unroll
                for (int e = 0; e < 16; ++e) {
                    const int j = 16 * c + e;
                    float h;
                    const float sp = tc::silu_and_grad(z[e] + V.b3[j], h);
                    dz[e] = dy * V.w4[j] * sp;
                    st_bf16(sm + kTrDZT, tc::kmaj_off(128, j, tid), dz[e]);
                    float v = dy * h;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                    if (lane == 0) red[warp * 65 + j] += v;
                }
                tc::st_row8(t.p, tc::kmaj_off(128, tid, 16 * c), dz);
                tc::st_row8(t.p, tc::kmaj_off(128, tid, 16 * c + 8), dz + 8);
            }
        }
        tc_publish(t);
        // dH2 = dZ3 G3 and DW3 += dZ3^T H2 (with db3 in column 64)
        if (tid == 0) {
            tc::fence_after();
            const uint32_t id64 = tc::idesc_bf16(128, 64), id80 = tc::idesc_bf16(128, 80);
            const uint32_t sp_ = tc::smem_addr(t.p), sg = tc::smem_addr(t.w + tc::kImgG3);
            const uint32_t sgl = tc::smem_addr(t.w + tc::kImgG3L);
            const uint32_t sdz = tc::smem_addr(sm + kTrDZT), sh = tc::smem_addr(sm + kTrH2T);
            for (int j = 0; j < 4; ++j) tc::mma(t.tmem + 192, tc::op_desc(sp_, 128, j), tc::op_desc(sg, 64, j), id64, j > 0);
            for (int j = 0; j < 4; ++j) tc::mma(t.tmem + 192, tc::op_desc(sp_, 128, j), tc::op_desc(sgl, 64, j), id64, 1u);
            for (int j = 0; j < 8; ++j)
                tc::mma(t.tmem + kColDW3, tc::op_desc(sdz, 128, j), tc::op_desc(sh, 80, j), id80, (!first || j > 0));
            tc::commit(t.mbar);
        }
        ok &= tc::mbar_wait(t.mbar, phase);
        phase ^= 1u;
        tc::fence_after();
        tc_backward_row(lane_t, 64, t.q, tid, sm + kTrDZT);  // dZ2 into Q and dZ2^T
        tc_publish(t);
        // dH1 = dZ2 G2 and DW2 += dZ2^T H1
        if (tid == 0) {
            tc::fence_after();
            const uint32_t id64 = tc::idesc_bf16(128, 64), id80 = tc::idesc_bf16(128, 80);
            const uint32_t sq = tc::smem_addr(t.q), sg = tc::smem_addr(t.w + tc::kImgG2);
            const uint32_t sgl = tc::smem_addr(t.w + tc::kImgG2L);
            const uint32_t sdz = tc::smem_addr(sm + kTrDZT), sh = tc::smem_addr(sm + kTrH1T);
            for (int j = 0; j < 4; ++j) tc::mma(t.tmem + 192, tc::op_desc(sq, 128, j), tc::op_desc(sg, 64, j), id64, j > 0);
            for (int j = 0; j < 4; ++j) tc::mma(t.tmem + 192, tc::op_desc(sq, 128, j), tc::op_desc(sgl, 64, j), id64, 1u);
            for (int j = 0; j < 8; ++j)
                tc::mma(t.tmem + kColDW2, tc::op_desc(sdz, 128, j), tc::op_desc(sh, 80, j), id80, (!first || j > 0));
            tc::commit(t.mbar);
        }
        ok &= tc::mbar_wait(t.mbar, phase);
        phase ^= 1u;
        tc::fence_after();
        tc_backward_row(lane_t, 0, nullptr, tid, sm + kTrDZT);  // dZ1^T only (DW1 += dZ1^T X)
        tc_publish(t);
        if (tid == 0) {
            tc::fence_after();
            const uint32_t id32 = tc::idesc_bf16(128, 32);
            const uint32_t sdz = tc::smem_addr(sm + kTrDZT), sx = tc::smem_addr(sm + kTrXT);
            for (int j = 0; j < 8; ++j)
                tc::mma(t.tmem + kColDW1, tc::op_desc(sdz, 128, j), tc::op_desc(sx, 32, j), id32, (!first || j > 0));
            tc::commit(t.mbar);
        }
        ok &= tc::mbar_wait(t.mbar, phase);
        phase ^= 1u;
        tc::fence_after();
        tc::fence_before();
        ok = __syncthreads_and(ok) != 0;
        tc::fence_after();
        first = false;
    }
    // the block's gradients: weights (and b1..b3) from tensor memory, rows = units 0..63
    if (!first && ok && warp < 2) {
        const int j = tid;  // unit
        float* g = a.grad;
#pragma unroll
        for (int c = 0; c < 5; ++c) {
            float v[16];
            tc::ld16(lane_t + kColDW3 + 16 * c, v);
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                const int k = 16 * c + e;
                if (k < 64) atomicAdd(g + P_W3 + j * 64 + k, v[e]);
                else if (k == 64) atomicAdd(g + P_B3 + j, v[e]);
            }
            tc::ld16(lane_t + kColDW2 + 16 * c, v);
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                const int k = 16 * c + e;
                if (k < 64) atomicAdd(g + P_W2 + j * 64 + k, v[e]);
                else if (k == 64) atomicAdd(g + P_B2 + j, v[e]);
            }
        }
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            float v[16];
            tc::ld16(lane_t + kColDW1 + 16 * c, v);
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                const int k = 16 * c + e;
                if (k < kMlpIn) atomicAdd(g + P_W1 + j * 16 + k, v[e]);
                else if (k == 16) atomicAdd(g + P_B1 + j, v[e]);
            }
        }
    }
    // b4 and the loss: warp sums, then the block's (w4's are in red already)
    {
        float v = gb4;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp * 65 + 64] = v;
        for (int o = 16; o > 0; o >>= 1) sse += __shfl_xor_sync(0xffffffffu, sse, o);
        if (lane == 0 && sse != 0.0) atomicAdd(a.loss, sse);
    }
    tc::fence_before();
    __syncthreads();
    if (tid < 65) {
        const float v = red[tid] + red[65 + tid] + red[130 + tid] + red[195 + tid];
        if (v != 0.f) atomicAdd(a.grad + (tid < 64 ? P_W4 + tid : P_B4), v);
    }
    if (warp == 0) {
        tc::fence_after();
        tc::tmem_dealloc(t.tmem, 512);
    }
    if (!ok && tid == 0) atomicOr(a.err, 1u);
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

// Network outputs for contiguous samples of one class (tests, calibration, audits): y
// and dy/dx' in normalised units, 128 samples per tile on the tensor cores.
constexpr uint32_t kPrW = 0, kPrX = tc::kImgBytes, kPrP = kPrX + kTcX, kPrQ = kPrP + kTcAct,
                   kPrBytes = kPrQ + kTcAct + 32768;

__global__ void __launch_bounds__(128) k_mlp_predict(const MlpDev* M, int cls, const float* feats, int n, float* y,
                                                     float* dydx, uint32_t* err)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5;
    const MlpVec& V = M->vec[cls];
    tc_load_weights(sm + kPrW, M->tcw[cls]);
    if (warp == 0) tc::tmem_alloc(tc::smem_addr(&tmem_base), 256);
    if (tid == 0) tc::mbar_init(tc::smem_addr(&mbar), 1);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    TcTile t;
    t.w = sm + kPrW;
    t.x = sm + kPrX;
    t.p = sm + kPrP;
    t.q = sm + kPrQ;
    t.mbar = tc::smem_addr(&mbar);
    t.tmem = tmem_base;
    t.bar_id = 1;
    uint32_t phase = 0;
    bool ok = true;
    for (int base = blockIdx.x * kTcRows; base < n && ok; base += gridDim.x * kTcRows) {
        const int s = base + tid;
        float x[kMlpIn];
#pragma unroll
        for (int f = 0; f < kMlpIn; ++f) x[f] = s < n ? (feats[(size_t)s * 8 + f] - V.mu[f]) * V.inv_sd[f] : 0.f;
        float yy, d[kMlpIn];
        ok &= tc_rows128(t, phase, V, x, yy, d);
        if (s < n) {
            y[s] = yy;
#pragma unroll
            for (int f = 0; f < kMlpIn; ++f) dydx[(size_t)s * kMlpIn + f] = d[f];
        }
        ok = __syncthreads_and(ok) != 0;
        tc::fence_after();
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        tc::tmem_dealloc(t.tmem, 256);
    }
    if (!ok && tid == 0) atomicOr(err, 1u);
}

}  // namespace

struct oxg_mlp {
    MlpDev* dev = nullptr;
    uint32_t* err = nullptr;  // set by a tensor-core kernel whose MMA wait gave up
    float* P = nullptr;   // masters, kMlpClasses * kMlpParams
    float* G = nullptr;   // gradients
    float* m1 = nullptr;  // Adam moments
    float* m2 = nullptr;
    double* loss = nullptr;
    int adam_t[kMlpClasses] = {0, 0};
    MlpVec vec_host[kMlpClasses];
};

namespace {

// A tensor-core kernel reports an MMA wait that gave up through m->err (read after a
// synchronisation, then cleared).
int mlp_check_err(oxg_mlp* m)
{
    uint32_t e = 0;
    MCUDA(cudaMemcpy(&e, m->err, sizeof(e), cudaMemcpyDeviceToHost));
    if (e) {
        MCUDA(cudaMemset(m->err, 0, sizeof(e)));
        return internal_set_error(OXG_ERR_TIMEOUT, "a tensor-core MMA of the surrogate did not complete");
    }
    return OXG_OK;
}

int mlp_repack(oxg_mlp* m, cudaStream_t st)
{
    const int nt = kMlpClasses * kPackPerClass;
    k_mlp_pack_tc<<<(nt + 255) / 256, 256, 0, st>>>(m->P, m->dev);
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
        cudaMalloc(&m->m2, np * 4) != cudaSuccess || cudaMalloc(&m->loss, sizeof(double)) != cudaSuccess ||
        cudaMalloc(&m->err, sizeof(uint32_t)) != cudaSuccess) {
        oxg_mlp_destroy(m);
        return internal_set_error(OXG_ERR_CUDA, "cudaMalloc failed");
    }
    cudaMemset(m->dev, 0, sizeof(MlpDev));
    cudaMemset(m->err, 0, sizeof(uint32_t));
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
    cudaFree(m->err);
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
    a.err = m->err;
    MCUDA(cudaMemsetAsync(m->loss, 0, sizeof(double), st));
    const int smem = (int)kTrBytes;
    MCUDA(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    const int tiles = (nb + kTcRows - 1) / kTcRows;
    const int blocks = std::max(1, std::min(tiles, internal_num_sms()));
    k_mlp_train<<<blocks, 128, smem, st>>>(a);
    MCUDA(cudaGetLastError());
    if (grad_host) {
        MCUDA(cudaMemcpyAsync(grad_host, a.grad, kMlpParams * 4, cudaMemcpyDeviceToHost, st));
        MCUDA(cudaMemsetAsync(a.grad, 0, kMlpParams * 4, st));
    }
    if (loss_host) MCUDA(cudaMemcpyAsync(loss_host, m->loss, sizeof(double), cudaMemcpyDeviceToHost, st));
    if (grad_host || loss_host) {
        MCUDA(cudaStreamSynchronize(st));
        return mlp_check_err(m);
    }
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
    const int smem = (int)kPrBytes;
    MCUDA(cudaFuncSetAttribute(k_mlp_predict, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    const int tiles = (n + kTcRows - 1) / kTcRows;
    const int blocks = std::min(tiles, 2 * internal_num_sms());
    k_mlp_predict<<<blocks, 128, smem, st>>>(m->dev, cls, feats, n, y, dydx, m->err);
    MCUDA(cudaGetLastError());
    MCUDA(cudaStreamSynchronize(st));
    return mlp_check_err(m);
}

}  // extern "C"
