// oxg_mlp.cuh - the learned surrogate of the fused hydrogen-bonding + cross-stacking
// pair term: a 7 -> 64 -> 64 -> 64 -> 1 SiLU MLP on BF16 tensor cores (FP32 accumulate).
//
// Inputs (the base-base geometry the plain evaluator computes, bb_geometry): the BASE-BASE
// distance and the cosines c1, c2, c3, c4, c7, c8; output: the pair energy. There is one
// network per pair class (complementary bases, which hydrogen-bond, and the rest, which
// only cross-stack). Forces and torques come from the analytic input gradient of the
// network (its backward pass), mapped onto positions and orientations.
//
// The warp is the unit of work: 16 pairs are the 16 rows of mma.m16n8k16 tiles, and the
// activations never leave registers. The C fragment of two neighbouring n-tiles of one
// layer, packed to BF16, is exactly the A fragment of one k-tile of the next layer, so
// the forward pass (3 GEMMs) and the input-gradient pass (3 more) chain in registers;
// the weights are pre-arranged on the device in per-lane fragment order (one 64-bit
// load per lane per tile).
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "oxg_device.cuh"

namespace oxg {

constexpr int kMlpIn = 7;      // r, c1, c2, c3, c4, c7, c8
constexpr int kMlpHid = 64;
constexpr int kMlpClasses = 2; // 0: non-complementary (cross-stacking only), 1: complementary
// fragment tiles per class: forward W1 (K16 x N64: 8), W2, W3 (K64 x N64: 32 each),
// backward W3^T, W2^T (32 each), W1^T (K64 x N16: 8)
constexpr int kFragF1 = 0, kFragF2 = 8, kFragF3 = 40, kFragG3 = 72, kFragG2 = 104, kFragG1 = 136;
constexpr int kFragTiles = 144;

// FP32 vectors of one class
struct MlpVec {
    float b1[kMlpHid], b2[kMlpHid], b3[kMlpHid], w4[kMlpHid];
    float b4;
    float mu[kMlpIn], inv_sd[kMlpIn];  // input normalisation x' = (x - mu) * inv_sd
    float e_scale, e_shift;            // E = e_scale * y + e_shift
    float pad[11];
};

// Device image of the surrogate (both classes): the mma fragments of the in-kernel
// warp pass, the vectors, and the tcgen05 weight images (B operands of the six GEMMs
// in the canonical K-major layout, oxg_tc.cuh).
struct MlpDev {
    uint2 frag[kMlpClasses][kFragTiles][32];  // BF16x2 pairs (b0, b1) per lane
    MlpVec vec[kMlpClasses];
    alignas(16) unsigned char tcw[kMlpClasses][36864];
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// D = A(16x16, bf16, row) * B(16x8, bf16, col) + C (fp32)
__device__ __forceinline__ void mma_bf16(float* d, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint2 b)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b.x), "r"(b.y));
}

__device__ __forceinline__ float sigmoidf_fast(float z) { return 1.f / (1.f + __expf(-z)); }

// One dense layer of 64 outputs over K = 16 * KT inputs given as A fragments:
// out[nt][0..3] (C fragments of n-tile nt) = sum_kt A[kt] * B[kt][nt].
template <int KT>
__device__ __forceinline__ void mlp_layer(const uint2* frag, const uint32_t (*A)[4], float (*out)[4],
                                          int lane)
{
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) out[nt][0] = out[nt][1] = out[nt][2] = out[nt][3] = 0.f;
#pragma unroll
    for (int kt = 0; kt < KT; ++kt)
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
            mma_bf16(out[nt], A[kt][0], A[kt][1], A[kt][2], A[kt][3], frag[(kt * 8 + nt) * 32 + lane]);
}

// A fragments of the next layer from the 64-column C fragments of this one.
__device__ __forceinline__ void c_to_a(const float (*c)[4], uint32_t (*A)[4])
{
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
        A[kt][0] = pack_bf16(c[2 * kt][0], c[2 * kt][1]);
        A[kt][1] = pack_bf16(c[2 * kt][2], c[2 * kt][3]);
        A[kt][2] = pack_bf16(c[2 * kt + 1][0], c[2 * kt + 1][1]);
        A[kt][3] = pack_bf16(c[2 * kt + 1][2], c[2 * kt + 1][3]);
    }
}

// Column of C-fragment element e of n-tile nt for this lane (rows: g for e < 2, g + 8 else).
__device__ __forceinline__ int frag_col(int nt, int e, int lane) { return nt * 8 + 2 * (lane & 3) + (e & 1); }

// z <- z + b; h = silu(z) (in place into z); s = silu'(z).
__device__ __forceinline__ void bias_silu(float (*z)[4], float (*s)[4], const float* b, int lane)
{
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float x = z[nt][e] + b[frag_col(nt, e, lane)];
            const float sg = sigmoidf_fast(x);
            z[nt][e] = x * sg;
            s[nt][e] = sg * (1.f + x * (1.f - sg));
        }
}

// silu'(z) of a layer kept as BF16 pairs (in the C-fragment order) for the backward pass.
__device__ __forceinline__ void pack_frags(const float (*c)[4], uint32_t (*p)[2])
{
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        p[nt][0] = pack_bf16(c[nt][0], c[nt][1]);
        p[nt][1] = pack_bf16(c[nt][2], c[nt][3]);
    }
}
__device__ __forceinline__ void mul_packed(float (*c)[4], const uint32_t (*p)[2])
{
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float2 lo = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&p[nt][0]));
        const float2 hi = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&p[nt][1]));
        c[nt][0] *= lo.x;
        c[nt][1] *= lo.y;
        c[nt][2] *= hi.x;
        c[nt][3] *= hi.y;
    }
}

// Energy and input gradient of 16 pairs (rows) of one class for a warp. x[f] holds the
// normalised features of row (lane & 15) in lanes 0..15 (any values in lanes 16..31).
// Returns, in lanes 0..15 for row (lane & 15): y (network output) and dy/dx'[0..6].
// The SiLU derivatives of the first two layers are kept as BF16 (they multiply values
// that are rounded to BF16 as the next MMA operand anyway), which keeps the pass within
// the register budget of the force kernels.
__device__ __forceinline__ void mlp_rows16(const MlpDev& M, int cls, const float* x, float& y,
                                           float* dydx)
{
    const int lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    const uint2* F = &M.frag[cls][0][0];
    const MlpVec& V = M.vec[cls];
    // A fragment of the inputs: rows g, g + 8; columns 2t, 2t + 1 (columns >= 7 are 0)
    float xg[kMlpIn], xg8[kMlpIn];
#pragma unroll
    for (int f = 0; f < kMlpIn; ++f) {
        xg[f] = __shfl_sync(0xffffffffu, x[f], g);
        xg8[f] = __shfl_sync(0xffffffffu, x[f], g + 8);
    }
    auto pick = [&](const float* v, int f) {
        float r = 0.f;
#pragma unroll
        for (int k = 0; k < kMlpIn; ++k) r = (k == f) ? v[k] : r;
        return r;
    };
    uint32_t A0[1][4];
    A0[0][0] = pack_bf16(pick(xg, 2 * t), pick(xg, 2 * t + 1));
    A0[0][1] = pack_bf16(pick(xg8, 2 * t), pick(xg8, 2 * t + 1));
    A0[0][2] = 0u;
    A0[0][3] = 0u;
    float z[8][4], s[8][4];
    uint32_t sp1[8][2], sp2[8][2];
    uint32_t A[4][4];
    mlp_layer<1>(F + kFragF1 * 32, A0, z, lane);
    bias_silu(z, s, V.b1, lane);
    pack_frags(s, sp1);
    c_to_a(z, A);
    mlp_layer<4>(F + kFragF2 * 32, A, z, lane);
    bias_silu(z, s, V.b2, lane);
    pack_frags(s, sp2);
    c_to_a(z, A);
    mlp_layer<4>(F + kFragF3 * 32, A, z, lane);
    bias_silu(z, s, V.b3, lane);
    // output: y[row] = h3[row] . w4 + b4 (rows g and g + 8; reduce over the 4 lanes of a
    // group); dy/dz3 = w4 * silu'(z3)
    float yg = 0.f, yg8 = 0.f;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float w0 = V.w4[frag_col(nt, 0, lane)], w1 = V.w4[frag_col(nt, 1, lane)];
        yg += z[nt][0] * w0 + z[nt][1] * w1;
        yg8 += z[nt][2] * w0 + z[nt][3] * w1;
        s[nt][0] *= w0;
        s[nt][1] *= w1;
        s[nt][2] *= w0;
        s[nt][3] *= w1;
    }
    yg += __shfl_xor_sync(0xffffffffu, yg, 1);
    yg += __shfl_xor_sync(0xffffffffu, yg, 2);
    yg8 += __shfl_xor_sync(0xffffffffu, yg8, 1);
    yg8 += __shfl_xor_sync(0xffffffffu, yg8, 2);
    // back through W3, W2 and W1
    c_to_a(s, A);
    mlp_layer<4>(F + kFragG3 * 32, A, z, lane);  // dy/dh2
    mul_packed(z, sp2);                          // dy/dz2
    c_to_a(z, A);
    mlp_layer<4>(F + kFragG2 * 32, A, z, lane);  // dy/dh1
    mul_packed(z, sp1);                          // dy/dz1
    c_to_a(z, A);
    // dy/dx' = dz1 * W1 (N = 16: two n-tiles; only n-tile 0, columns 0..6, are inputs)
    float dx[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) mma_bf16(dx, A[kt][0], A[kt][1], A[kt][2], A[kt][3], F[(kFragG1 + kt * 2) * 32 + lane]);
    // gather to the lane owning the row: row r lives in lanes (r & 7) * 4 + t, elements
    // (0, 1) for r < 8 and (2, 3) for r >= 8; columns 2t, 2t + 1
    const int r = lane & 15, src0 = (r & 7) * 4;
    const float ya = __shfl_sync(0xffffffffu, yg, src0), yb = __shfl_sync(0xffffffffu, yg8, src0);
    y = (r < 8 ? ya : yb) + V.b4;
#pragma unroll
    for (int tt = 0; tt < 4; ++tt) {
        const float v0 = __shfl_sync(0xffffffffu, dx[0], src0 + tt), v1 = __shfl_sync(0xffffffffu, dx[1], src0 + tt);
        const float v2 = __shfl_sync(0xffffffffu, dx[2], src0 + tt), v3 = __shfl_sync(0xffffffffu, dx[3], src0 + tt);
        if (2 * tt < kMlpIn) dydx[2 * tt] = r < 8 ? v0 : v2;
        if (2 * tt + 1 < kMlpIn) dydx[2 * tt + 1] = r < 8 ? v1 : v3;
    }
}

// Features of a base-base geometry: r, c1, c2, c3, c4, c7, c8.
OXG_HD void mlp_features(const BBGeom& g, float* x)
{
    x[0] = g.rmod;
    x[1] = g.c1;
    x[2] = g.c2;
    x[3] = g.c3;
    x[4] = g.c4;
    x[5] = g.c7;
    x[6] = g.c8;
}

// Forces and torques of an energy E(r, c1, c2, c3, c4, c7, c8) of the base-base geometry
// g (cosines as in bb_geometry) with gradient dE = dE/d(features): the force on j is
// -dE/dr_vec (r_vec = r_j + base_j - r_i - base_i); a rotation of particle i moves its
// axes and its base site, hence tau_i = -sum_a a x dE/da + base_i x dE/dr_vec and
// tau_j = -sum_b b x dE/db - base_j x dE/dr_vec.
OXG_HD void mlp_grad_to_forces(const BBGeom& g, const Frame& fi, const Frame& fj, const float* dE,
                               PairAcc& acc)
{
    const float3 d = g.rdir;
    const float inv = 1.f / g.rmod;
    const float3 a1 = fi.a1, a3 = fi.a3, b1 = fj.a1, b3 = fj.a3;
    // d(u . d)/dr_vec = (u - d (u . d)) / r
    float3 dEdr = d * dE[0];
    dEdr += (b1 - d * dot(b1, d)) * (-dE[2] * inv);  // c2 = -b1 . d
    dEdr += (a1 - d * dot(a1, d)) * (dE[3] * inv);   // c3 = a1 . d
    dEdr += (b3 - d * dot(b3, d)) * (-dE[5] * inv);  // c7 = -b3 . d
    dEdr += (a3 - d * dot(a3, d)) * (dE[6] * inv);   // c8 = a3 . d
    const float3 dEa1 = b1 * (-dE[1]) + d * dE[3];   // c1 = -a1 . b1
    const float3 dEa3 = b3 * dE[4] + d * dE[6];      // c4 = a3 . b3
    const float3 dEb1 = a1 * (-dE[1]) + d * (-dE[2]);
    const float3 dEb3 = a3 * dE[4] + d * (-dE[5]);
    acc.fi += dEdr;  // F_i = +dE/dr_vec
    acc.ti += cross(g.base_i, dEdr) - cross(a1, dEa1) - cross(a3, dEa3);
    acc.tj += -cross(g.base_j, dEdr) - cross(b1, dEb1) - cross(b3, dEb3);
}

}  // namespace oxg
