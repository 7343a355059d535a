// oxg_mlp.cuh - the learned surrogate of the fused hydrogen-bonding + cross-stacking
// pair term: a 7 -> 64 -> 64 -> 64 -> 1 SiLU MLP on the fifth-generation tensor cores
// (tcgen05: BF16 operands, FP32 accumulation in tensor memory).
//
// Inputs (the base-base geometry the plain evaluator computes, bb_geometry): the BASE-BASE
// distance and the cosines c1, c2, c3, c4, c7, c8; output: the pair energy. There is one
// network per pair class (complementary bases, which hydrogen-bond, and the rest, which
// only cross-stack). Forces and torques come from the analytic input gradient of the
// network (its backward pass), mapped onto positions and orientations.
//
// The tile is the unit of work: a warpgroup (128 threads) runs 128 rows (pairs or
// training samples), a row per thread. Every GEMM has M = 128 rows: the layer's input
// rows are written as BF16 into shared memory in the canonical K-major layout, one
// thread issues the MMAs (weights in shared memory as the B operand), the FP32
// accumulator lands in tensor memory and comes back a row per thread for the bias /
// SiLU epilogue, which writes the next layer's operand. The SiLU derivatives of the
// forward pass are written back into tensor memory over the pre-activations, so the
// backward (input-gradient) GEMMs need no recomputation.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "oxg_device.cuh"
#include "oxg_tc.cuh"

namespace oxg {

constexpr int kMlpIn = 7;      // r, c1, c2, c3, c4, c7, c8
constexpr int kMlpHid = 64;
constexpr int kMlpClasses = 2; // 0: non-complementary (cross-stacking only), 1: complementary

// FP32 vectors of one class
struct MlpVec {
    float b1[kMlpHid], b2[kMlpHid], b3[kMlpHid], w4[kMlpHid];
    float b4;
    float mu[kMlpIn], inv_sd[kMlpIn];  // input normalisation x' = (x - mu) * inv_sd
    float e_scale, e_shift;            // E = e_scale * y + e_shift
    float pad[11];
};

// Device image of the surrogate (both classes): the FP32 vectors and the BF16 weight
// images (the B operands of the six GEMMs in the canonical K-major layout, oxg_tc.cuh).
struct MlpDev {
    MlpVec vec[kMlpClasses];
    alignas(16) unsigned char tcw[kMlpClasses][tc::kImgBytes];
};

// ---------------------------------------------------------------- a 128-row tile
constexpr int kTcRows = 128;
constexpr uint32_t kTcX = 4096, kTcAct = 16384;  // A buffers: 128 x 16 and 128 x 64 BF16

struct TcTile {
    unsigned char* w;  // weight image of the class (tc::kImgBytes)
    unsigned char* x;  // 128 x 16 inputs
    unsigned char* p;  // 128 x 64 activations / gradients (two buffers)
    unsigned char* q;
    uint32_t mbar;     // shared address of the MMA-completion mbarrier
    uint32_t tmem;     // tensor-memory base of the tile's 256 columns: D1 [0, 64), D2 [64,
                       // 128), D3 [128, 192), D4 [192, 256); the input gradient in [0, 16)
    int bar_id;        // named barrier of the warpgroup
};

__device__ __forceinline__ void wg_sync(int id) { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }

__device__ __forceinline__ void st_bf16(unsigned char* base, uint32_t off, float v)
{
    *reinterpret_cast<__nv_bfloat16*>(base + off) = __float2bfloat16_rn(v);
}

// Shared-memory writes of this warpgroup become operands of the MMAs issued next: make
// them visible to the tensor cores, order earlier tensor-memory accesses, and meet.
__device__ __forceinline__ void tc_publish(const TcTile& t)
{
    tc::fence_smem_async();
    tc::fence_before();
    wg_sync(t.bar_id);
}

// One thread issues `steps` K = 16 MMAs D(col) = A * B (+ D) and commits them; every
// thread then waits for their completion. Returns false if the wait gave up.
__device__ __forceinline__ bool tc_gemm(const TcTile& t, uint32_t& phase, uint32_t dcol, const unsigned char* A,
                                        int a_rows, const unsigned char* B, int b_rows, int n, int steps,
                                        bool first_acc)
{
    if ((threadIdx.x & 127) == 0) {
        tc::fence_after();
        const uint32_t sa = tc::smem_addr(A), sb = tc::smem_addr(B), id = tc::idesc_bf16(128, n);
        for (int j = 0; j < steps; ++j)
            tc::mma(t.tmem + dcol, tc::op_desc(sa, a_rows, j), tc::op_desc(sb, b_rows, j), id,
                    (first_acc || j > 0) ? 1u : 0u);
        tc::commit(t.mbar);
    }
    const bool ok = tc::mbar_wait(t.mbar, phase);
    phase ^= 1u;
    tc::fence_after();
    return ok;
}

// As tc_gemm with the weights held as hi + lo images: `steps` MMAs with B_hi, then
// `steps` with B_lo into the same accumulator, one commit and one wait.
__device__ __forceinline__ bool tc_gemm_split(const TcTile& t, uint32_t& phase, uint32_t dcol, const unsigned char* A,
                                              int a_rows, const unsigned char* Bhi, const unsigned char* Blo,
                                              int b_rows, int n, int steps)
{
    if ((threadIdx.x & 127) == 0) {
        tc::fence_after();
        const uint32_t sa = tc::smem_addr(A), sh = tc::smem_addr(Bhi), sl = tc::smem_addr(Blo);
        const uint32_t id = tc::idesc_bf16(128, n);
        for (int j = 0; j < steps; ++j)
            tc::mma(t.tmem + dcol, tc::op_desc(sa, a_rows, j), tc::op_desc(sh, b_rows, j), id, j > 0 ? 1u : 0u);
        for (int j = 0; j < steps; ++j)
            tc::mma(t.tmem + dcol, tc::op_desc(sa, a_rows, j), tc::op_desc(sl, b_rows, j), id, 1u);
        tc::commit(t.mbar);
    }
    const bool ok = tc::mbar_wait(t.mbar, phase);
    phase ^= 1u;
    tc::fence_after();
    return ok;
}

// The layer-1 operand row of normalised inputs x: bf16(x) in columns 0..6 and the
// remainders x - bf16(x) in columns 7..13 (rounded to BF16 when stored), zeros after.
__device__ __forceinline__ void split_inputs(const float* x, float* xr)
{
#pragma unroll
    for (int f = 0; f < 16; ++f) xr[f] = 0.f;
#pragma unroll
    for (int f = 0; f < kMlpIn; ++f) {
        const float hi = __bfloat162float(__float2bfloat16_rn(x[f]));
        xr[f] = hi;
        xr[kMlpIn + f] = x[f] - hi;
    }
}

// Forward epilogue of this thread's row: z = D (64 columns from col) + b; silu(z) as the
// row of the next A operand (dst, if set) and as this row's column of a transposed
// operand with tr_rows rows (dstT, if set); silu'(z) written back over z.
__device__ __forceinline__ void tc_forward_row(uint32_t lane_t, uint32_t col, const float* b, unsigned char* dst,
                                               int row, unsigned char* dstT = nullptr, int tr_rows = 80)
{
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        float z[16], h[16];
        tc::ld16(lane_t + col + 16 * c, z);
#pragma unroll
        for (int e = 0; e < 16; ++e) {
            z[e] = tc::silu_and_grad(z[e] + b[16 * c + e], h[e]);
            if (dstT) st_bf16(dstT, tc::kmaj_off(tr_rows, 16 * c + e, row), h[e]);
        }
        tc::st16(lane_t + col + 16 * c, z);
        if (dst) {
            tc::st_row8(dst, tc::kmaj_off(128, row, 16 * c), h);
            tc::st_row8(dst, tc::kmaj_off(128, row, 16 * c + 8), h + 8);
        }
    }
}

// Backward epilogue of this thread's row: dz = g * silu'(z), g from D4 and silu'(z) from
// the forward columns scol; written as the row of an A operand (dst, if set) and as this
// row's column of a transposed operand of 128 rows (dstT, if set).
__device__ __forceinline__ void tc_backward_row(uint32_t lane_t, uint32_t scol, unsigned char* dst, int row,
                                                unsigned char* dstT = nullptr)
{
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        float g[16], sp[16], dz[16];
        tc::ld16(lane_t + 192 + 16 * c, g);
        tc::ld16(lane_t + scol + 16 * c, sp);
#pragma unroll
        for (int e = 0; e < 16; ++e) {
            dz[e] = g[e] * sp[e];
            if (dstT) st_bf16(dstT, tc::kmaj_off(128, 16 * c + e, row), dz[e]);
        }
        if (dst) {
            tc::st_row8(dst, tc::kmaj_off(128, row, 16 * c), dz);
            tc::st_row8(dst, tc::kmaj_off(128, row, 16 * c + 8), dz + 8);
        }
    }
}

// Energy and input gradient of 128 rows: x (this thread's row, 7 normalised features;
// zeros for an unused row) -> y and dy/dx'. All 128 threads of the warpgroup call it.
// Returns false if an MMA wait gave up.
__device__ __forceinline__ bool tc_rows128(const TcTile& t, uint32_t& phase, const MlpVec& V, const float* x,
                                           float& y, float* dydx)
{
    const int row = threadIdx.x & 127;
    const uint32_t lane_t = t.tmem + ((uint32_t)(((threadIdx.x >> 5) & 3) * 32) << 16);
    bool ok = true;
    {
        float xr[16];
        split_inputs(x, xr);
        tc::st_row8(t.x, tc::kmaj_off(128, row, 0), xr);
        tc::st_row8(t.x, tc::kmaj_off(128, row, 8), xr + 8);
    }
    tc_publish(t);
    ok &= tc_gemm_split(t, phase, 0, t.x, 128, t.w + tc::kImgF1, t.w + tc::kImgF1L, 64, 64, 1);    // D1 = X W1
    tc_forward_row(lane_t, 0, V.b1, t.p, row);
    tc_publish(t);
    ok &= tc_gemm_split(t, phase, 64, t.p, 128, t.w + tc::kImgF2, t.w + tc::kImgF2L, 64, 64, 4);   // D2 = H1 W2
    tc_forward_row(lane_t, 64, V.b2, t.q, row);
    tc_publish(t);
    ok &= tc_gemm_split(t, phase, 128, t.q, 128, t.w + tc::kImgF3, t.w + tc::kImgF3L, 64, 64, 4);  // D3 = H2 W3
    // output and dy/dz3 = w4 * silu'(z3)
    float yy = V.b4;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        float z[16], dz[16];
        tc::ld16(lane_t + 128 + 16 * c, z);
#pragma unroll
        for (int e = 0; e < 16; ++e) {
            float h;
            const float sp = tc::silu_and_grad(z[e] + V.b3[16 * c + e], h);
            yy += h * V.w4[16 * c + e];
            dz[e] = sp * V.w4[16 * c + e];
        }
        tc::st_row8(t.p, tc::kmaj_off(128, row, 16 * c), dz);
        tc::st_row8(t.p, tc::kmaj_off(128, row, 16 * c + 8), dz + 8);
    }
    y = yy;
    tc_publish(t);
    ok &= tc_gemm_split(t, phase, 192, t.p, 128, t.w + tc::kImgG3, t.w + tc::kImgG3L, 64, 64, 4);  // dH2 = dZ3 W3^T
    tc_backward_row(lane_t, 64, t.q, row);                                                       // dZ2
    tc_publish(t);
    ok &= tc_gemm_split(t, phase, 192, t.q, 128, t.w + tc::kImgG2, t.w + tc::kImgG2L, 64, 64, 4);  // dH1 = dZ2 W2^T
    tc_backward_row(lane_t, 0, t.p, row);                                                        // dZ1
    tc_publish(t);
    ok &= tc_gemm(t, phase, 0, t.p, 128, t.w + tc::kImgG1, 16, 16, 4, false);  // dZ1 [W1_hi | W1_lo]^T
    float dx[16];
    tc::ld16(lane_t, dx);
#pragma unroll
    for (int f = 0; f < kMlpIn; ++f) dydx[f] = dx[f] + dx[kMlpIn + f];
    tc::fence_before();  // the next tile's MMAs overwrite these columns after a barrier
    return ok;
}

// The class's weight image into shared memory (every thread of the block, 16-byte
// loads), made visible to the tensor cores.
__device__ __forceinline__ void tc_load_weights(unsigned char* dst, const unsigned char* src)
{
    for (int k = threadIdx.x; k < (int)(tc::kImgBytes / 16); k += blockDim.x)
        reinterpret_cast<uint4*>(dst)[k] = reinterpret_cast<const uint4*>(src)[k];
    tc::fence_smem_async();
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
