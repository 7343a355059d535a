// oxg_tc.cuh - fifth-generation tensor cores (tcgen05) for the surrogate network: BF16
// operands in shared memory described by matrix descriptors, FP32 accumulators in tensor
// memory (TMEM), MMAs issued by one thread and tracked by an mbarrier, and row-per-thread
// read-back of the accumulators. sm_100a / sm_103a only.
//
// Operand layout: the canonical K-major layout without swizzling. A matrix of R rows
// (M or N) and K columns is stored as core matrices of 8 rows x 16 bytes (8 BF16 along
// K), each 128 contiguous bytes; core matrix (row group g, K chunk c) sits at
// c * (R / 8) * 128 + g * 128. In a descriptor the leading byte offset is the distance of
// K-adjacent core matrices ((R / 8) * 128) and the stride byte offset that of row-
// adjacent ones (128). One MMA consumes K = 16 (two K chunks).
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace oxg {
namespace tc {

// byte offset of element (r, k) of an R-row operand
__host__ __device__ constexpr uint32_t kmaj_off(int R, int r, int k)
{
    return (uint32_t)((k >> 3) * (R >> 3) * 128 + (r >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// Instruction descriptor of kind::f16 with BF16 A and B, FP32 D, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4)                        // D format: F32
           | (1u << 7)                      // A format: BF16
           | (1u << 10)                     // B format: BF16
           | ((uint32_t)(N >> 3) << 17)     // N / 8
           | ((uint32_t)(M >> 4) << 24);    // M / 16
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor (no swizzle): start address, leading (K) and stride
// (row) byte offsets, all in 16-byte units; bits 46-47 hold the descriptor version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// K step j (K = 16 each) of an R-row operand starting at saddr
__device__ __forceinline__ uint64_t op_desc(uint32_t saddr, int R, int j)
{
    const uint32_t lbo = (uint32_t)(R >> 3) * 128u;
    return sdesc(saddr + (uint32_t)j * 2u * lbo, lbo, 128u);
}

// Tensor-memory allocation; one full warp executes each of these.
__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t addr, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(addr), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t addr, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(addr), "r"(parity)
        : "memory");
    return ok != 0u;
}
// Wait for the mbarrier phase with this parity; gives up (false) after ~2^31 cycles.
__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity)
{
    const long long t0 = clock64();
    while (!mbar_try_wait(addr, parity))
        if (clock64() - t0 > (1LL << 31)) return false;
    return true;
}

// D (tmem) = A * B (+ D when acc != 0); one thread issues.
__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}
// The mbarrier receives one arrival when every MMA this thread issued before has completed.
__device__ __forceinline__ void commit(uint32_t mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes made visible to the tensor cores' (async proxy) reads
__device__ __forceinline__ void fence_smem_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane (warp w of a warpgroup reads
// lanes 32 (w % 4) .. + 31), waited for in the same statement.
__device__ __forceinline__ void ld16(uint32_t taddr, float* v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

// 16 consecutive FP32 columns of this thread's TMEM lane written from registers, waited
// for in the same statement.
__device__ __forceinline__ void st16(uint32_t taddr, const float* v)
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};\n\t"
        "tcgen05.wait::st.sync.aligned;" ::"r"(taddr),
        "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
        "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
        "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
        "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15]))
        : "memory");
}

// SiLU h = z sigmoid(z) and its derivative sigmoid(z) (1 + z (1 - sigmoid(z))), with the
// sigmoid as 1/2 + tanh(z / 2) / 2: one special-function instruction per value.
__device__ __forceinline__ float silu_and_grad(float z, float& h)
{
    float th;
    asm("tanh.approx.f32 %0, %1;" : "=f"(th) : "f"(0.5f * z));
    const float sg = fmaf(0.5f, th, 0.5f);
    h = z * sg;
    return sg * fmaf(z, 1.f - sg, 1.f);
}

__device__ __forceinline__ uint32_t pack2(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}
// 8 values as BF16 into one 16-byte core-matrix row
__device__ __forceinline__ void st_row8(unsigned char* base, uint32_t off, const float* v)
{
    *reinterpret_cast<uint4*>(base + off) =
        make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]), pack2(v[4], v[5]), pack2(v[6], v[7]));
}

// ---- weight image of one class (bytes), B operands of the GEMMs --------------------
// Every weight w is held as two BF16 numbers, hi = bf16(w) and lo = bf16(w - hi), and a
// GEMM with weights W runs as A W_hi + A W_lo into the same FP32 accumulator: the
// weights then carry ~16 significant bits instead of 8 (BF16 weights alone leave a
// pointwise energy error of a few 1e-4 of the pair energy, above the term's 1e-4 budget
// where many pairs share one geometry, as in built duplexes).
// forward:  F1 (N 64 outputs x K 16 inputs), F2, F3 (64 x 64): element (n, k) = W[n][k];
//           F1 also holds W1_hi in input columns 7..13, which multiply the low parts
//           x - bf16(x) of the 7 inputs (so the inputs carry ~16 bits too)
// backward: G3, G2 (N 64 inputs x K 64 outputs): element (n, k) = W[k][n];
//           G1 (N 16 inputs x K 64 outputs): W1_hi[k][n] in rows n < 7 and W1_lo[k][n - 7]
//           in rows 7..13 (the input gradient is the sum of the two row blocks)
// the lo images F1L (W1_lo in input columns 0..6), F2L, F3L, G3L, G2L follow the hi ones
constexpr uint32_t kImgF1 = 0, kImgF2 = 2048, kImgF3 = 10240, kImgG3 = 18432, kImgG2 = 26624,
                   kImgG1 = 34816, kImgF1L = 36864, kImgF2L = 38912, kImgF3L = 47104, kImgG3L = 55296,
                   kImgG2L = 63488, kImgBytes = 71680;

}  // namespace tc
}  // namespace oxg
