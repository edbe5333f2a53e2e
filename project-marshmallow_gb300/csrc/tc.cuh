// tc.cuh - Blackwell 5th-generation tensor core (tcgen05) building blocks in inline PTX.
//
// Operands live in shared memory in the no-swizzle K-major layout: the matrix is cut into "core
// matrices" of 8 rows x 16 bytes (8 x 8 bf16), each stored as 128 contiguous bytes (row-major inside).
// For an R x K bf16 operand the core matrix (row group g, K chunk c) starts at
//     g * kSbo + c * kLbo,   kLbo = 128 bytes (K-adjacent chunks contiguous),
//                            kSbo = (K / 8) * 128 bytes (next group of 8 rows),
// and one MMA of K = 16 reads two K chunks, so the k-th MMA of a K loop starts 256 * k bytes in.
// The accumulator lives in tensor memory (TMEM): for M = 128 (cta_group::1) row i is TMEM lane i and
// column j is TMEM column base + j, 32-bit FP32.  Warp w of the CTA reads lanes 32w .. 32w + 31.
//
// Every wait on an mbarrier is bounded: after kSpinLimit polls the caller sets an error flag and
// stops waiting, so a fault in the protocol ends the kernel instead of hanging the GPU.
#ifndef MM_TC_CUH_
#define MM_TC_CUH_

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace mm {
namespace tc {

constexpr uint32_t kSpinLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Byte offset of element (r, k) of an R x K bf16 operand in the layout above.
__device__ __forceinline__ uint32_t kmajor_offset(int r, int k, int K) {
    return (uint32_t)((r >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor (tcgen05): start address, leading/stride byte offsets (>> 4),
// descriptor version 1 at bits 46-47, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor, kind::f16: D FP32, A and B BF16, both K-major, shape M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// The same with A and/or B read MN-major (bits 15 and 16): the operand's M (or N) index runs
// along the 16-byte rows of its core matrices and K across the 8 rows.  A tile stored in the
// K-major layout above as [K][MN] (kmajor_offset(k, mn, MN)) is such an operand, with core-matrix
// strides 128 bytes along MN and (MN / 8) * 128 bytes along K, so the transpose of a stored
// activation tile is read in place.
__host__ __device__ constexpr uint32_t idesc_bf16_mn(int M, int N, bool a_mn, bool b_mn) {
    return idesc_bf16(M, N) | (a_mn ? (1u << 15) : 0u) | (b_mn ? (1u << 16) : 0u);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Waits for the phase with parity `parity` to complete; returns false if it gave up after `limit`
// polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit = kSpinLimit) {
    const uint32_t a = smem_u32(bar);
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// One arrival on `bar` (count 1 completes the current phase).
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}" ::"r"(smem_u32(bar)) : "memory");
}

// Generic-proxy shared-memory writes become visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// TMEM allocation by one whole warp; the TMEM address is written to *slot.
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, one instruction (K = 16 for bf16).  One thread issues.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrives on `bar` once every MMA this thread issued before has completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 16 consecutive FP32 columns of the calling thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Issues D = A * B^T over K (K/16 instructions) from one thread.
// A: M = 128 rows x K at sa, B: N rows x K at sb, both in the K-major layout above.
__device__ __forceinline__ void gemm_mmas(uint32_t d_tmem, uint32_t sa, uint32_t sb, int K, int N) {
    const uint32_t sbo = (uint32_t)(K / 8) * 128;
    const uint32_t idesc = idesc_bf16(128, N);
    for (int kk = 0; kk < K / 16; ++kk)
        mma_bf16(d_tmem, smem_desc(sa + kk * 256, 128, sbo), smem_desc(sb + kk * 256, 128, sbo), idesc, kk > 0 ? 1u : 0u);
}

// As gemm_mmas, but the first MMA adds to D when `accumulate` is 1 (D += A * B^T): a sum over
// several launches of the same GEMM shape stays in tensor memory.
__device__ __forceinline__ void gemm_mmas_acc(uint32_t d_tmem, uint32_t sa, uint32_t sb, int K, int N,
                                              uint32_t accumulate) {
    const uint32_t sbo = (uint32_t)(K / 8) * 128;
    const uint32_t idesc = idesc_bf16(128, N);
    for (int kk = 0; kk < K / 16; ++kk)
        mma_bf16(d_tmem, smem_desc(sa + kk * 256, 128, sbo), smem_desc(sb + kk * 256, 128, sbo), idesc,
                 kk > 0 ? 1u : accumulate);
}

// gemm_mmas followed by a commit to `bar`.
__device__ __forceinline__ void gemm_issue(uint32_t d_tmem, uint32_t sa, uint32_t sb, int K, int N, uint64_t* bar) {
    gemm_mmas(d_tmem, sa, sb, K, N);
    mma_commit(bar);
}

// Packs 8 floats into 8 bf16 (one 16-byte core-matrix row).
__device__ __forceinline__ uint4 pack8_bf16(const float* v) {
    uint4 u;
    __nv_bfloat162 a = __floats2bfloat162_rn(v[0], v[1]), b = __floats2bfloat162_rn(v[2], v[3]);
    __nv_bfloat162 c = __floats2bfloat162_rn(v[4], v[5]), d = __floats2bfloat162_rn(v[6], v[7]);
    u.x = *reinterpret_cast<uint32_t*>(&a);
    u.y = *reinterpret_cast<uint32_t*>(&b);
    u.z = *reinterpret_cast<uint32_t*>(&c);
    u.w = *reinterpret_cast<uint32_t*>(&d);
    return u;
}

}  // namespace tc
}  // namespace mm

#endif  // MM_TC_CUH_
