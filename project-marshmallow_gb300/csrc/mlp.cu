// mlp.cu - tcgen05 (5th-generation tensor core) kernels of the learned sun-cone surrogate.
//
// Network: 16 inputs -> 64 -> 64 -> 64 (ReLU) -> 1 (sigmoid).  Parameters are kept in FP32 (the
// Adam master copy) with BF16 copies of W1..W3 for the tensor cores.  Rounding points, which the
// CPU reference of the tests reproduces:
//   z1 = bf16(x) W1b^T + b1,  h1 = bf16(relu(z1))
//   z2 = h1 W2b^T + b2,       h2 = bf16(relu(z2))
//   z3 = h2 W3b^T + b3,       h3 = relu(z3)              (FP32)
//   y  = sigmoid(h3 . w4 + b4)                         (FP32, CUDA cores)
// GEMMs accumulate in FP32 in tensor memory.  One CTA of 4 warps handles 128 samples at a time,
// one sample per thread (= one TMEM lane) in the epilogues.
//
// Training (one kernel per step, then Adam): the backward pass keeps every GEMM on the tensor
// cores.  With dz = 2 (y - t) y (1 - y) / B:
//   dw4 = sum_r dz h3, db4 = sum_r dz                   (CUDA cores, warp reductions)
//   d3  = bf16(dz w4 * [z3 > 0])
//   dW3 = d3^T h2, db3 = d3^T 1                          (A = d3^T, B = [h2^T; 1])
//   d2  = bf16((d3 W3b) * [z2 > 0])                      (A = d3,   B = W3b^T)
//   dW2 = d2^T h1, db2 = d2^T 1; d1 = bf16((d2 W2b) * [z1 > 0]); dW1 = d1^T x, db1 = d1^T 1.
// Weight-gradient GEMMs reduce over the 128 samples (K = 128) with M padded from 64 to 128 rows;
// the ones row appended to B yields the bias gradient as one more output column.  Each layer's
// weight gradient accumulates in its own tensor-memory columns over all the tiles a CTA trains on,
// and the CTA adds it to a global FP32 buffer with atomics once, at its end.
//
// The file also holds the tensor-core GEMM self-check used to validate the operand layout and the
// MMA/TMEM protocol of tc.cuh on the device.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <new>

#include "mm_internal.h"
#include "tc.cuh"

namespace mm {
namespace mlp {

// D[128 x N] = A[128 x K] * B[N x K]^T in one CTA of 4 warps; `variant` swaps the two stride
// fields of the operand descriptors (layout self-check).
__global__ void __launch_bounds__(128) tc_gemm_kernel(const __nv_bfloat16* __restrict__ A,
                                                      const __nv_bfloat16* __restrict__ B, int K, int N,
                                                      int variant, float* __restrict__ D, int* status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint8_t* sA = smem;
    uint8_t* sB = smem + 128 * K * 2;
    for (int i = tid; i < 128 * K; i += 128)
        *reinterpret_cast<__nv_bfloat16*>(sA + tc::kmajor_offset(i / K, i % K, K)) = A[i];
    for (int i = tid; i < N * K; i += 128)
        *reinterpret_cast<__nv_bfloat16*>(sB + tc::kmajor_offset(i / K, i % K, K)) = B[i];
    const uint32_t ncols = N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256));
    if (tid == 0) tc::mbar_init(&bar, 1);
    if (warp == 0) tc::tmem_alloc(&tslot, ncols);
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = tslot;
    if (tid == 0) {
        const uint32_t kchunks = (uint32_t)(K / 8) * 128;
        const uint32_t lbo = variant == 0 ? 128u : kchunks;
        const uint32_t sbo = variant == 0 ? kchunks : 128u;
        const uint32_t idesc = tc::idesc_bf16(128, N);
        for (int kk = 0; kk < K / 16; ++kk) {
            const uint64_t ad = tc::smem_desc(tc::smem_u32(sA) + kk * 256, lbo, sbo);
            const uint64_t bd = tc::smem_desc(tc::smem_u32(sB) + kk * 256, lbo, sbo);
            tc::mma_bf16(taddr, ad, bd, idesc, kk > 0 ? 1u : 0u);
        }
        tc::mma_commit(&bar);
    }
    const bool ok = tc::mbar_wait(&bar, 0);
    tc::fence_after_sync();
    if (ok) {
        const int row = warp * 32 + lane;
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tc::tmem_ld16(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) D[row * N + c0 + i] = v[i];
        }
    } else if (lane == 0) {
        atomicExch(status, 1);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(taddr, ncols);
}

// MN-major operand self-check: D[128 x N] = A[128 x K] * B[N x K]^T with A supplied as A^T ([K][128]
// row-major) when a_mn and B as B^T ([K][N]) when b_mn; each is staged as a [K][MN] tile in the
// K-major layout and read MN-major.  lbo_k selects which descriptor field carries the stride
// between K groups of an MN-major operand (1: the leading-byte-offset field, 0: the stride field).
// The operands sit 64 KB apart in a 192 KB buffer, so either reading stays inside it.
__global__ void __launch_bounds__(128) tc_gemm_mn_kernel(const __nv_bfloat16* __restrict__ A,
                                                         const __nv_bfloat16* __restrict__ B, int K, int N, int a_mn,
                                                         int b_mn, int lbo_k, float* __restrict__ D, int* status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint8_t* sA = smem;
    uint8_t* sB = smem + 65536;
    for (int i = tid; i < 128 * K; i += 128) {
        if (a_mn)
            *reinterpret_cast<__nv_bfloat16*>(sA + tc::kmajor_offset(i / 128, i % 128, 128)) = A[i];  // A^T[k][m]
        else
            *reinterpret_cast<__nv_bfloat16*>(sA + tc::kmajor_offset(i / K, i % K, K)) = A[i];
    }
    for (int i = tid; i < N * K; i += 128) {
        if (b_mn)
            *reinterpret_cast<__nv_bfloat16*>(sB + tc::kmajor_offset(i / N, i % N, N)) = B[i];  // B^T[k][n]
        else
            *reinterpret_cast<__nv_bfloat16*>(sB + tc::kmajor_offset(i / K, i % K, K)) = B[i];
    }
    const uint32_t ncols = N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256));
    if (tid == 0) tc::mbar_init(&bar, 1);
    if (warp == 0) tc::tmem_alloc(&tslot, ncols);
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = tslot;
    if (tid == 0) {
        const uint32_t idesc = tc::idesc_bf16_mn(128, N, a_mn != 0, b_mn != 0);
        for (int kk = 0; kk < K / 16; ++kk) {
            uint64_t ad, bd;
            if (a_mn) {
                const uint32_t kstride = (128 / 8) * 128;
                ad = tc::smem_desc(tc::smem_u32(sA) + kk * 2 * kstride, lbo_k ? kstride : 128u, lbo_k ? 128u : kstride);
            } else {
                ad = tc::smem_desc(tc::smem_u32(sA) + kk * 256, 128, (uint32_t)(K / 8) * 128);
            }
            if (b_mn) {
                const uint32_t kstride = (uint32_t)(N / 8) * 128;
                bd = tc::smem_desc(tc::smem_u32(sB) + kk * 2 * kstride, lbo_k ? kstride : 128u, lbo_k ? 128u : kstride);
            } else {
                bd = tc::smem_desc(tc::smem_u32(sB) + kk * 256, 128, (uint32_t)(K / 8) * 128);
            }
            tc::mma_bf16(taddr, ad, bd, idesc, kk > 0 ? 1u : 0u);
        }
        tc::mma_commit(&bar);
    }
    const bool ok = tc::mbar_wait(&bar, 0);
    tc::fence_after_sync();
    if (ok) {
        const int row = warp * 32 + lane;
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tc::tmem_ld16(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) D[row * N + c0 + i] = v[i];
        }
    } else if (lane == 0) {
        atomicExch(status, 1);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(taddr, ncols);
}

// ------------------------------------------------------------------------------ parameters

// FP32 parameter vector layout.
constexpr int kIn = 16, kHid = 64;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + kHid * kIn, OFF_W2 = OFF_B1 + kHid, OFF_B2 = OFF_W2 + kHid * kHid,
              OFF_W3 = OFF_B2 + kHid, OFF_B3 = OFF_W3 + kHid * kHid, OFF_W4 = OFF_B3 + kHid, OFF_B4 = OFF_W4 + kHid,
              kParams = OFF_B4 + 1;
// BF16 copies of W1..W3 (row-major [out][in], which is the K-major B operand of the forward GEMMs).
constexpr int OFFB_W1 = 0, OFFB_W2 = OFFB_W1 + kHid * kIn, OFFB_W3 = OFFB_W2 + kHid * kHid, kBf16 = OFFB_W3 + kHid * kHid;

// Shared-memory image of the weights for one CTA.
struct SmemWeights {
    alignas(128) uint8_t w1[kHid * kIn * 2];     // B of layer 1: [64 out][16 in]
    alignas(128) uint8_t w2[kHid * kHid * 2];    // B of layer 2
    alignas(128) uint8_t w3[kHid * kHid * 2];    // B of layer 3
    float b1[kHid], b2[kHid], b3[kHid], w4[kHid];
    float b4;
    float pad_[3];
};

__device__ void load_weights(SmemWeights& sw, const float* __restrict__ P, const __nv_bfloat16* __restrict__ WB) {
    // 8 consecutive inputs of one output row are one 16-byte core-matrix row: one vector copy each.
    const uint4* wb = reinterpret_cast<const uint4*>(WB);
    for (int i = threadIdx.x; i < kHid * kIn / 8; i += blockDim.x)
        *reinterpret_cast<uint4*>(sw.w1 + tc::kmajor_offset(i / (kIn / 8), (i % (kIn / 8)) * 8, kIn)) =
            __ldg(wb + OFFB_W1 / 8 + i);
    for (int i = threadIdx.x; i < kHid * kHid / 8; i += blockDim.x) {
        const int o = i / (kHid / 8), k = (i % (kHid / 8)) * 8;
        *reinterpret_cast<uint4*>(sw.w2 + tc::kmajor_offset(o, k, kHid)) = __ldg(wb + OFFB_W2 / 8 + i);
        *reinterpret_cast<uint4*>(sw.w3 + tc::kmajor_offset(o, k, kHid)) = __ldg(wb + OFFB_W3 / 8 + i);
    }
    for (int i = threadIdx.x; i < kHid; i += blockDim.x) {
        sw.b1[i] = P[OFF_B1 + i];
        sw.b2[i] = P[OFF_B2 + i];
        sw.b3[i] = P[OFF_B3 + i];
        sw.w4[i] = P[OFF_W4 + i];
    }
    if (threadIdx.x == 0) sw.b4 = P[OFF_B4];
}

// ------------------------------------------------------------------------------ inference

struct InferSmem {
    SmemWeights w;
    alignas(128) uint8_t x[128 * kIn * 2];
    alignas(128) uint8_t h[128 * kHid * 2];
    uint64_t bar;
    uint32_t tslot;
};

// Where the prediction goes: Y[row] (forward), or folded into its ray's transmittance (the
// surrogate march's deferred cone terms): with meta[row] = (ray, g) and ray_b[ray] = (l_n, mix),
// beers = mix(y, max(y, 0.7 y^(1/4)), mix) (compute-clouds.comp:456-460 with exp(-dal) = y) and
// ray_u[ray].x += beers * exp(g + l_n).
struct InferOut {
    float* y;
    const float2* meta;
    const float2* ray_b;
    float4* ray_u;
};

__device__ __forceinline__ void load_x_regs(const __nv_bfloat16* __restrict__ X, int row, int n, uint4& a, uint4& b) {
    a = make_uint4(0, 0, 0, 0);
    b = a;
    if (row < n) {
        const uint4* src = reinterpret_cast<const uint4*>(X + (size_t)row * kIn);
        a = __ldcs(src);
        b = __ldcs(src + 1);
    }
}

// Hidden-layer epilogue of this thread's TMEM lane, 16 columns at a time: + bias, ReLU, bf16 into
// row r of the next layer's A tile.
__device__ __forceinline__ void epilogue_hidden(uint32_t t_row, const float* bias, uint8_t* s, int r) {
#pragma unroll
    for (int c = 0; c < kHid; c += 16) {
        float v[16];
        tc::tmem_ld16(t_row + c, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = fmaxf(v[j] + bias[c + j], 0.0f);
        *reinterpret_cast<uint4*>(s + tc::kmajor_offset(r, c, kHid)) = tc::pack8_bf16(v);
        *reinterpret_cast<uint4*>(s + tc::kmajor_offset(r, c + 8, kHid)) = tc::pack8_bf16(v + 8);
    }
}

// Last layer: z = b4 + sum_j relu(z3_j + b3_j) w4_j, summed in column order.
__device__ __forceinline__ float epilogue_out(uint32_t t_row, const SmemWeights& w) {
    float z = w.b4;
#pragma unroll
    for (int c = 0; c < kHid; c += 16) {
        float v[16];
        tc::tmem_ld16(t_row + c, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) z += fmaxf(v[j] + w.b3[c + j], 0.0f) * w.w4[c + j];
    }
    return z;
}

// One CTA of 4 warps per 128-sample tile, persistent over tiles.  The features of the CTA's next
// tile are loaded into registers while the current tile's three GEMMs and epilogues run.
template <bool kAccumulate>
__global__ void __launch_bounds__(128, 5) infer_kernel(const __nv_bfloat16* __restrict__ X, int n,
                                                       const unsigned int* __restrict__ n_dev,
                                                       const float* __restrict__ P, const __nv_bfloat16* __restrict__ WB,
                                                       InferOut out, int* status) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    InferSmem& S = *reinterpret_cast<InferSmem*>(smem_raw);
    if (n_dev) n = min(n, (int)*n_dev);  // sample count written by an earlier kernel
    const int tid = threadIdx.x, warp = tid >> 5;
    load_weights(S.w, P, WB);
    if (tid == 0) tc::mbar_init(&S.bar, 1);
    if (warp == 0) tc::tmem_alloc(&S.tslot, 64);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = S.tslot;
    const uint32_t t_row = taddr + ((uint32_t)(warp * 32) << 16);
    const uint32_t sx = tc::smem_u32(S.x), sh = tc::smem_u32(S.h);
    uint32_t phase = 0;
    bool failed = false;
    uint4 xa, xb;
    load_x_regs(X, (int)blockIdx.x * 128 + tid, n, xa, xb);
    // Accumulating epilogue: the record's (ray, g) and its ray's (l_n, mix) are loaded one tile
    // ahead as well, so the epilogue's only memory operation is a fire-and-forget atomic add.
    float2 meta_next = make_float2(0.0f, 0.0f), rb_next = make_float2(0.0f, 0.0f);
    if (kAccumulate && (int)blockIdx.x * 128 + tid < n) {
        meta_next = __ldcs(out.meta + (int)blockIdx.x * 128 + tid);
        rb_next = out.ray_b[__float_as_int(meta_next.x)];
    }
    for (int tile = blockIdx.x; tile * 128 < n && !failed; tile += gridDim.x) {
        const int row = tile * 128 + tid;
        *reinterpret_cast<uint4*>(S.x + tc::kmajor_offset(tid, 0, kIn)) = xa;
        *reinterpret_cast<uint4*>(S.x + tc::kmajor_offset(tid, 8, kIn)) = xb;
        const int next = (tile + (int)gridDim.x) * 128 + tid;
        load_x_regs(X, next, n, xa, xb);
        const float2 meta = meta_next, rb = rb_next;
        if (kAccumulate && next < n) meta_next = __ldcs(out.meta + next);
        for (int layer = 0; layer < 3; ++layer) {
            if (kAccumulate && layer == 1 && next < n) rb_next = out.ray_b[__float_as_int(meta_next.x)];
            tc::fence_async_smem();
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
            if (tid == 0) {
                if (layer == 0)
                    tc::gemm_issue(taddr, sx, tc::smem_u32(S.w.w1), kIn, kHid, &S.bar);
                else
                    tc::gemm_issue(taddr, sh, tc::smem_u32(layer == 1 ? S.w.w2 : S.w.w3), kHid, kHid, &S.bar);
            }
            const bool ok = tc::mbar_wait(&S.bar, phase);
            phase ^= 1u;
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            tc::fence_after_sync();
            if (layer < 2) epilogue_hidden(t_row, layer == 0 ? S.w.b1 : S.w.b2, S.h, tid);
        }
        if (failed) break;
        const float z = epilogue_out(t_row, S.w);
        if (row < n) {
            const float y = 1.0f / (1.0f + __expf(-z));
            if (kAccumulate) {
                const float beers = y * (1.0f - rb.y) + fmaxf(y, 0.7f * sqrtf(sqrtf(y))) * rb.y;
                atomicAdd(&out.ray_u[__float_as_int(meta.x)].x, beers * __expf(meta.y + rb.x));
            } else {
                out.y[row] = y;
            }
        }
    }
    if (failed && tid == 0) atomicExch(status, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(taddr, 64);
}

// ------------------------------------------------------------------------------ training
//
// Shared-memory tiles, all in the K-major layout of tc.cuh, each also read MN-major (transposed in
// place) by the weight-gradient GEMMs:
//   x  [128][32]:  features in columns 0..15, a ones column 16, zeros 17..31
//   h1 [128][80], h2 [128][80]: activations in 0..63, ones column 64, zeros 65..79
//   d  [128][128]: the delta of the current layer in 0..63, zeros 64..127
// GEMMs per tile (D in TMEM, A x B^T):
//   forward       z1 = x W1^T      A = x (K-major, K = 16)    B = W1 (K-major)
//                 z2 = h1 W2^T, z3 = h2 W3^T
//   weight grads  dW3|db3 += d3^T [h2 1]   A = d (MN-major, M = 128 rows of which 64 real, K = 128 samples)
//                                          B = h2 (MN-major, N = 80)
//                 dW2|db2 += d2^T [h1 1],  dW1|db1 += d1^T [x 1] (N = 32)
//   deltas        d2 = (d3 W3) * [z2 > 0]  A = d (K-major, K = 64), B = W3 (MN-major: [out][in] read as [in][out])
//                 d1 = (d2 W2) * [z1 > 0]
// The ones columns turn the bias gradients into one more output column of the weight-gradient GEMMs.

struct TrainSmem {
    SmemWeights w;
    alignas(128) uint8_t x[128 * 32 * 2];
    alignas(128) uint8_t h1[128 * 80 * 2];
    alignas(128) uint8_t h2[128 * 80 * 2];
    alignas(128) uint8_t d[128 * 128 * 2];
    uint64_t bar;
    uint32_t tslot;
};

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Writes a weight-gradient tile (TMEM columns [0, n_in] of lanes 0..63 from t_row, the last one the
// bias) into the CTA's row of partial gradients.  Run by warps 0 and 1.
__device__ __forceinline__ void flush_dw(uint32_t t_row, int o, int n_in, float* Gp, int off_w, int off_b) {
    float v[16];
    for (int c = 0; c < n_in + 16; c += 16) {
        tc::tmem_ld16(t_row + c, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int i = c + j;
            if (i < n_in)
                Gp[off_w + o * n_in + i] = v[j];
            else if (i == n_in)
                Gp[off_b + o] = v[j];
        }
    }
}

// K-major x K-major GEMM where the operand tiles are wider than the K used: a_cols / b_cols are the
// tiles' widths (their 8-row groups are (cols / 8) * 128 bytes apart).
__device__ __forceinline__ void gemm_kk(uint32_t d_tmem, uint32_t sa, int a_cols, uint32_t sb, int b_cols, int K, int N,
                                        uint32_t idesc, uint32_t accumulate) {
    for (int kk = 0; kk < K / 16; ++kk)
        tc::mma_bf16(d_tmem, tc::smem_desc(sa + kk * 256, 128, (uint32_t)(a_cols / 8) * 128),
                     tc::smem_desc(sb + kk * 256, 128, (uint32_t)(b_cols / 8) * 128), idesc, kk > 0 ? 1u : accumulate);
}

// Weight-gradient GEMM: A = d read MN-major (M = 128, K = 128 samples), B = an activation tile of
// width n_cols read MN-major (N = n_cols).  MN-major operands: K groups (8 samples) are
// (cols / 8) * 128 bytes apart (descriptor leading-byte-offset field), MN groups 128 bytes.
__device__ __forceinline__ void gemm_dw(uint32_t d_tmem, uint32_t s_d, uint32_t s_act, int n_cols, uint32_t accumulate) {
    const uint32_t idesc = tc::idesc_bf16_mn(128, n_cols, true, true);
    const uint32_t ka = (128 / 8) * 128, kb = (uint32_t)(n_cols / 8) * 128;
    for (int kk = 0; kk < 128 / 16; ++kk)
        tc::mma_bf16(d_tmem, tc::smem_desc(s_d + kk * 2 * ka, ka, 128), tc::smem_desc(s_act + kk * 2 * kb, kb, 128), idesc,
                     kk > 0 ? 1u : accumulate);
}

// Delta GEMM: D = d (K-major, K = 64, tile width 128) x W (the [64 out][64 in] forward weight tile
// read MN-major as [in][out]).
__device__ __forceinline__ void gemm_delta(uint32_t d_tmem, uint32_t s_d, uint32_t s_w) {
    const uint32_t idesc = tc::idesc_bf16_mn(128, kHid, false, true);
    const uint32_t kb = (kHid / 8) * 128;
    for (int kk = 0; kk < kHid / 16; ++kk)
        tc::mma_bf16(d_tmem, tc::smem_desc(s_d + kk * 256, 128, (128 / 8) * 128),
                     tc::smem_desc(s_w + kk * 2 * kb, kb, 128), idesc, kk > 0 ? 1u : 0u);
}

// Features of the thread's row (zeros past n) and its target.
__device__ __forceinline__ void load_sample(const __nv_bfloat16* __restrict__ X, const float* __restrict__ T, int row,
                                            int n, uint4& a, uint4& b, float& t) {
    a = make_uint4(0, 0, 0, 0);
    b = a;
    t = 0.0f;
    if (row < n) {
        const uint4* src = reinterpret_cast<const uint4*>(X + (size_t)row * kIn);
        a = __ldg(src);
        b = __ldg(src + 1);
        t = __ldg(T + row);
    }
}

// Hidden-layer epilogue into an activation tile of width 80: + bias, ReLU, bf16.
__device__ __forceinline__ void train_epilogue_hidden(uint32_t t_row, const float* bias, uint8_t* s, int r) {
#pragma unroll
    for (int c = 0; c < kHid; c += 16) {
        float v[16];
        tc::tmem_ld16(t_row + c, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = fmaxf(v[j] + bias[c + j], 0.0f);
        *reinterpret_cast<uint4*>(s + tc::kmajor_offset(r, c, 80)) = tc::pack8_bf16(v);
        *reinterpret_cast<uint4*>(s + tc::kmajor_offset(r, c + 8, 80)) = tc::pack8_bf16(v + 8);
    }
}

// Delta epilogue: (TMEM row) * [activation of the layer below > 0] as bf16 into d.
__device__ __forceinline__ void train_epilogue_delta(uint32_t t_row, const uint8_t* act, uint8_t* d, int r) {
#pragma unroll
    for (int c = 0; c < kHid; c += 16) {
        float v[16];
        tc::tmem_ld16(t_row + c, v);
#pragma unroll
        for (int j = 0; j < 16; j += 8) {
            const uint4 m = *reinterpret_cast<const uint4*>(act + tc::kmajor_offset(r, c + j, 80));
            const __nv_bfloat16* mb = reinterpret_cast<const __nv_bfloat16*>(&m);
#pragma unroll
            for (int q = 0; q < 8; ++q) v[j + q] = __bfloat162float(mb[q]) > 0.0f ? v[j + q] : 0.0f;
        }
        *reinterpret_cast<uint4*>(d + tc::kmajor_offset(r, c, 128)) = tc::pack8_bf16(v);
        *reinterpret_cast<uint4*>(d + tc::kmajor_offset(r, c + 8, 128)) = tc::pack8_bf16(v + 8);
    }
}

// Each CTA trains on tiles tile0 + blockIdx.x, + gridDim.x, ... and writes its gradient sum (and
// its squared-error sum at index kParams) as row blockIdx.x of Gp (kParams + 1 floats per row);
// the rows are summed by the Adam (or gradient) kernel, so no two CTAs write the same address.
__global__ void __launch_bounds__(128, 2) train_kernel(const __nv_bfloat16* __restrict__ X, const float* __restrict__ T,
                                                       int n, int tile0, int tiles, float inv_batch,
                                                       const float* __restrict__ P,
                                                       const __nv_bfloat16* __restrict__ WB, float* __restrict__ Gp_all,
                                                       int* status) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>(smem_raw);
    __shared__ float s_out[kHid + 2];  // w4 gradient, b4 gradient, loss of the CTA
    float* Gp = Gp_all + (size_t)blockIdx.x * (kParams + 1);
    if (threadIdx.x < kHid + 2) s_out[threadIdx.x] = 0.0f;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    load_weights(S.w, P, WB);
    // Constant columns: ones (bias gradients) and zeros (padding), written once.
    {
        const __nv_bfloat16 one = __float2bfloat16_rn(1.0f), zero = __float2bfloat16_rn(0.0f);
        for (int c = 16; c < 32; ++c)
            *reinterpret_cast<__nv_bfloat16*>(S.x + tc::kmajor_offset(tid, c, 32)) = c == 16 ? one : zero;
        for (int c = 64; c < 80; ++c) {
            *reinterpret_cast<__nv_bfloat16*>(S.h1 + tc::kmajor_offset(tid, c, 80)) = c == 64 ? one : zero;
            *reinterpret_cast<__nv_bfloat16*>(S.h2 + tc::kmajor_offset(tid, c, 80)) = c == 64 ? one : zero;
        }
        for (int c = 64; c < 128; c += 8)
            *reinterpret_cast<uint4*>(S.d + tc::kmajor_offset(tid, c, 128)) = make_uint4(0, 0, 0, 0);
    }
    if (tid == 0) tc::mbar_init(&S.bar, 1);
    if (warp == 0) tc::tmem_alloc(&S.tslot, 256);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = S.tslot;
    const uint32_t lane_off = (uint32_t)(warp * 32) << 16;
    // Tensor-memory columns: activations / deltas (64), then the weight gradients of layers 3 and 2
    // (64 + bias + padding = 80 each) and 1 (16 + bias + padding = 32), summed over the CTA's tiles.
    const uint32_t tA = taddr, tW3 = taddr + 64, tW2 = taddr + 144, tW1 = taddr + 224;
    const uint32_t sx = tc::smem_u32(S.x), sh1 = tc::smem_u32(S.h1), sh2 = tc::smem_u32(S.h2), sd = tc::smem_u32(S.d);
    const uint32_t idesc_fwd = tc::idesc_bf16(128, kHid);
    uint32_t acc_dw = 0;  // 0 for the CTA's first tile: its gradient GEMMs overwrite the columns
    uint32_t phase = 0;
    bool failed = false;
    float acc_dw4[kHid];
#pragma unroll
    for (int j = 0; j < kHid; ++j) acc_dw4[j] = 0.0f;
    float acc_db4 = 0.0f, acc_loss = 0.0f;

    // Issues one group of MMAs from thread 0 after the block's shared-memory writes, then waits.
    auto run_mma = [&](auto&& issue) -> bool {
        tc::fence_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (tid == 0) {
            issue();
            tc::mma_commit(&S.bar);
        }
        const bool ok = tc::mbar_wait(&S.bar, phase);
        phase ^= 1u;
        if (__syncthreads_or(!ok)) return false;
        tc::fence_after_sync();
        return true;
    };

    uint4 xa, xb;
    float tv;
    load_sample(X, T, (tile0 + (int)blockIdx.x) * 128 + tid, n, xa, xb, tv);
    for (int tile = tile0 + blockIdx.x; tile < tile0 + tiles && !failed; tile += gridDim.x) {
        const int row = tile * 128 + tid;
        const bool valid = row < n;
        const float target = tv;
        *reinterpret_cast<uint4*>(S.x + tc::kmajor_offset(tid, 0, 32)) = xa;
        *reinterpret_cast<uint4*>(S.x + tc::kmajor_offset(tid, 8, 32)) = xb;
        if (tile + (int)gridDim.x < tile0 + tiles) load_sample(X, T, (tile + (int)gridDim.x) * 128 + tid, n, xa, xb, tv);
        // ---- forward
        if (!(failed = !run_mma([&] { gemm_kk(tA, sx, 32, tc::smem_u32(S.w.w1), kIn, kIn, kHid, idesc_fwd, 0u); }))) {
            train_epilogue_hidden(tA + lane_off, S.w.b1, S.h1, tid);
        }
        if (failed) break;
        if (!(failed = !run_mma([&] { gemm_kk(tA, sh1, 80, tc::smem_u32(S.w.w2), kHid, kHid, kHid, idesc_fwd, 0u); }))) {
            train_epilogue_hidden(tA + lane_off, S.w.b2, S.h2, tid);
        }
        if (failed) break;
        if ((failed = !run_mma([&] { gemm_kk(tA, sh2, 80, tc::smem_u32(S.w.w3), kHid, kHid, kHid, idesc_fwd, 0u); })))
            break;
        // ---- output layer, loss, and the output-layer delta (CUDA cores)
        float z = S.w.b4;
#pragma unroll
        for (int c = 0; c < kHid; c += 16) {
            float v[16];
            tc::tmem_ld16(tA + lane_off + c, v);
#pragma unroll
            for (int j = 0; j < 16; ++j) z += fmaxf(v[j] + S.w.b3[c + j], 0.0f) * S.w.w4[c + j];
        }
        const float y = 1.0f / (1.0f + expf(-z));
        const float err = valid ? y - target : 0.0f;
        const float dz = 2.0f * err * y * (1.0f - y) * inv_batch;
        acc_loss += err * err;
        acc_db4 += dz;
#pragma unroll
        for (int c = 0; c < kHid; c += 16) {
            float v[16];
            tc::tmem_ld16(tA + lane_off + c, v);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const float h = fmaxf(v[j] + S.w.b3[c + j], 0.0f);
                acc_dw4[c + j] += dz * h;
                v[j] = h > 0.0f ? dz * S.w.w4[c + j] : 0.0f;
            }
            *reinterpret_cast<uint4*>(S.d + tc::kmajor_offset(tid, c, 128)) = tc::pack8_bf16(v);
            *reinterpret_cast<uint4*>(S.d + tc::kmajor_offset(tid, c + 8, 128)) = tc::pack8_bf16(v + 8);
        }
        // ---- layer 3: dW3 and the delta of layer 2
        if (!(failed = !run_mma([&] {
                  gemm_dw(tW3, sd, sh2, 80, acc_dw);
                  gemm_delta(tA, sd, tc::smem_u32(S.w.w3));
              }))) {
            train_epilogue_delta(tA + lane_off, S.h2, S.d, tid);
        }
        if (failed) break;
        // ---- layer 2: dW2 and the delta of layer 1
        if (!(failed = !run_mma([&] {
                  gemm_dw(tW2, sd, sh1, 80, acc_dw);
                  gemm_delta(tA, sd, tc::smem_u32(S.w.w2));
              }))) {
            train_epilogue_delta(tA + lane_off, S.h1, S.d, tid);
        }
        if (failed) break;
        // ---- layer 1: dW1
        if ((failed = !run_mma([&] { gemm_dw(tW1, sd, sx, 32, acc_dw); }))) break;
        acc_dw = 1u;
    }
    // ---- hidden-layer weight gradients of all the CTA's tiles
    if (!failed && acc_dw && warp < 2) {
        const int o = warp * 32 + lane;
        flush_dw(tW3 + lane_off, o, kHid, Gp, OFF_W3, OFF_B3);
        flush_dw(tW2 + lane_off, o, kHid, Gp, OFF_W2, OFF_B2);
        flush_dw(tW1 + lane_off, o, kIn, Gp, OFF_W1, OFF_B1);
    }
    // ---- output-layer gradients and loss: warp sums, then the CTA's sum
#pragma unroll
    for (int j = 0; j < kHid; ++j) {
        const float v = warp_sum(acc_dw4[j]);
        if (lane == 0) atomicAdd(&s_out[j], v);
    }
    {
        const float v = warp_sum(acc_db4), l2 = warp_sum(acc_loss);
        if (lane == 0) {
            atomicAdd(&s_out[kHid], v);
            atomicAdd(&s_out[kHid + 1], l2);
        }
    }
    __syncthreads();
    if (tid < kHid) Gp[OFF_W4 + tid] = s_out[tid];
    if (tid == kHid) Gp[OFF_B4] = s_out[kHid];
    if (tid == kHid + 1) Gp[kParams] = s_out[kHid + 1];
    if (failed && tid == 0) atomicExch(status, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(taddr, 256);
}

// Adam on the FP32 parameters; refreshes the BF16 copies and clears the gradient buffer.
// Sum of the training kernel's `parts` partial rows at index i (i == kParams: the squared error).
__device__ __forceinline__ float sum_parts(const float* __restrict__ Gp, int parts, int i) {
    float g = 0.0f;
    for (int c = 0; c < parts; ++c) g += Gp[(size_t)c * (kParams + 1) + i];
    return g;
}

// Gradient (and loss) of a training launch into G and *loss, for callers that read the gradient.
__global__ void reduce_grad_kernel(const float* __restrict__ Gp, int parts, float* __restrict__ G,
                                   float* __restrict__ loss) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kParams) G[i] = sum_parts(Gp, parts, i);
    if (i == kParams && loss) *loss = sum_parts(Gp, parts, i);
}

__global__ void adam_kernel(float* __restrict__ P, __nv_bfloat16* __restrict__ WB, const float* __restrict__ Gp,
                            int parts, float* __restrict__ loss, float* __restrict__ Mo, float* __restrict__ Vo,
                            float lr, float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == kParams && loss) *loss = sum_parts(Gp, parts, i);
    if (i >= kParams) return;
    const float g = sum_parts(Gp, parts, i);
    const float m = b1 * Mo[i] + (1.0f - b1) * g;
    const float v = b2 * Vo[i] + (1.0f - b2) * g * g;
    Mo[i] = m;
    Vo[i] = v;
    const float p = P[i] - lr * (m / c1) / (sqrtf(v / c2) + eps);
    P[i] = p;
    if (i < OFF_B1)
        WB[OFFB_W1 + (i - OFF_W1)] = __float2bfloat16_rn(p);
    else if (i >= OFF_W2 && i < OFF_B2)
        WB[OFFB_W2 + (i - OFF_W2)] = __float2bfloat16_rn(p);
    else if (i >= OFF_W3 && i < OFF_B3)
        WB[OFFB_W3 + (i - OFF_W3)] = __float2bfloat16_rn(p);
}

__global__ void refresh_bf16_kernel(const float* __restrict__ P, __nv_bfloat16* __restrict__ WB) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kHid * kIn) WB[OFFB_W1 + i] = __float2bfloat16_rn(P[OFF_W1 + i]);
    if (i < kHid * kHid) {
        WB[OFFB_W2 + i] = __float2bfloat16_rn(P[OFF_W2 + i]);
        WB[OFFB_W3 + i] = __float2bfloat16_rn(P[OFF_W3 + i]);
    }
}

}  // namespace mlp
}  // namespace mm

// ------------------------------------------------------------------------------ host side

struct mm_mlp_s {
    float* P = nullptr;          // FP32 parameters
    __nv_bfloat16* WB = nullptr;  // BF16 copies of W1..W3
    float* Gp = nullptr;         // per-CTA partial gradients + squared error of a training launch
    float* M = nullptr;          // Adam first moment
    float* V = nullptr;          // Adam second moment
    float* loss = nullptr;       // one float
    int* status = nullptr;       // bounded-wait failure flag
    long long step = 0;          // Adam steps taken
    int num_sms = 0;
};

namespace {

size_t infer_smem() { return sizeof(mm::mlp::InferSmem) + 1024; }
size_t train_smem() { return sizeof(mm::mlp::TrainSmem) + 1024; }

int set_smem_limits() {
    static bool done = false;
    if (done) return MM_OK;
    MM_CUDA_TRY(cudaFuncSetAttribute(mm::mlp::infer_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)infer_smem()));
    MM_CUDA_TRY(cudaFuncSetAttribute(mm::mlp::infer_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)infer_smem()));
    MM_CUDA_TRY(cudaFuncSetAttribute(mm::mlp::train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem()));
    done = true;
    return MM_OK;
}

int check_status(mm_mlp m, cudaStream_t s) {
    int st = 0;
    MM_CUDA_TRY(cudaMemcpyAsync(&st, m->status, sizeof(int), cudaMemcpyDeviceToHost, s));
    MM_CUDA_TRY(cudaStreamSynchronize(s));
    if (st) return mm::fail(MM_ERR_TIMEOUT, "mlp: a tensor-core wait gave up");
    return MM_OK;
}

int refresh(mm_mlp m, cudaStream_t s) {
    mm::mlp::refresh_bf16_kernel<<<(mm::mlp::kHid * mm::mlp::kHid + 255) / 256, 256, 0, s>>>(m->P, m->WB);
    MM_CUDA_TRY(cudaGetLastError());
    mm::count_launch();
    return MM_OK;
}

// Partial-gradient rows of a training launch over `tiles` tiles: two CTAs per SM, each at least one tile.
int train_grid(mm_mlp m, int tiles) { return tiles < 2 * m->num_sms ? tiles : 2 * m->num_sms; }

// Runs the training kernel over tiles [tile0, tile0 + tiles) of (X, T) into m->Gp (train_grid rows).
int run_train(mm_mlp m, const void* X, const float* T, int n, int tile0, int tiles, float inv_batch, cudaStream_t s) {
    const int grid = train_grid(m, tiles);
    // The shared-memory image needs 1024-byte alignment; the kernel takes the dynamic buffer as is.
    mm::mlp::train_kernel<<<grid, 128, train_smem(), s>>>((const __nv_bfloat16*)X, T, n, tile0, tiles, inv_batch, m->P,
                                                         m->WB, m->Gp, m->status);
    MM_CUDA_TRY(cudaGetLastError());
    mm::count_launch();
    return MM_OK;
}

}  // namespace

namespace mm {

// Inference on up to `cap` deferred cone samples of the surrogate march (the actual count read from
// device memory), each prediction folded into its ray's transmittance (InferOut above).
int mlp_infer_accumulate(mm_mlp m, const void* d_x, int cap, const unsigned int* d_count, const float2* meta,
                         const float2* ray_b, float4* ray_u, cudaStream_t s) {
    int r = set_smem_limits();
    if (r) return r;
    const int tiles = (cap + 127) / 128;
    const int grid = tiles < 5 * m->num_sms ? tiles : 5 * m->num_sms;
    mlp::InferOut o{nullptr, meta, ray_b, ray_u};
    mlp::infer_kernel<true><<<grid, 128, infer_smem(), s>>>((const __nv_bfloat16*)d_x, cap, d_count, m->P, m->WB, o,
                                                            m->status);
    MM_CUDA_TRY(cudaGetLastError());
    count_launch();
    return MM_OK;
}

int* mlp_status_ptr(mm_mlp m) { return m->status; }

}  // namespace mm

extern "C" {

int mm_mlp_param_count(void) { return mm::mlp::kParams; }

int mm_mlp_create(uint32_t seed, mm_mlp* out) {
    using namespace mm::mlp;
    if (!out) return mm::fail(MM_ERR_INVALID_ARGUMENT, "mlp: null output");
    int r = set_smem_limits();
    if (r) return r;
    mm_mlp m = new (std::nothrow) mm_mlp_s;
    if (!m) return mm::fail(MM_ERR_OUT_OF_MEMORY, "mlp: host allocation");
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&m->num_sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaSuccess;
    e = e ? e : cudaMalloc(&m->P, kParams * sizeof(float));
    e = e ? e : cudaMalloc(&m->WB, kBf16 * sizeof(__nv_bfloat16));
    e = e ? e : cudaMalloc(&m->Gp, (size_t)2 * m->num_sms * (kParams + 1) * sizeof(float));
    e = e ? e : cudaMalloc(&m->M, kParams * sizeof(float));
    e = e ? e : cudaMalloc(&m->V, kParams * sizeof(float));
    e = e ? e : cudaMalloc(&m->loss, sizeof(float));
    e = e ? e : cudaMalloc(&m->status, sizeof(int));
    if (e != cudaSuccess) {
        mm_mlp_destroy(m);
        return mm::cuda_fail(e, "mlp buffers");
    }
    // He-uniform initialisation from a 64-bit LCG (seeded, host side), zero biases.
    float* h = new float[kParams];
    uint64_t st = 0x9E3779B97F4A7C15ull ^ seed;
    auto uni = [&]() {
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        return (float)((st >> 40) * (1.0 / 16777216.0)) * 2.0f - 1.0f;
    };
    for (int i = 0; i < kParams; ++i) h[i] = 0.0f;
    const float a1 = sqrtf(6.0f / kIn), a2 = sqrtf(6.0f / kHid);
    for (int i = 0; i < kHid * kIn; ++i) h[OFF_W1 + i] = a1 * uni();
    for (int i = 0; i < kHid * kHid; ++i) h[OFF_W2 + i] = a2 * uni();
    for (int i = 0; i < kHid * kHid; ++i) h[OFF_W3 + i] = a2 * uni();
    for (int i = 0; i < kHid; ++i) h[OFF_W4 + i] = a2 * 0.5f * uni();
    e = cudaMemcpy(m->P, h, kParams * sizeof(float), cudaMemcpyHostToDevice);
    delete[] h;
    e = e ? e : cudaMemset(m->M, 0, kParams * sizeof(float));
    e = e ? e : cudaMemset(m->V, 0, kParams * sizeof(float));
    e = e ? e : cudaMemset(m->status, 0, sizeof(int));
    if (e != cudaSuccess || (r = refresh(m, 0)) != MM_OK || (e = cudaDeviceSynchronize()) != cudaSuccess) {
        mm_mlp_destroy(m);
        return r ? r : mm::cuda_fail(e, "mlp init");
    }
    *out = m;
    return MM_OK;
}

int mm_mlp_destroy(mm_mlp m) {
    if (!m) return mm::fail(MM_ERR_INVALID_ARGUMENT, "mlp: null handle");
    cudaFree(m->P);
    cudaFree(m->WB);
    cudaFree(m->Gp);
    cudaFree(m->M);
    cudaFree(m->V);
    cudaFree(m->loss);
    cudaFree(m->status);
    delete m;
    return MM_OK;
}

int mm_mlp_get_params(mm_mlp m, float* host, int n) {
    if (!m || !host || n != mm::mlp::kParams) return mm::fail(MM_ERR_INVALID_ARGUMENT, "mlp: bad get_params");
    MM_CUDA_TRY(cudaMemcpy(host, m->P, n * sizeof(float), cudaMemcpyDeviceToHost));
    return MM_OK;
}

int mm_mlp_set_params(mm_mlp m, const float* host, int n) {
    if (!m || !host || n != mm::mlp::kParams) return mm::fail(MM_ERR_INVALID_ARGUMENT, "mlp: bad set_params");
    MM_CUDA_TRY(cudaMemcpy(m->P, host, n * sizeof(float), cudaMemcpyHostToDevice));
    int r = refresh(m, 0);
    if (r) return r;
    MM_CUDA_TRY(cudaDeviceSynchronize());
    return MM_OK;
}

int mm_mlp_forward(mm_mlp m, const void* d_x, int n, float* d_y, void* stream) {
    if (!m || !d_x || !d_y || n < 0) return mm::fail(MM_ERR_INVALID_ARGUMENT, "mlp: bad forward arguments");
    if (((uintptr_t)d_x) % 16) return mm::fail(MM_ERR_INVALID_ARGUMENT, "mlp: features must be 16-byte aligned");
    if (n == 0) return MM_OK;
    int r = set_smem_limits();
    if (r) return r;
    cudaStream_t s = (cudaStream_t)stream;
    const int tiles = (n + 127) / 128;
    const int grid = tiles < 5 * m->num_sms ? tiles : 5 * m->num_sms;
    mm::mlp::InferOut o{d_y, nullptr, nullptr, nullptr};
    mm::mlp::infer_kernel<false><<<grid, 128, infer_smem(), s>>>((const __nv_bfloat16*)d_x, n, nullptr, m->P, m->WB, o,
                                                                 m->status);
    MM_CUDA_TRY(cudaGetLastError());
    mm::count_launch();
    return MM_OK;
}

int mm_mlp_gradients(mm_mlp m, const void* d_x, const float* d_t, int n, float* d_grad, float* h_loss, void* stream) {
    if (!m || !d_x || !d_t || !d_grad || n <= 0) return mm::fail(MM_ERR_INVALID_ARGUMENT, "mlp: bad gradient arguments");
    if (((uintptr_t)d_x) % 16) return mm::fail(MM_ERR_INVALID_ARGUMENT, "mlp: features must be 16-byte aligned");
    int r = set_smem_limits();
    if (r) return r;
    cudaStream_t s = (cudaStream_t)stream;
    const int tiles = (n + 127) / 128;
    if ((r = run_train(m, d_x, d_t, n, 0, tiles, 1.0f / (float)n, s))) return r;
    mm::mlp::reduce_grad_kernel<<<(mm::mlp::kParams + 256) / 256, 256, 0, s>>>(m->Gp, train_grid(m, tiles), d_grad,
                                                                              m->loss);
    MM_CUDA_TRY(cudaGetLastError());
    mm::count_launch();
    if ((r = check_status(m, s))) return r;
    if (h_loss) {
        float l = 0.0f;
        MM_CUDA_TRY(cudaMemcpy(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost));
        *h_loss = l / (float)n;
    }
    return MM_OK;
}

int mm_mlp_train(mm_mlp m, const void* d_x, const float* d_t, int n, int batch, int steps, float lr,
                 float* h_loss_history, void* stream) {
    if (!m || !d_x || !d_t || n < 128 || batch < 128 || batch % 128 || steps <= 0 || !(lr > 0.0f))
        return mm::fail(MM_ERR_INVALID_ARGUMENT, "mlp: bad training arguments");
    if (((uintptr_t)d_x) % 16) return mm::fail(MM_ERR_INVALID_ARGUMENT, "mlp: features must be 16-byte aligned");
    int r = set_smem_limits();
    if (r) return r;
    cudaStream_t s = (cudaStream_t)stream;
    const int total_tiles = n / 128;  // whole tiles only
    const int tiles = batch / 128 < total_tiles ? batch / 128 : total_tiles;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    int cursor = 0;
    for (int k = 0; k < steps; ++k) {
        if (cursor + tiles > total_tiles) cursor = 0;
        if ((r = run_train(m, d_x, d_t, n, cursor, tiles, 1.0f / (float)(tiles * 128), s))) return r;
        cursor += tiles;
        m->step += 1;
        const float c1 = 1.0f - powf(b1, (float)m->step), c2 = 1.0f - powf(b2, (float)m->step);
        mm::mlp::adam_kernel<<<(mm::mlp::kParams + 256) / 256, 256, 0, s>>>(
            m->P, m->WB, m->Gp, train_grid(m, tiles), h_loss_history ? m->loss : nullptr, m->M, m->V, lr, b1, b2, eps,
            c1, c2);
        MM_CUDA_TRY(cudaGetLastError());
        mm::count_launch();
        if (h_loss_history) {
            float l = 0.0f;
            MM_CUDA_TRY(cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, s));
            MM_CUDA_TRY(cudaStreamSynchronize(s));
            h_loss_history[k] = l / (float)(tiles * 128);
        }
    }
    return check_status(m, s);
}

// Checkpoint: "MMMLP001", int32 parameter count, int64 Adam step, then P, M, V (FP32).
int mm_mlp_save(mm_mlp m, const char* path) {
    if (!m || !path) return mm::fail(MM_ERR_INVALID_ARGUMENT, "mlp: bad save arguments");
    const int n = mm::mlp::kParams;
    float* h = new float[3 * (size_t)n];
    cudaError_t e = cudaMemcpy(h, m->P, n * sizeof(float), cudaMemcpyDeviceToHost);
    e = e ? e : cudaMemcpy(h + n, m->M, n * sizeof(float), cudaMemcpyDeviceToHost);
    e = e ? e : cudaMemcpy(h + 2 * n, m->V, n * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        delete[] h;
        return mm::cuda_fail(e, "mlp save copy");
    }
    FILE* f = fopen(path, "wb");
    if (!f) {
        delete[] h;
        return mm::fail(MM_ERR_INVALID_ARGUMENT, "mlp: cannot open %s", path);
    }
    const int32_t cnt = n;
    const int64_t step = m->step;
    bool ok = fwrite("MMMLP001", 1, 8, f) == 8 && fwrite(&cnt, 4, 1, f) == 1 && fwrite(&step, 8, 1, f) == 1 &&
              fwrite(h, sizeof(float), 3 * (size_t)n, f) == 3 * (size_t)n;
    ok = (fclose(f) == 0) && ok;
    delete[] h;
    return ok ? MM_OK : mm::fail(MM_ERR_INVALID_ARGUMENT, "mlp: short write to %s", path);
}

int mm_mlp_load(mm_mlp m, const char* path) {
    if (!m || !path) return mm::fail(MM_ERR_INVALID_ARGUMENT, "mlp: bad load arguments");
    const int n = mm::mlp::kParams;
    FILE* f = fopen(path, "rb");
    if (!f) return mm::fail(MM_ERR_INVALID_ARGUMENT, "mlp: cannot open %s", path);
    char magic[8];
    int32_t cnt = 0;
    int64_t step = 0;
    float* h = new float[3 * (size_t)n];
    bool ok = fread(magic, 1, 8, f) == 8 && memcmp(magic, "MMMLP001", 8) == 0 && fread(&cnt, 4, 1, f) == 1 &&
              cnt == n && fread(&step, 8, 1, f) == 1 && fread(h, sizeof(float), 3 * (size_t)n, f) == 3 * (size_t)n;
    fclose(f);
    if (!ok) {
        delete[] h;
        return mm::fail(MM_ERR_INVALID_ARGUMENT, "mlp: %s is not a checkpoint of this network", path);
    }
    cudaError_t e = cudaMemcpy(m->P, h, n * sizeof(float), cudaMemcpyHostToDevice);
    e = e ? e : cudaMemcpy(m->M, h + n, n * sizeof(float), cudaMemcpyHostToDevice);
    e = e ? e : cudaMemcpy(m->V, h + 2 * n, n * sizeof(float), cudaMemcpyHostToDevice);
    delete[] h;
    if (e != cudaSuccess) return mm::cuda_fail(e, "mlp load copy");
    m->step = step;
    int r = refresh(m, 0);
    if (r) return r;
    MM_CUDA_TRY(cudaDeviceSynchronize());
    return MM_OK;
}

}  // extern "C"

extern "C" int mm_tc_gemm_check(const void* d_a, const void* d_b, int K, int N, int variant, float* d_out,
                                int* d_status, void* stream) {
    using namespace mm;
    if (!d_a || !d_b || !d_out || !d_status) return fail(MM_ERR_INVALID_ARGUMENT, "tc gemm: null pointer");
    if (K < 16 || K > 128 || K % 16 || N < 16 || N > 128 || N % 16)
        return fail(MM_ERR_INVALID_ARGUMENT, "tc gemm: K and N must be multiples of 16 in [16, 128]");
    const size_t smem = (size_t)(128 + N) * K * 2;
    cudaStream_t s = (cudaStream_t)stream;
    MM_CUDA_TRY(cudaFuncSetAttribute(mlp::tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    mlp::tc_gemm_kernel<<<1, 128, smem, s>>>((const __nv_bfloat16*)d_a, (const __nv_bfloat16*)d_b, K, N, variant,
                                             d_out, d_status);
    MM_CUDA_TRY(cudaGetLastError());
    count_launch();
    return MM_OK;
}

extern "C" int mm_tc_gemm_mn_check(const void* d_a, const void* d_b, int K, int N, int a_mn, int b_mn, int lbo_k,
                                   float* d_out, int* d_status, void* stream) {
    using namespace mm;
    if (!d_a || !d_b || !d_out || !d_status) return fail(MM_ERR_INVALID_ARGUMENT, "tc gemm: null pointer");
    if (K < 16 || K > 128 || K % 16 || N < 16 || N > 128 || N % 16)
        return fail(MM_ERR_INVALID_ARGUMENT, "tc gemm: K and N must be multiples of 16 in [16, 128]");
    const size_t smem = 3 * 65536;
    cudaStream_t s = (cudaStream_t)stream;
    MM_CUDA_TRY(cudaFuncSetAttribute(mlp::tc_gemm_mn_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    mlp::tc_gemm_mn_kernel<<<1, 128, smem, s>>>((const __nv_bfloat16*)d_a, (const __nv_bfloat16*)d_b, K, N, a_mn, b_mn,
                                                lbo_k, d_out, d_status);
    MM_CUDA_TRY(cudaGetLastError());
    count_launch();
    return MM_OK;
}

// ------------------------------------------------------------------------------ bounded-wait self-test

namespace {

// One thread initializes an mbarrier (arrival count 1), arrives on it or not, and waits for its
// phase with a poll limit: status 0 = the phase completed, 1 = the wait gave up (nothing arrived).
__global__ void wait_check_kernel(int arrive, unsigned int limit, int* status) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x != 0) return;
    mm::tc::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (arrive) mm::tc::mbar_arrive(&bar);
    *status = mm::tc::mbar_wait(&bar, 0, limit) ? 0 : 1;
}

}  // namespace

extern "C" int mm_tc_wait_check(int arrive, unsigned int poll_limit, int* d_status, void* stream) {
    if (!d_status || poll_limit == 0 || poll_limit > (1u << 24))
        return mm::fail(MM_ERR_INVALID_ARGUMENT, "wait check: bad arguments");
    wait_check_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(arrive ? 1 : 0, poll_limit, d_status);
    MM_CUDA_TRY(cudaGetLastError());
    mm::count_launch();
    return MM_OK;
}
