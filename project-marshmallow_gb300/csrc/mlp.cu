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
// the ones row appended to B yields the bias gradient as one more output column.  Each CTA adds
// its tile's gradients to a global FP32 buffer with atomics.
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
    for (int i = threadIdx.x; i < kHid * kIn; i += blockDim.x)
        *reinterpret_cast<__nv_bfloat16*>(sw.w1 + tc::kmajor_offset(i / kIn, i % kIn, kIn)) = WB[OFFB_W1 + i];
    for (int i = threadIdx.x; i < kHid * kHid; i += blockDim.x) {
        *reinterpret_cast<__nv_bfloat16*>(sw.w2 + tc::kmajor_offset(i / kHid, i % kHid, kHid)) = WB[OFFB_W2 + i];
        *reinterpret_cast<__nv_bfloat16*>(sw.w3 + tc::kmajor_offset(i / kHid, i % kHid, kHid)) = WB[OFFB_W3 + i];
    }
    for (int i = threadIdx.x; i < kHid; i += blockDim.x) {
        sw.b1[i] = P[OFF_B1 + i];
        sw.b2[i] = P[OFF_B2 + i];
        sw.b3[i] = P[OFF_B3 + i];
        sw.w4[i] = P[OFF_W4 + i];
    }
    if (threadIdx.x == 0) sw.b4 = P[OFF_B4];
}

// Loads the 16 bf16 features of sample `row` (zeros past n) into the calling thread's row of a
// 128 x 16 K-major tile.
__device__ __forceinline__ void load_x_row(uint8_t* sx, const __nv_bfloat16* __restrict__ X, int row, int n, int r) {
    uint4 a = make_uint4(0, 0, 0, 0), b = a;
    if (row < n) {
        const uint4* src = reinterpret_cast<const uint4*>(X + (size_t)row * kIn);
        a = src[0];
        b = src[1];
    }
    *reinterpret_cast<uint4*>(sx + tc::kmajor_offset(r, 0, kIn)) = a;
    *reinterpret_cast<uint4*>(sx + tc::kmajor_offset(r, 8, kIn)) = b;
}

// Epilogue of a hidden layer: 64 accumulator columns of this thread's TMEM lane + bias, ReLU.
__device__ __forceinline__ void epilogue_relu(uint32_t t_row, const float* bias, float* h) {
#pragma unroll
    for (int c = 0; c < kHid; c += 16) {
        tc::tmem_ld16(t_row + c, h + c);
#pragma unroll
        for (int j = 0; j < 16; ++j) h[c + j] = fmaxf(h[c + j] + bias[c + j], 0.0f);
    }
}

// Stores 64 activations of row r as bf16 into a 128 x 64 K-major tile.
__device__ __forceinline__ void store_row64(uint8_t* s, int r, const float* h) {
#pragma unroll
    for (int c = 0; c < kHid; c += 8) *reinterpret_cast<uint4*>(s + tc::kmajor_offset(r, c, kHid)) = tc::pack8_bf16(h + c);
}

// Stores 64 values of row r transposed (element [c][r]) as bf16 into an R x 128 K-major tile.
__device__ __forceinline__ void store_col64(uint8_t* s, int r, const float* h) {
#pragma unroll
    for (int c = 0; c < kHid; ++c)
        *reinterpret_cast<__nv_bfloat16*>(s + tc::kmajor_offset(c, r, 128)) = __float2bfloat16_rn(h[c]);
}

// ------------------------------------------------------------------------------ inference

struct InferSmem {
    SmemWeights w;
    alignas(128) uint8_t x[128 * kIn * 2];
    alignas(128) uint8_t h[128 * kHid * 2];
    uint64_t bar;
    uint32_t tslot;
};

__global__ void __launch_bounds__(128, 4) infer_kernel(const __nv_bfloat16* __restrict__ X, int n,
                                                       const unsigned int* __restrict__ n_dev,
                                                       const float* __restrict__ P, const __nv_bfloat16* __restrict__ WB,
                                                       float* __restrict__ Y, int* status) {
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
    float h[kHid];
    for (int tile = blockIdx.x; tile * 128 < n && !failed; tile += gridDim.x) {
        const int row = tile * 128 + tid;
        load_x_row(S.x, X, row, n, tid);
        for (int layer = 0; layer < 3; ++layer) {
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
            epilogue_relu(t_row, layer == 0 ? S.w.b1 : (layer == 1 ? S.w.b2 : S.w.b3), h);
            if (layer < 2) store_row64(S.h, tid, h);
        }
        if (failed) break;
        float z = S.w.b4;
#pragma unroll
        for (int j = 0; j < kHid; ++j) z += h[j] * S.w.w4[j];
        if (row < n) Y[row] = 1.0f / (1.0f + __expf(-z));
    }
    if (failed && tid == 0) atomicExch(status, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(taddr, 64);
}

// ------------------------------------------------------------------------------ training

struct TrainSmem {
    SmemWeights w;
    alignas(128) uint8_t w2t[kHid * kHid * 2];    // B of d1 = d2 W2b: [in][out]
    alignas(128) uint8_t w3t[kHid * kHid * 2];    // B of d2 = d3 W3b
    alignas(128) uint8_t x[128 * kIn * 2];        // A of layer 1
    alignas(128) uint8_t xt[32 * 128 * 2];        // B of dW1: rows 0..15 x^T, row 16 ones, rest zero
    alignas(128) uint8_t h1[128 * kHid * 2];      // A of layer 2 (and ReLU mask of layer 1)
    alignas(128) uint8_t h2[128 * kHid * 2];      // A of layer 3 (and ReLU mask of layer 2)
    alignas(128) uint8_t h1t[80 * 128 * 2];       // B of dW2: rows 0..63 h1^T, row 64 ones, rest zero
    alignas(128) uint8_t h2t[80 * 128 * 2];       // B of dW3
    alignas(128) uint8_t d[128 * kHid * 2];       // A of the d_{l-1} GEMM
    alignas(128) uint8_t dt[128 * 128 * 2];       // A of dW: rows 0..63 d^T, rows 64..127 zero
    uint64_t bar;
    uint32_t tslot;
};

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Adds the weight gradient tile of layer l (TMEM columns [col, col + n_in] of lanes 0..63, the
// last one the bias) to the global gradient buffer.  Run by warps 0 and 1.
__device__ __forceinline__ void flush_dw(uint32_t t_row, int o, int n_in, float* G, int off_w, int off_b) {
    float v[16];
    for (int c = 0; c < n_in + 16; c += 16) {
        tc::tmem_ld16(t_row + c, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int i = c + j;
            if (i < n_in)
                atomicAdd(G + off_w + o * n_in + i, v[j]);
            else if (i == n_in)
                atomicAdd(G + off_b + o, v[j]);
        }
    }
}

// Writes row r of a delta: row layout (A of the next delta GEMM) and transposed (A of dW).
__device__ __forceinline__ void store_delta(TrainSmem& S, int r, const float* d) {
    store_row64(S.d, r, d);
    store_col64(S.dt, r, d);
}

__global__ void __launch_bounds__(128, 1) train_kernel(const __nv_bfloat16* __restrict__ X, const float* __restrict__ T,
                                                       int n, int tile0, int tiles, float inv_batch,
                                                       const float* __restrict__ P,
                                                       const __nv_bfloat16* __restrict__ WB, float* __restrict__ G,
                                                       float* __restrict__ loss, int* status) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    load_weights(S.w, P, WB);
    for (int i = tid; i < kHid * kHid; i += 128) {
        const int o = i / kHid, in = i % kHid;
        *reinterpret_cast<__nv_bfloat16*>(S.w2t + tc::kmajor_offset(in, o, kHid)) = WB[OFFB_W2 + i];
        *reinterpret_cast<__nv_bfloat16*>(S.w3t + tc::kmajor_offset(in, o, kHid)) = WB[OFFB_W3 + i];
    }
    // Padding rows of the transposed operands: ones rows give bias gradients, the rest stay zero.
    {
        const __nv_bfloat16 one = __float2bfloat16_rn(1.0f), zero = __float2bfloat16_rn(0.0f);
        for (int i = tid; i < 16 * 128; i += 128) {
            const int rr = 16 + i / 128, k = i % 128;
            *reinterpret_cast<__nv_bfloat16*>(S.xt + tc::kmajor_offset(rr, k, 128)) = rr == 16 ? one : zero;
        }
        for (int i = tid; i < 16 * 128; i += 128) {
            const int rr = 64 + i / 128, k = i % 128;
            *reinterpret_cast<__nv_bfloat16*>(S.h1t + tc::kmajor_offset(rr, k, 128)) = rr == 64 ? one : zero;
            *reinterpret_cast<__nv_bfloat16*>(S.h2t + tc::kmajor_offset(rr, k, 128)) = rr == 64 ? one : zero;
        }
        for (int i = tid; i < 64 * 128; i += 128)
            *reinterpret_cast<__nv_bfloat16*>(S.dt + tc::kmajor_offset(64 + i / 128, i % 128, 128)) = zero;
    }
    if (tid == 0) tc::mbar_init(&S.bar, 1);
    if (warp == 0) tc::tmem_alloc(&S.tslot, 256);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = S.tslot;
    const uint32_t lane_off = (uint32_t)(warp * 32) << 16;
    const uint32_t tA = taddr, tB = taddr + 128;  // activations / deltas; weight gradients
    uint32_t phase = 0;
    bool failed = false;
    float acc_dw4[kHid];
#pragma unroll
    for (int j = 0; j < kHid; ++j) acc_dw4[j] = 0.0f;
    float acc_db4 = 0.0f, acc_loss = 0.0f;

    auto sync_mma = [&]() {
        tc::fence_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
    };
    auto wait_mma = [&]() -> bool {
        const bool ok = tc::mbar_wait(&S.bar, phase);
        phase ^= 1u;
        if (__syncthreads_or(!ok)) return false;
        tc::fence_after_sync();
        return true;
    };

    for (int tile = tile0 + blockIdx.x; tile < tile0 + tiles && !failed; tile += gridDim.x) {
        const int row = tile * 128 + tid;
        const bool valid = row < n;
        // ---- forward
        load_x_row(S.x, X, row, n, tid);
        {
            const __nv_bfloat16* xr = X + (size_t)row * kIn;
#pragma unroll
            for (int c = 0; c < kIn; ++c)
                *reinterpret_cast<__nv_bfloat16*>(S.xt + tc::kmajor_offset(c, tid, 128)) =
                    valid ? xr[c] : __float2bfloat16_rn(0.0f);
        }
        float h[kHid];
        for (int layer = 0; layer < 3; ++layer) {
            sync_mma();
            if (tid == 0) {
                if (layer == 0)
                    tc::gemm_issue(tA, tc::smem_u32(S.x), tc::smem_u32(S.w.w1), kIn, kHid, &S.bar);
                else
                    tc::gemm_issue(tA, tc::smem_u32(layer == 1 ? S.h1 : S.h2), tc::smem_u32(layer == 1 ? S.w.w2 : S.w.w3),
                                   kHid, kHid, &S.bar);
            }
            if (!wait_mma()) {
                failed = true;
                break;
            }
            epilogue_relu(tA + lane_off, layer == 0 ? S.w.b1 : (layer == 1 ? S.w.b2 : S.w.b3), h);
            if (layer == 0) {
                store_row64(S.h1, tid, h);
                store_col64(S.h1t, tid, h);
            } else if (layer == 1) {
                store_row64(S.h2, tid, h);
                store_col64(S.h2t, tid, h);
            }
        }
        if (failed) break;
        // ---- output layer and loss (CUDA cores)
        float z = S.w.b4;
#pragma unroll
        for (int j = 0; j < kHid; ++j) z += h[j] * S.w.w4[j];
        const float y = 1.0f / (1.0f + expf(-z));
        const float err = valid ? y - T[row] : 0.0f;
        const float dz = 2.0f * err * y * (1.0f - y) * inv_batch;
        acc_loss += err * err;
        acc_db4 += dz;
        float d[kHid];
#pragma unroll
        for (int j = 0; j < kHid; ++j) {
            acc_dw4[j] += dz * h[j];
            d[j] = h[j] > 0.0f ? dz * S.w.w4[j] : 0.0f;
        }
        // ---- layers 3, 2, 1
        for (int l = 3; l >= 1 && !failed; --l) {
            store_delta(S, tid, d);
            sync_mma();
            if (tid == 0) {
                const uint32_t sdt = tc::smem_u32(S.dt);
                if (l == 3) tc::gemm_mmas(tB, sdt, tc::smem_u32(S.h2t), 128, 80);
                if (l == 2) tc::gemm_mmas(tB, sdt, tc::smem_u32(S.h1t), 128, 80);
                if (l == 1) tc::gemm_mmas(tB, sdt, tc::smem_u32(S.xt), 128, 32);
                if (l > 1) tc::gemm_mmas(tA, tc::smem_u32(S.d), tc::smem_u32(l == 3 ? S.w3t : S.w2t), kHid, kHid);
                tc::mma_commit(&S.bar);
            }
            if (!wait_mma()) {
                failed = true;
                break;
            }
            if (warp < 2) {
                const int o = warp * 32 + lane;
                if (l == 3) flush_dw(tB + lane_off, o, kHid, G, OFF_W3, OFF_B3);
                if (l == 2) flush_dw(tB + lane_off, o, kHid, G, OFF_W2, OFF_B2);
                if (l == 1) flush_dw(tB + lane_off, o, kIn, G, OFF_W1, OFF_B1);
            }
            if (l > 1) {
                const uint8_t* hm = l == 3 ? S.h2 : S.h1;  // ReLU mask of the layer below
#pragma unroll
                for (int c = 0; c < kHid; c += 16) {
                    float v[16];
                    tc::tmem_ld16(tA + lane_off + c, v);
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const float hv = __bfloat162float(
                            *reinterpret_cast<const __nv_bfloat16*>(hm + tc::kmajor_offset(tid, c + j, kHid)));
                        d[c + j] = hv > 0.0f ? v[j] : 0.0f;
                    }
                }
            }
            // the next iteration overwrites S.d / S.dt, which these MMAs read: they have completed
        }
    }
    // ---- output-layer gradients and loss
    for (int j = 0; j < kHid; ++j) {
        const float v = warp_sum(acc_dw4[j]);
        if (lane == 0) atomicAdd(G + OFF_W4 + j, v);
    }
    {
        const float v = warp_sum(acc_db4), l2 = warp_sum(acc_loss);
        if (lane == 0) {
            atomicAdd(G + OFF_B4, v);
            if (loss) atomicAdd(loss, l2);
        }
    }
    if (failed && tid == 0) atomicExch(status, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(taddr, 256);
}

// Adam on the FP32 parameters; refreshes the BF16 copies and clears the gradient buffer.
__global__ void adam_kernel(float* __restrict__ P, __nv_bfloat16* __restrict__ WB, float* __restrict__ G,
                            float* __restrict__ Mo, float* __restrict__ Vo, float lr, float b1, float b2, float eps,
                            float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    const float g = G[i];
    const float m = b1 * Mo[i] + (1.0f - b1) * g;
    const float v = b2 * Vo[i] + (1.0f - b2) * g * g;
    Mo[i] = m;
    Vo[i] = v;
    const float p = P[i] - lr * (m / c1) / (sqrtf(v / c2) + eps);
    P[i] = p;
    G[i] = 0.0f;
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
    float* G = nullptr;          // gradient accumulator (kept zero between steps)
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
    MM_CUDA_TRY(cudaFuncSetAttribute(mm::mlp::infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)infer_smem()));
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

// Runs the training kernel over tiles [tile0, tile0 + tiles) of (X, T) adding into m->G.
int run_train(mm_mlp m, const void* X, const float* T, int n, int tile0, int tiles, float inv_batch, cudaStream_t s) {
    const int grid = tiles < m->num_sms ? tiles : m->num_sms;
    // The shared-memory image needs 1024-byte alignment; the kernel takes the dynamic buffer as is.
    mm::mlp::train_kernel<<<grid, 128, train_smem(), s>>>((const __nv_bfloat16*)X, T, n, tile0, tiles, inv_batch, m->P,
                                                         m->WB, m->G, m->loss, m->status);
    MM_CUDA_TRY(cudaGetLastError());
    mm::count_launch();
    return MM_OK;
}

}  // namespace

namespace mm {

// Inference on up to `cap` samples, the actual count read from device memory (surrogate march).
int mlp_infer_device_count(mm_mlp m, const void* d_x, int cap, const unsigned int* d_count, float* d_y,
                           cudaStream_t s) {
    int r = set_smem_limits();
    if (r) return r;
    const int tiles = (cap + 127) / 128;
    const int grid = tiles < 4 * m->num_sms ? tiles : 4 * m->num_sms;
    mlp::infer_kernel<<<grid, 128, infer_smem(), s>>>((const __nv_bfloat16*)d_x, cap, d_count, m->P, m->WB, d_y,
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
    e = e ? e : cudaMalloc(&m->G, kParams * sizeof(float));
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
    e = e ? e : cudaMemset(m->G, 0, kParams * sizeof(float));
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
    cudaFree(m->G);
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
    const int grid = tiles < 4 * m->num_sms ? tiles : 4 * m->num_sms;
    mm::mlp::infer_kernel<<<grid, 128, infer_smem(), s>>>((const __nv_bfloat16*)d_x, n, nullptr, m->P, m->WB, d_y,
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
    MM_CUDA_TRY(cudaMemsetAsync(m->G, 0, mm::mlp::kParams * sizeof(float), s));
    MM_CUDA_TRY(cudaMemsetAsync(m->loss, 0, sizeof(float), s));
    if ((r = run_train(m, d_x, d_t, n, 0, (n + 127) / 128, 1.0f / (float)n, s))) return r;
    MM_CUDA_TRY(cudaMemcpyAsync(d_grad, m->G, mm::mlp::kParams * sizeof(float), cudaMemcpyDeviceToDevice, s));
    MM_CUDA_TRY(cudaMemsetAsync(m->G, 0, mm::mlp::kParams * sizeof(float), s));
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
        if (h_loss_history) MM_CUDA_TRY(cudaMemsetAsync(m->loss, 0, sizeof(float), s));
        if ((r = run_train(m, d_x, d_t, n, cursor, tiles, 1.0f / (float)(tiles * 128), s))) return r;
        cursor += tiles;
        m->step += 1;
        const float c1 = 1.0f - powf(b1, (float)m->step), c2 = 1.0f - powf(b2, (float)m->step);
        mm::mlp::adam_kernel<<<(mm::mlp::kParams + 255) / 256, 256, 0, s>>>(m->P, m->WB, m->G, m->M, m->V, lr, b1, b2,
                                                                           eps, c1, c2);
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
