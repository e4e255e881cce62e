// The learned return-map closure: a 14 -> 64 -> 64 -> 7 MLP with ReLU, BF16
// weights and activations, FP32 accumulation.  Training and the standalone
// forward pass run on tcgen05 MMAs with TMEM accumulators, 128 samples per
// CTA (des_mlp_tc.cuh).  Inside the FP32 stress pass the network is evaluated
// by one warp per 16 candidates with warp-level MMAs (m16n8k16, BF16 x BF16
// -> FP32, below): there every warp works through its own share of the list of
// undecided elements, and its tiles fill as candidates come.
//
// Shapes (inputs and outputs padded for the 16x16 / 16x8 MMA tiles):
//   x  [rows][16]   14 normalised inputs + 2 zeros
//   W1 [64][16]     layer 1, stored [out][in] (the MMA's column-major B)
//   W2 [64][64]     layer 2
//   W3 [8][64]      layer 3 (7 outputs + 1 zero row)
// One warp evaluates 16 rows: 8 + 32 + 4 MMAs.
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

namespace des {

constexpr int kMlpIn = 16, kMlpHid = 64, kMlpOut = 8;
constexpr int kMlpInUsed = 14, kMlpOutUsed = 7;
constexpr int kHStride = 72;   // padded row stride (bf16) of activation tiles in shared memory

// Parameters of the network as the kernels read them (device memory).
struct MlpDev {
    __nv_bfloat16 w1[kMlpHid * kMlpIn], w2[kMlpHid * kMlpHid], w3[kMlpOut * kMlpHid];
    float b1[kMlpHid], b2[kMlpHid], b3[kMlpOut];
    float in_mean[kMlpIn], in_scale[kMlpIn];     // x = (raw - mean) * scale
    float out_scale[kMlpOut];                    // raw output = y * scale
    float env_lo[kMlpIn], env_hi[kMlpIn];        // training envelope of x
    float tol;                                   // relative yield-residual tolerance
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}
__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16 *p)
{
    return *reinterpret_cast<const uint32_t *>(p);
}
__device__ __forceinline__ uint32_t ld2(const __nv_bfloat16 *p, const __nv_bfloat16 *q)
{
    __nv_bfloat162 v;
    v.x = *p;
    v.y = *q;
    return *reinterpret_cast<uint32_t *>(&v);
}

// D += A (16x16, row-major) * B (16x8, column-major), BF16 in, FP32 accumulate
__device__ __forceinline__ void mma_bf16(float d[4], const uint32_t a[4], const uint32_t b[2])
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// A fragment of rows r0..r0+15, columns k0..k0+15 of a row-major bf16 matrix
// with row stride ld (elements).
__device__ __forceinline__ void frag_a_row(uint32_t a[4], const __nv_bfloat16 *M, int ld, int r0, int k0)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    a[0] = ld32(M + (r0 + g) * ld + k0 + 2 * t);
    a[1] = ld32(M + (r0 + g + 8) * ld + k0 + 2 * t);
    a[2] = ld32(M + (r0 + g) * ld + k0 + 8 + 2 * t);
    a[3] = ld32(M + (r0 + g + 8) * ld + k0 + 8 + 2 * t);
}
// B fragment (k0..k0+15) x (n0..n0+7) of a matrix stored [n][k] with row stride ld
__device__ __forceinline__ void frag_b_nk(uint32_t b[2], const __nv_bfloat16 *W, int ld, int k0, int n0)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    b[0] = ld32(W + (n0 + g) * ld + k0 + 2 * t);
    b[1] = ld32(W + (n0 + g) * ld + k0 + 8 + 2 * t);
}
// general strided fragments (element (r, c) at M[r * rs + c * cs]); used by the
// backward pass, where operands are transposed views
__device__ __forceinline__ void frag_a_gen(uint32_t a[4], const __nv_bfloat16 *M, int rs, int cs, int r0,
                                           int k0)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int ra = r0 + g, rb = r0 + g + 8, ka = k0 + 2 * t, kb = k0 + 8 + 2 * t;
    a[0] = ld2(M + ra * rs + ka * cs, M + ra * rs + (ka + 1) * cs);
    a[1] = ld2(M + rb * rs + ka * cs, M + rb * rs + (ka + 1) * cs);
    a[2] = ld2(M + ra * rs + kb * cs, M + ra * rs + (kb + 1) * cs);
    a[3] = ld2(M + rb * rs + kb * cs, M + rb * rs + (kb + 1) * cs);
}
// B element (k, n) at M[k * ks + n * ns]
__device__ __forceinline__ void frag_b_gen(uint32_t b[2], const __nv_bfloat16 *M, int ks, int ns, int k0,
                                           int n0)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int n = n0 + g, ka = k0 + 2 * t, kb = k0 + 8 + 2 * t;
    b[0] = ld2(M + ka * ks + n * ns, M + (ka + 1) * ks + n * ns);
    b[1] = ld2(M + kb * ks + n * ns, M + (kb + 1) * ks + n * ns);
}

// bias + ReLU on an accumulator fragment of columns n0..n0+7, stored as bf16
// rows r0..r0+15 of H (row stride kHStride)
__device__ __forceinline__ void store_relu(const float d[4], const float *bias, __nv_bfloat16 *H, int r0,
                                           int n0)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int c = n0 + 2 * t;
    float v0 = fmaxf(d[0] + bias[c], 0.f), v1 = fmaxf(d[1] + bias[c + 1], 0.f);
    float v2 = fmaxf(d[2] + bias[c], 0.f), v3 = fmaxf(d[3] + bias[c + 1], 0.f);
    *reinterpret_cast<uint32_t *>(H + (r0 + g) * kHStride + c) = pack_bf16(v0, v1);
    *reinterpret_cast<uint32_t *>(H + (r0 + g + 8) * kHStride + c) = pack_bf16(v2, v3);
}

// Forward pass of 16 rows by one warp.  X: [16][16] bf16 rows at X + r0*16;
// H1, H2: [16][kHStride] per-warp scratch; Y: [16][8] fp32 outputs (biased).
// W*: bf16 weights (shared or global), b*: fp32 biases.
__device__ __forceinline__ void mlp_forward16(const __nv_bfloat16 *X, const __nv_bfloat16 *W1,
                                              const __nv_bfloat16 *W2, const __nv_bfloat16 *W3,
                                              const float *b1, const float *b2, const float *b3,
                                              __nv_bfloat16 *H1, __nv_bfloat16 *H2, float *Y)
{
    uint32_t a[4], b[2];
    frag_a_row(a, X, kMlpIn, 0, 0);
#pragma unroll
    for (int nt = 0; nt < kMlpHid / 8; ++nt) {
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        frag_b_nk(b, W1, kMlpIn, 0, nt * 8);
        mma_bf16(d, a, b);
        store_relu(d, b1, H1, 0, nt * 8);
    }
    __syncwarp();
    uint32_t a2[4][4];
#pragma unroll
    for (int kt = 0; kt < kMlpHid / 16; ++kt) frag_a_row(a2[kt], H1, kHStride, 0, kt * 16);
#pragma unroll
    for (int nt = 0; nt < kMlpHid / 8; ++nt) {
        float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int kt = 0; kt < kMlpHid / 16; ++kt) {
            frag_b_nk(b, W2, kMlpHid, kt * 16, nt * 8);
            mma_bf16(d, a2[kt], b);
        }
        store_relu(d, b2, H2, 0, nt * 8);
    }
    __syncwarp();
    float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int kt = 0; kt < kMlpHid / 16; ++kt) {
        frag_a_row(a, H2, kHStride, 0, kt * 16);
        frag_b_nk(b, W3, kMlpHid, kt * 16, 0);
        mma_bf16(d, a, b);
    }
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    Y[g * kMlpOut + 2 * t] = d[0] + b3[2 * t];
    Y[g * kMlpOut + 2 * t + 1] = d[1] + b3[2 * t + 1];
    Y[(g + 8) * kMlpOut + 2 * t] = d[2] + b3[2 * t];
    Y[(g + 8) * kMlpOut + 2 * t + 1] = d[3] + b3[2 * t + 1];
    __syncwarp();
}

}  // namespace des
