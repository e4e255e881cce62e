// The learned closure's network (14 -> 64 -> 64 -> 7, des_mlp.cuh) on the
// fifth-generation tensor cores: CTAs of 128 threads over tiles of 128
// samples (persistent: a CTA takes every gridDim.x-th tile), BF16 operands in shared memory (K-major, no swizzle, des_tc.cuh),
// FP32 accumulators in tensor memory, every MMA issued by one thread and
// committed to an mbarrier; the other threads move data between TMEM and
// shared memory (tcgen05.ld, one sample per thread: TMEM lane = sample).
//
// Forward (M = 128 samples):
//   D1 = X W1^T (K 16, N 64)   -> H1 = relu(D1 + b1)
//   D2 = H1 W2^T (K 64, N 64)  -> H2 = relu(D2 + b2)
//   D3 = H2 W3^T (K 64, N 16)  -> Y = D3 + b3 (7 of 16 columns)
// Backward (loss = mean over the batch of the summed squared error):
//   dY = 2 (Y - T) / count
//   dH2 = (dY W3) . [H2 > 0]          (K 16, N 64)
//   dW3^T = H2^T dY, db3 = 1^T dY      (M = 64 hidden + a row of ones, K = 128 samples)
//   dH1 = (dH2 W2) . [H1 > 0]          (K 64, N 64)
//   [dW2 | . | db2] and [. | dW1 | db1] = [dH2^T ; dH1^T] [H1^T ; X^T ; 1]^T
//                                        (M = 128, N = 96, K = 128 samples)
// The last product forms both weight gradients and the bias gradients (the
// row of ones) in one chain of MMAs; its off-diagonal blocks are not used.
// TMEM columns (256 allocated): D1 / dH2 0-63, D2 / dH1 64-127, D3 128-143,
// weight gradients 144-239, dW3^T 240-255.
#pragma once

#include <cuda_bf16.h>
#include <cstddef>

#include "des_mlp.cuh"
#include "des_tc.cuh"

namespace des {

constexpr int kTcRows = 128;
constexpr uint32_t kTcCols = 256;

struct MlpTcSmem {
    alignas(1024) unsigned char x[kTcRows * 16 * 2];      // A of D1        [128][16]
    alignas(1024) unsigned char w1[64 * 16 * 2];          // B of D1        [64][16]
    alignas(1024) unsigned char w2[64 * 64 * 2];          // B of D2        [64 out][64 in]
    alignas(1024) unsigned char w3[16 * 64 * 2];          // B of D3        [16 out][64]
    alignas(1024) unsigned char h1[kTcRows * 64 * 2];     // A of D2        [128][64]
    alignas(1024) unsigned char h2[kTcRows * 64 * 2];     // A of D3        [128][64]
    alignas(1024) unsigned char w3t[64 * 16 * 2];         // B of dH2       [64 hidden][16 out]
    alignas(1024) unsigned char w2t[64 * 64 * 2];         // B of dH1       [64 in][64 out]
    alignas(1024) unsigned char dy[kTcRows * 16 * 2];     // A of dH2       [128][16]
    alignas(1024) unsigned char dyt[16 * kTcRows * 2];    // B of dW3^T     [16 out][128]
    alignas(1024) unsigned char h2t[128 * kTcRows * 2];   // A of dW3^T     [H2^T; 1; 0][128]
    alignas(1024) unsigned char dh2[kTcRows * 64 * 2];    // A of dH1       [128][64]
    alignas(1024) unsigned char ag[128 * kTcRows * 2];    // A of the gradients [dH2^T; dH1^T][128]
    alignas(1024) unsigned char bg[96 * kTcRows * 2];     // B of the gradients [H1^T; X^T; 1; 0][128]
    float b1[64], b2[64], b3[16];
    uint64_t bar;
    uint32_t tmem;
};

// bytes of dynamic shared memory a launch asks for (the struct plus room to
// align its start to 1024 bytes)
constexpr size_t kMlpTcSmemBytes = sizeof(MlpTcSmem) + 1024;

namespace mlptc {

__device__ __forceinline__ void put_bf16(unsigned char *tile, int r, int k, int K, float v)
{
    *reinterpret_cast<__nv_bfloat16 *>(tile + tc::kmajor_offset(r, k, K)) = __float2bfloat16(v);
}
__device__ __forceinline__ float get_bf16(const unsigned char *tile, int r, int k, int K)
{
    return __bfloat162float(*reinterpret_cast<const __nv_bfloat16 *>(tile + tc::kmajor_offset(r, k, K)));
}
// eight consecutive columns k0..k0+7 of row r (16 bytes, one store)
__device__ __forceinline__ void put8(unsigned char *tile, int r, int k0, int K, const float *v)
{
    uint4 q;
    q.x = pack_bf16(v[0], v[1]);
    q.y = pack_bf16(v[2], v[3]);
    q.z = pack_bf16(v[4], v[5]);
    q.w = pack_bf16(v[6], v[7]);
    *reinterpret_cast<uint4 *>(tile + tc::kmajor_offset(r, k0, K)) = q;
}

// descriptor of the 16-column slice kk of a K-major tile with K columns
__device__ __forceinline__ uint64_t desc(const unsigned char *tile, int K, int kk)
{
    return tc::smem_desc(tc::smem_addr(tile) + 256u * (uint32_t)kk, 128u, (uint32_t)(16 * K));
}

// D[tmem col] = A B^T over K (K / 16 MMAs), or D += A B^T with accumulate,
// then (with commit_now) a commit
__device__ __forceinline__ void gemm(uint32_t d, const unsigned char *A, const unsigned char *B, int K, int N,
                                     uint64_t *bar, bool commit_now, bool accumulate = false)
{
    const uint32_t id = tc::idesc_bf16(kTcRows, N);
    for (int kk = 0; kk < K / 16; ++kk) tc::mma_bf16(d, desc(A, K, kk), desc(B, K, kk), id, accumulate || kk > 0);
    if (commit_now) tc::commit(bar);
}

// all threads: shared-memory operands written, TMEM reads done -> MMAs may run
__device__ __forceinline__ void hand_to_tensor_cores()
{
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
}

// all threads: wait for the k-th commit; false (in every thread) on a time-out
__device__ __forceinline__ bool wait_commit(uint64_t *bar, int k)
{
    const bool ok = tc::mbar_wait(bar, (uint32_t)(k & 1));
    tc::fence_after_sync();
    return !__syncthreads_or(!ok);
}

// offsets of the parameter groups in the flat FP32 vector (des_mlp.cu's layout)
constexpr int oW1 = 0, oB1 = 64 * 16, oW2 = oB1 + 64, oB2 = oW2 + 64 * 64, oW3 = oB2 + 64,
              oB3 = oW3 + 8 * 64;

}  // namespace mlptc

// flat FP32 parameters (w1 [64][16], b1, w2 [64][64], b2, w3 [8][64], b3) ->
// the shared-memory tiles; every other tile zeroed
__device__ __forceinline__ void mlptc_load(MlpTcSmem &S, const float *P, bool backward)
{
    using namespace mlptc;
    {
        uint4 *z = reinterpret_cast<uint4 *>(&S);
        const int n = (int)(offsetof(MlpTcSmem, b1) / sizeof(uint4));
        for (int i = threadIdx.x; i < n; i += blockDim.x) z[i] = make_uint4(0, 0, 0, 0);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 64 * 16; i += blockDim.x) put_bf16(S.w1, i / 16, i % 16, 16, P[oW1 + i]);
    for (int i = threadIdx.x; i < 64 * 64; i += blockDim.x) {
        const float v = P[oW2 + i];
        put_bf16(S.w2, i / 64, i % 64, 64, v);
        if (backward) put_bf16(S.w2t, i % 64, i / 64, 64, v);
    }
    for (int i = threadIdx.x; i < kMlpOutUsed * 64; i += blockDim.x) {
        const float v = P[oW3 + i];
        put_bf16(S.w3, i / 64, i % 64, 64, v);
        if (backward) put_bf16(S.w3t, i % 64, i / 64, 16, v);
    }
    for (int i = threadIdx.x; i < 64; i += blockDim.x) {
        S.b1[i] = P[oB1 + i];
        S.b2[i] = P[oB2 + i];
    }
    for (int i = threadIdx.x; i < 16; i += blockDim.x) S.b3[i] = i < kMlpOutUsed ? P[oB3 + i] : 0.f;
    if (backward)
        for (int r = threadIdx.x; r < kTcRows; r += blockDim.x) {
            put_bf16(S.h2t, 64, r, kTcRows, 1.f);      // db3 = 1^T dY
            put_bf16(S.bg, 80, r, kTcRows, 1.f);       // db2, db1 = [dH2^T; dH1^T] 1
        }
}

// Tiles k = blockIdx.x, blockIdx.x + gridDim.x, ... (< ntiles) of 128
// samples from row_begin, by one CTA of 128 threads: the forward pass,
// writing y_out [n][8]; with BACKWARD instead the loss (added to *loss) and
// the gradient (added to grad, the flat FP32 layout of P).  The weights are
// staged once per CTA; the weight and bias gradients accumulate in TMEM over
// the CTA's tiles and are added to grad with one atomic per parameter per
// CTA at the end.  Returns false after a tensor-core wait timed out; TMEM is
// released either way.
template <bool BACKWARD>
__device__ bool mlptc_tiles(MlpTcSmem &S, const float *P, const float *x, const float *yt, long long n,
                            long long row_begin, long long ntiles, float inv_count, float *y_out, float *grad,
                            double *loss)
{
    using namespace mlptc;
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    const uint32_t lane_base = (uint32_t)(32 * w) << 16;
    if (w == 0) tc::tmem_alloc(&S.tmem, kTcCols);
    if (t == 0) tc::mbar_init(&S.bar, 1);
    mlptc_load(S, P, BACKWARD);
    const uint32_t tm = S.tmem;
    int phase = 0;
    bool ok = true, first = true;
    // this thread's sample of a tile: inputs and (BACKWARD) targets, loaded one
    // tile ahead so that the loads run under the previous tile's MMAs
    float xn[16], yn[kMlpOut] = {};
    auto fetch = [&](long long tile) {
        const long long r = row_begin + tile * kTcRows + t;
        const bool v = tile < ntiles && r < n;
        for (int k = 0; k < 16; ++k) xn[k] = v ? x[r * kMlpIn + k] : 0.f;
        if (BACKWARD)
            for (int j = 0; j < kMlpOut; ++j) yn[j] = v ? yt[r * kMlpOut + j] : 0.f;
    };
    fetch(blockIdx.x);
    for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, first = false) {
        const long long row = row_begin + tile * kTcRows + t;
        const bool valid = row < n;
        float ycur[kMlpOut];
        {
            float v[16];
            for (int k = 0; k < 16; ++k) v[k] = xn[k];
            for (int j = 0; j < kMlpOut; ++j) ycur[j] = yn[j];
            put8(S.x, t, 0, 16, v);
            put8(S.x, t, 8, 16, v + 8);
            if (BACKWARD)
                for (int k = 0; k < 16; ++k) put_bf16(S.bg, 64 + k, t, kTcRows, v[k]);
        }
        fetch(tile + gridDim.x);
        hand_to_tensor_cores();

        // H1 = relu(X W1^T + b1)
        if (t == 0) gemm(tm + 0, S.x, S.w1, 16, 64, &S.bar, true);
        ok = wait_commit(&S.bar, phase++);
        if (ok)
            for (int c = 0; c < 64; c += 16) {
                float v[16];
                tc::tmem_ld16(tm + lane_base + c, v);
                for (int i = 0; i < 16; ++i) v[i] = fmaxf(v[i] + S.b1[c + i], 0.f);
                put8(S.h1, t, c, 64, v);
                put8(S.h1, t, c + 8, 64, v + 8);
                if (BACKWARD)
                    for (int i = 0; i < 16; ++i) put_bf16(S.bg, c + i, t, kTcRows, v[i]);
            }
        hand_to_tensor_cores();
        // H2 = relu(H1 W2^T + b2)
        if (ok) {
            if (t == 0) gemm(tm + 64, S.h1, S.w2, 64, 64, &S.bar, true);
            ok = wait_commit(&S.bar, phase++);
        }
        if (ok)
            for (int c = 0; c < 64; c += 16) {
                float v[16];
                tc::tmem_ld16(tm + lane_base + 64 + c, v);
                for (int i = 0; i < 16; ++i) v[i] = fmaxf(v[i] + S.b2[c + i], 0.f);
                put8(S.h2, t, c, 64, v);
                put8(S.h2, t, c + 8, 64, v + 8);
                if (BACKWARD)
                    for (int i = 0; i < 16; ++i) put_bf16(S.h2t, c + i, t, kTcRows, v[i]);
            }
        hand_to_tensor_cores();
        // Y = H2 W3^T + b3
        if (ok) {
            if (t == 0) gemm(tm + 128, S.h2, S.w3, 64, 16, &S.bar, true);
            ok = wait_commit(&S.bar, phase++);
        }
        if (ok) {
            float v[16];
            tc::tmem_ld16(tm + lane_base + 128, v);
            for (int j = 0; j < 16; ++j) v[j] = j < kMlpOutUsed ? v[j] + S.b3[j] : 0.f;
            if (!BACKWARD) {
                if (valid)
                    for (int j = 0; j < kMlpOut; ++j) y_out[row * kMlpOut + j] = v[j];
            } else {
                double l = 0.0;
                float g[16];
                for (int j = 0; j < 16; ++j) {
                    const float e = (valid && j < kMlpOutUsed) ? v[j] - ycur[j] : 0.f;
                    l += (double)e * e;
                    g[j] = 2.f * e * inv_count;
                }
                put8(S.dy, t, 0, 16, g);
                for (int j = 0; j < kMlpOutUsed; ++j) put_bf16(S.dyt, j, t, kTcRows, g[j]);
                for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
                if (lane == 0) atomicAdd(loss, l * inv_count);
            }
        }
        if (BACKWARD) {
            hand_to_tensor_cores();
            // dH2 (before the mask) and dW3^T, db3 (accumulated over the tiles)
            if (ok) {
                if (t == 0) {
                    gemm(tm + 0, S.dy, S.w3t, 16, 64, &S.bar, false);
                    gemm(tm + 240, S.h2t, S.dyt, kTcRows, 16, &S.bar, true, !first);
                }
                ok = wait_commit(&S.bar, phase++);
            }
            if (ok)
                for (int c = 0; c < 64; c += 16) {
                    float v[16];
                    tc::tmem_ld16(tm + lane_base + c, v);
                    for (int i = 0; i < 16; ++i) v[i] = get_bf16(S.h2, t, c + i, 64) > 0.f ? v[i] : 0.f;
                    put8(S.dh2, t, c, 64, v);
                    put8(S.dh2, t, c + 8, 64, v + 8);
                    for (int i = 0; i < 16; ++i) put_bf16(S.ag, c + i, t, kTcRows, v[i]);
                }
            hand_to_tensor_cores();
            // dH1 (before the mask)
            if (ok) {
                if (t == 0) gemm(tm + 64, S.dh2, S.w2t, 64, 64, &S.bar, true);
                ok = wait_commit(&S.bar, phase++);
            }
            if (ok)
                for (int c = 0; c < 64; c += 16) {
                    float v[16];
                    tc::tmem_ld16(tm + lane_base + 64 + c, v);
                    for (int i = 0; i < 16; ++i) {
                        const float h = get_bf16(S.h1, t, c + i, 64);
                        put_bf16(S.ag, 64 + c + i, t, kTcRows, h > 0.f ? v[i] : 0.f);
                    }
                }
            hand_to_tensor_cores();
            // [dW2 | . | db2] over lanes 0-63, [. | dW1 | db1] over lanes 64-127
            // (accumulated over the tiles)
            if (ok) {
                if (t == 0) gemm(tm + 144, S.ag, S.bg, kTcRows, 96, &S.bar, true, !first);
                ok = wait_commit(&S.bar, phase++);
            }
        }
    }
    if (BACKWARD && ok && !first) {
        const int m = t;                       // this thread's TMEM lane
        float v[16];
        if (w < 2) {
            for (int c = 0; c < 64; c += 16) {
                tc::tmem_ld16(tm + lane_base + 144 + c, v);
                for (int i = 0; i < 16; ++i) atomicAdd(grad + oW2 + m * 64 + c + i, v[i]);
            }
            tc::tmem_ld16(tm + lane_base + 144 + 80, v);
            atomicAdd(grad + oB2 + m, v[0]);
            tc::tmem_ld16(tm + lane_base + 240, v);            // row m of dW3^T
            for (int j = 0; j < kMlpOutUsed; ++j) atomicAdd(grad + oW3 + j * 64 + m, v[j]);
        } else {
            tc::tmem_ld16(tm + lane_base + 144 + 64, v);
            for (int i = 0; i < 16; ++i) atomicAdd(grad + oW1 + (m - 64) * 16 + i, v[i]);
            tc::tmem_ld16(tm + lane_base + 144 + 80, v);
            atomicAdd(grad + oB1 + (m - 64), v[0]);
            tc::tmem_ld16(tm + lane_base + 240, v);            // lane 64: db3
            if (m == 64)
                for (int j = 0; j < kMlpOutUsed; ++j) atomicAdd(grad + oB3 + j, v[j]);
        }
    }
    // after a time-out, give the MMAs of that phase one more bounded wait
    // before their TMEM is released
    if (!ok) tc::mbar_wait(&S.bar, (uint32_t)((phase - 1) & 1));
    tc::fence_before_sync();
    __syncthreads();
    if (w == 0) tc::tmem_dealloc(tm, kTcCols);
    return ok;
}

}  // namespace des
