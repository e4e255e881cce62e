// Training and standalone evaluation of the learned return-map closure
// (see des_mlp.cuh for the network).  Forward and backward passes run on the
// tensor cores (BF16 operands, FP32 accumulation); Adam keeps FP32 master
// weights and moments and writes the BF16 copies the MMAs read.
//
// Per CTA: one tile of 64 samples (4 warps x 16 rows).  Backward GEMMs:
//   dW3 = dY^T H2, dH2 = (dY W3) * [H2 > 0], dW2 = dH2^T H1,
//   dH1 = (dH2 W2) * [H1 > 0], dW1 = dH1^T X, biases = column sums;
// every partial gradient of the tile is added to the global FP32 gradient
// with atomics (one add per parameter per tile).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "des_gpu.h"
#include "des_mlp.cuh"

using namespace des;

namespace {

constexpr int kTile = 64;                    // samples per CTA
constexpr int kNW1 = kMlpHid * kMlpIn, kNW2 = kMlpHid * kMlpHid, kNW3 = kMlpOut * kMlpHid;
constexpr int kNParams = kNW1 + kMlpHid + kNW2 + kMlpHid + kNW3 + kMlpOut;   // 5,768
// offsets of the parameter groups in a flat FP32 vector
constexpr int kOW1 = 0, kOB1 = kOW1 + kNW1, kOW2 = kOB1 + kMlpHid, kOB2 = kOW2 + kNW2,
              kOW3 = kOB2 + kMlpHid, kOB3 = kOW3 + kNW3;

struct TrainSmem {
    __nv_bfloat16 x[kTile * kMlpIn];
    __nv_bfloat16 h1[kTile * kHStride], h2[kTile * kHStride];
    __nv_bfloat16 dh1[kTile * kHStride], dh2[kTile * kHStride];
    __nv_bfloat16 dy[kTile * 16];
    float y[kTile * kMlpOut];
    __nv_bfloat16 w1[kNW1], w2[kNW2], w3p[16 * kMlpHid];
    float b1[kMlpHid], b2[kMlpHid], b3[kMlpOut];
};

// flat FP32 parameters -> the BF16/FP32 arrays a CTA keeps in shared memory
__device__ void load_params(TrainSmem &S, const float *P)
{
    for (int i = threadIdx.x; i < kNW1; i += blockDim.x) S.w1[i] = __float2bfloat16(P[kOW1 + i]);
    for (int i = threadIdx.x; i < kNW2; i += blockDim.x) S.w2[i] = __float2bfloat16(P[kOW2 + i]);
    for (int i = threadIdx.x; i < 16 * kMlpHid; i += blockDim.x)
        S.w3p[i] = __float2bfloat16(i < kNW3 ? P[kOW3 + i] : 0.f);
    for (int i = threadIdx.x; i < kMlpHid; i += blockDim.x) {
        S.b1[i] = P[kOB1 + i];
        S.b2[i] = P[kOB2 + i];
    }
    for (int i = threadIdx.x; i < kMlpOut; i += blockDim.x) S.b3[i] = P[kOB3 + i];
}

// loads rows [row0, row0 + 64) of x (FP32 [n][16]) as bf16, zero rows past n
__device__ void load_x(TrainSmem &S, const float *x, long long n, long long row0)
{
    for (int i = threadIdx.x; i < kTile * kMlpIn; i += blockDim.x) {
        long long r = row0 + i / kMlpIn;
        S.x[i] = __float2bfloat16(r < n ? x[r * kMlpIn + (i % kMlpIn)] : 0.f);
    }
}

__global__ void __launch_bounds__(128) k_mlp_forward(const float *P, const float *x, long long n, float *y)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainSmem &S = *reinterpret_cast<TrainSmem *>(smem_raw);
    const long long row0 = (long long)blockIdx.x * kTile;
    load_params(S, P);
    load_x(S, x, n, row0);
    __syncthreads();
    const int w = threadIdx.x >> 5;
    mlp_forward16(S.x + w * 16 * kMlpIn, S.w1, S.w2, S.w3p, S.b1, S.b2, S.b3, S.h1 + w * 16 * kHStride,
                  S.h2 + w * 16 * kHStride, S.y + w * 16 * kMlpOut);
    __syncthreads();
    for (int i = threadIdx.x; i < kTile * kMlpOut; i += blockDim.x) {
        long long r = row0 + i / kMlpOut;
        if (r < n) y[r * kMlpOut + (i % kMlpOut)] = S.y[i];
    }
}

// accumulator fragment -> atomic adds into a [rows][cols] FP32 gradient
__device__ __forceinline__ void atomic_frag(float *G, int ldg, int r0, int n0, const float d[4], int rmax)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int c = n0 + 2 * t;
    if (r0 + g < rmax) {
        atomicAdd(G + (r0 + g) * ldg + c, d[0]);
        atomicAdd(G + (r0 + g) * ldg + c + 1, d[1]);
    }
    if (r0 + g + 8 < rmax) {
        atomicAdd(G + (r0 + g + 8) * ldg + c, d[2]);
        atomicAdd(G + (r0 + g + 8) * ldg + c + 1, d[3]);
    }
}

// masked store of a fragment into a bf16 [rows][kHStride] tile: value * [H > 0]
__device__ __forceinline__ void store_masked(__nv_bfloat16 *D, const __nv_bfloat16 *H, int r0, int n0,
                                             const float d[4])
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int c = n0 + 2 * t;
    const int i0 = (r0 + g) * kHStride + c, i1 = (r0 + g + 8) * kHStride + c;
    float m0 = __bfloat162float(H[i0]) > 0.f ? 1.f : 0.f, m1 = __bfloat162float(H[i0 + 1]) > 0.f ? 1.f : 0.f;
    float m2 = __bfloat162float(H[i1]) > 0.f ? 1.f : 0.f, m3 = __bfloat162float(H[i1 + 1]) > 0.f ? 1.f : 0.f;
    *reinterpret_cast<uint32_t *>(D + i0) = pack_bf16(d[0] * m0, d[1] * m1);
    *reinterpret_cast<uint32_t *>(D + i1) = pack_bf16(d[2] * m2, d[3] * m3);
}

// one tile: forward, loss, backward; grad += d(loss)/d(params) where loss is
// the mean over `count` samples of the summed squared error of the 7 outputs
__global__ void __launch_bounds__(128) k_mlp_grad(const float *P, const float *x, const float *yt,
                                                  long long n, long long row_begin, float inv_count,
                                                  float *grad, double *loss)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainSmem &S = *reinterpret_cast<TrainSmem *>(smem_raw);
    const long long row0 = row_begin + (long long)blockIdx.x * kTile;
    const int w = threadIdx.x >> 5;
    load_params(S, P);
    load_x(S, x, n, row0);
    __syncthreads();
    mlp_forward16(S.x + w * 16 * kMlpIn, S.w1, S.w2, S.w3p, S.b1, S.b2, S.b3, S.h1 + w * 16 * kHStride,
                  S.h2 + w * 16 * kHStride, S.y + w * 16 * kMlpOut);
    __syncthreads();
    // dY and the loss of this tile
    double l = 0.0;
    for (int i = threadIdx.x; i < kTile * 16; i += blockDim.x) {
        int r = i / 16, j = i % 16;
        long long gr = row0 + r;
        float dv = 0.f;
        if (j < kMlpOutUsed && gr < n) {
            float e = S.y[r * kMlpOut + j] - yt[gr * kMlpOut + j];
            l += (double)e * e;
            dv = 2.f * e * inv_count;
        }
        S.dy[i] = __float2bfloat16(dv);
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, l * inv_count);
    __syncthreads();
    uint32_t a[4], b[2];
    // dW3 [8 x 64] (M padded to 16): A(j, r) = dY[r][j], B(r, c) = H2[r][c]
    for (int nt = w * 2; nt < w * 2 + 2; ++nt) {
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        for (int kt = 0; kt < kTile / 16; ++kt) {
            frag_a_gen(a, S.dy, 1, 16, 0, kt * 16);
            frag_b_gen(b, S.h2, kHStride, 1, kt * 16, nt * 8);
            mma_bf16(d, a, b);
        }
        atomic_frag(grad + kOW3, kMlpHid, 0, nt * 8, d, kMlpOutUsed);
    }
    // dH2 = dY W3 * [H2 > 0], rows of this warp: A = dY rows, B(j, c) = W3[j][c]
    for (int nt = 0; nt < kMlpHid / 8; ++nt) {
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        frag_a_row(a, S.dy, 16, w * 16, 0);
        frag_b_gen(b, S.w3p, kMlpHid, 1, 0, nt * 8);
        mma_bf16(d, a, b);
        store_masked(S.dh2, S.h2, w * 16, nt * 8, d);
    }
    __syncthreads();
    // dW2 [64 x 64]: A(o, r) = dH2[r][o], B(r, i) = H1[r][i]; warp w owns rows o in [16w, 16w+16)
    for (int nt = 0; nt < kMlpHid / 8; ++nt) {
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        for (int kt = 0; kt < kTile / 16; ++kt) {
            frag_a_gen(a, S.dh2, 1, kHStride, w * 16, kt * 16);
            frag_b_gen(b, S.h1, kHStride, 1, kt * 16, nt * 8);
            mma_bf16(d, a, b);
        }
        atomic_frag(grad + kOW2, kMlpHid, w * 16, nt * 8, d, kMlpHid);
    }
    // dH1 = dH2 W2 * [H1 > 0]: A = dH2 rows of this warp, B(o, i) = W2[o][i]
    for (int nt = 0; nt < kMlpHid / 8; ++nt) {
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        for (int kt = 0; kt < kMlpHid / 16; ++kt) {
            frag_a_row(a, S.dh2, kHStride, w * 16, kt * 16);
            frag_b_gen(b, S.w2, kMlpHid, 1, kt * 16, nt * 8);
            mma_bf16(d, a, b);
        }
        store_masked(S.dh1, S.h1, w * 16, nt * 8, d);
    }
    __syncthreads();
    // dW1 [64 x 16]: A(o, r) = dH1[r][o], B(r, i) = X[r][i]
    for (int nt = 0; nt < kMlpIn / 8; ++nt) {
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        for (int kt = 0; kt < kTile / 16; ++kt) {
            frag_a_gen(a, S.dh1, 1, kHStride, w * 16, kt * 16);
            frag_b_gen(b, S.x, kMlpIn, 1, kt * 16, nt * 8);
            mma_bf16(d, a, b);
        }
        atomic_frag(grad + kOW1, kMlpIn, w * 16, nt * 8, d, kMlpHid);
    }
    // bias gradients: column sums of dY, dH2, dH1 (bf16 values, as the MMAs use)
    for (int c = threadIdx.x; c < kMlpHid; c += blockDim.x) {
        float s1 = 0.f, s2 = 0.f;
        for (int r = 0; r < kTile; ++r) {
            s1 += __bfloat162float(S.dh1[r * kHStride + c]);
            s2 += __bfloat162float(S.dh2[r * kHStride + c]);
        }
        atomicAdd(grad + kOB1 + c, s1);
        atomicAdd(grad + kOB2 + c, s2);
    }
    for (int j = threadIdx.x; j < kMlpOutUsed; j += blockDim.x) {
        float s3 = 0.f;
        for (int r = 0; r < kTile; ++r) s3 += __bfloat162float(S.dy[r * 16 + j]);
        atomicAdd(grad + kOB3 + j, s3);
    }
}

// Adam (Kingma & Ba 2015) on the flat FP32 parameters; padded entries stay 0
__global__ void k_adam(float *P, float *m, float *v, const float *grad, int t, float lr)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kNParams) return;
    // padding: input columns 14, 15 of W1 and output row 7 of W3 / b3
    if (i < kOB1 && (i % kMlpIn) >= kMlpInUsed) return;
    if (i >= kOW3 && i < kOB3 && (i - kOW3) / kMlpHid >= kMlpOutUsed) return;
    if (i >= kOB3 && (i - kOB3) >= kMlpOutUsed) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    float g = grad[i];
    float mi = b1 * m[i] + (1.f - b1) * g;
    float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    float mh = mi / (1.f - powf(b1, (float)t)), vh = vi / (1.f - powf(b2, (float)t));
    P[i] -= lr * mh / (sqrtf(vh) + eps);
}

void pack(const des_mlp &net, std::vector<float> &P)
{
    P.assign(kNParams, 0.f);
    std::memcpy(&P[kOW1], net.w1, sizeof(net.w1));
    std::memcpy(&P[kOB1], net.b1, sizeof(net.b1));
    std::memcpy(&P[kOW2], net.w2, sizeof(net.w2));
    std::memcpy(&P[kOB2], net.b2, sizeof(net.b2));
    std::memcpy(&P[kOW3], net.w3, sizeof(net.w3));
    std::memcpy(&P[kOB3], net.b3, sizeof(net.b3));
}
void unpack(const std::vector<float> &P, des_mlp &net)
{
    std::memcpy(net.w1, &P[kOW1], sizeof(net.w1));
    std::memcpy(net.b1, &P[kOB1], sizeof(net.b1));
    std::memcpy(net.w2, &P[kOW2], sizeof(net.w2));
    std::memcpy(net.b2, &P[kOB2], sizeof(net.b2));
    std::memcpy(net.w3, &P[kOW3], sizeof(net.w3));
    std::memcpy(net.b3, &P[kOB3], sizeof(net.b3));
}

struct DevBuf {
    void *p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
    template <class T> T *as() { return static_cast<T *>(p); }
    int alloc(size_t bytes) { return cudaMalloc(&p, bytes ? bytes : 1) == cudaSuccess ? DES_OK : DES_ERR_NOMEM; }
};

int smem_setup(const void *fn)
{
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TrainSmem)) ==
                   cudaSuccess
               ? DES_OK
               : DES_ERR_CUDA;
}

}  // namespace

extern "C" {

int des_mlp_forward(const des_mlp *net, const float *x, long long n, float *y)
{
    if (!net || !x || !y || n < 1) return DES_ERR_ARG;
    std::vector<float> P;
    pack(*net, P);
    DevBuf dP, dx, dy;
    if (dP.alloc(sizeof(float) * kNParams) || dx.alloc(sizeof(float) * n * kMlpIn) ||
        dy.alloc(sizeof(float) * n * kMlpOut))
        return DES_ERR_NOMEM;
    if (smem_setup((const void *)k_mlp_forward)) return DES_ERR_CUDA;
    if (cudaMemcpy(dP.p, P.data(), sizeof(float) * kNParams, cudaMemcpyHostToDevice) ||
        cudaMemcpy(dx.p, x, sizeof(float) * n * kMlpIn, cudaMemcpyHostToDevice))
        return DES_ERR_CUDA;
    int grid = (int)((n + kTile - 1) / kTile);
    k_mlp_forward<<<grid, 128, sizeof(TrainSmem)>>>(dP.as<float>(), dx.as<float>(), n, dy.as<float>());
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return DES_ERR_CUDA;
    return cudaMemcpy(y, dy.p, sizeof(float) * n * kMlpOut, cudaMemcpyDeviceToHost) == cudaSuccess ? DES_OK
                                                                                                    : DES_ERR_CUDA;
}

int des_mlp_loss_grad(const des_mlp *net, const float *x, const float *y, long long n, double *loss,
                      des_mlp *grad)
{
    if (!net || !x || !y || n < 1 || !loss || !grad) return DES_ERR_ARG;
    std::vector<float> P;
    pack(*net, P);
    DevBuf dP, dx, dy, dg, dl;
    if (dP.alloc(sizeof(float) * kNParams) || dx.alloc(sizeof(float) * n * kMlpIn) ||
        dy.alloc(sizeof(float) * n * kMlpOut) || dg.alloc(sizeof(float) * kNParams) || dl.alloc(sizeof(double)))
        return DES_ERR_NOMEM;
    if (smem_setup((const void *)k_mlp_grad)) return DES_ERR_CUDA;
    if (cudaMemcpy(dP.p, P.data(), sizeof(float) * kNParams, cudaMemcpyHostToDevice) ||
        cudaMemcpy(dx.p, x, sizeof(float) * n * kMlpIn, cudaMemcpyHostToDevice) ||
        cudaMemcpy(dy.p, y, sizeof(float) * n * kMlpOut, cudaMemcpyHostToDevice) ||
        cudaMemset(dg.p, 0, sizeof(float) * kNParams) || cudaMemset(dl.p, 0, sizeof(double)))
        return DES_ERR_CUDA;
    int grid = (int)((n + kTile - 1) / kTile);
    k_mlp_grad<<<grid, 128, sizeof(TrainSmem)>>>(dP.as<float>(), dx.as<float>(), dy.as<float>(), n, 0,
                                                 1.f / (float)n, dg.as<float>(), dl.as<double>());
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return DES_ERR_CUDA;
    std::vector<float> G(kNParams);
    if (cudaMemcpy(G.data(), dg.p, sizeof(float) * kNParams, cudaMemcpyDeviceToHost) ||
        cudaMemcpy(loss, dl.p, sizeof(double), cudaMemcpyDeviceToHost))
        return DES_ERR_CUDA;
    std::memset(grad, 0, sizeof(*grad));
    unpack(G, *grad);
    return DES_OK;
}

int des_mlp_train(des_mlp *net, const float *x, const float *y, long long n, int steps, int batch,
                  float lr, unsigned long long seed, float *loss_trace)
{
    if (!net || !x || !y || n < kTile || steps < 1 || batch < kTile) return DES_ERR_ARG;
    batch = (int)std::min<long long>((batch / kTile) * kTile, (n / kTile) * kTile);
    // shuffle once on the host; mini-batches are contiguous slices after that
    std::vector<long long> perm(n);
    std::iota(perm.begin(), perm.end(), 0LL);
    std::mt19937_64 rng(seed);
    std::shuffle(perm.begin(), perm.end(), rng);
    std::vector<float> xs((size_t)n * kMlpIn), ys((size_t)n * kMlpOut);
    for (long long i = 0; i < n; ++i) {
        std::memcpy(&xs[i * kMlpIn], &x[perm[i] * kMlpIn], sizeof(float) * kMlpIn);
        std::memcpy(&ys[i * kMlpOut], &y[perm[i] * kMlpOut], sizeof(float) * kMlpOut);
    }
    std::vector<float> P;
    pack(*net, P);
    DevBuf dP, dx, dy, dg, dm, dv, dl;
    if (dP.alloc(sizeof(float) * kNParams) || dx.alloc(sizeof(float) * n * kMlpIn) ||
        dy.alloc(sizeof(float) * n * kMlpOut) || dg.alloc(sizeof(float) * kNParams) ||
        dm.alloc(sizeof(float) * kNParams) || dv.alloc(sizeof(float) * kNParams) ||
        dl.alloc(sizeof(double) * (size_t)steps))
        return DES_ERR_NOMEM;
    if (smem_setup((const void *)k_mlp_grad)) return DES_ERR_CUDA;
    if (cudaMemcpy(dP.p, P.data(), sizeof(float) * kNParams, cudaMemcpyHostToDevice) ||
        cudaMemcpy(dx.p, xs.data(), sizeof(float) * n * kMlpIn, cudaMemcpyHostToDevice) ||
        cudaMemcpy(dy.p, ys.data(), sizeof(float) * n * kMlpOut, cudaMemcpyHostToDevice) ||
        cudaMemset(dm.p, 0, sizeof(float) * kNParams) || cudaMemset(dv.p, 0, sizeof(float) * kNParams) ||
        cudaMemset(dl.p, 0, sizeof(double) * (size_t)steps))
        return DES_ERR_CUDA;
    const long long nb = n / batch;
    const int grid = batch / kTile;
    for (int s = 0; s < steps; ++s) {
        long long begin = (long long)(s % nb) * batch;
        // cosine decay of the step size from lr to lr / 100
        const float lr_s = lr * (0.01f + 0.99f * 0.5f * (1.f + cosf(3.14159265f * (float)s / (float)steps)));
        cudaMemsetAsync(dg.p, 0, sizeof(float) * kNParams);
        k_mlp_grad<<<grid, 128, sizeof(TrainSmem)>>>(dP.as<float>(), dx.as<float>(), dy.as<float>(), n,
                                                     begin, 1.f / (float)batch, dg.as<float>(),
                                                     dl.as<double>() + s);
        k_adam<<<(kNParams + 255) / 256, 256>>>(dP.as<float>(), dm.as<float>(), dv.as<float>(),
                                               dg.as<float>(), s + 1, lr_s);
    }
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return DES_ERR_CUDA;
    if (cudaMemcpy(P.data(), dP.p, sizeof(float) * kNParams, cudaMemcpyDeviceToHost)) return DES_ERR_CUDA;
    unpack(P, *net);
    if (loss_trace) {
        std::vector<double> L(steps);
        if (cudaMemcpy(L.data(), dl.p, sizeof(double) * steps, cudaMemcpyDeviceToHost)) return DES_ERR_CUDA;
        for (int s = 0; s < steps; ++s) loss_trace[s] = (float)L[s];
    }
    return DES_OK;
}

}  // extern "C"
