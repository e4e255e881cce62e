// Training and standalone evaluation of the learned return-map closure
// (see des_mlp.cuh for the network).  Forward and backward passes run on the
// fifth-generation tensor cores (des_mlp_tc.cuh: tcgen05 MMAs, BF16 operands
// in shared memory, FP32 accumulators in tensor memory), persistent CTAs (at
// most one per multiprocessor) over tiles of 128 samples; a CTA's weight
// gradients accumulate in TMEM over its tiles and are added to the global
// FP32 gradient with atomics once (one add per parameter per CTA).  Adam keeps FP32 master weights
// and moments.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "des_gpu.h"
#include "des_mlp.cuh"
#include "des_mlp_tc.cuh"

using namespace des;

namespace {

constexpr int kTile = kTcRows;               // samples per CTA
constexpr int kNW1 = kMlpHid * kMlpIn, kNW2 = kMlpHid * kMlpHid, kNW3 = kMlpOut * kMlpHid;
constexpr int kNParams = kNW1 + kMlpHid + kNW2 + kMlpHid + kNW3 + kMlpOut;   // 5,768
// offsets of the parameter groups in a flat FP32 vector
constexpr int kOW1 = 0, kOB1 = kOW1 + kNW1, kOW2 = kOB1 + kMlpHid, kOB2 = kOW2 + kNW2,
              kOW3 = kOB2 + kMlpHid, kOB3 = kOW3 + kNW3;
static_assert(kOB1 == mlptc::oB1 && kOW2 == mlptc::oW2 && kOB2 == mlptc::oB2 && kOW3 == mlptc::oW3 &&
                  kOB3 == mlptc::oB3,
              "parameter layout");

__device__ __forceinline__ MlpTcSmem &tc_smem(unsigned char *raw)
{
    return *reinterpret_cast<MlpTcSmem *>((reinterpret_cast<uintptr_t>(raw) + 1023) & ~uintptr_t(1023));
}

__global__ void __launch_bounds__(kTcRows) k_mlp_forward(const float *P, const float *x, long long n, float *y,
                                                         int *err)
{
    extern __shared__ unsigned char smem_raw[];
    MlpTcSmem &S = tc_smem(smem_raw);
    const bool ok = mlptc_tiles<false>(S, P, x, nullptr, n, 0, (n + kTile - 1) / kTile, 0.f, y, nullptr,
                                       nullptr);
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
}

// ntiles tiles from row_begin: forward, loss, backward; grad +=
// d(loss)/d(params) where loss is the mean over `count` samples of the
// summed squared error of the 7 outputs
__global__ void __launch_bounds__(kTcRows) k_mlp_grad(const float *P, const float *x, const float *yt,
                                                      long long n, long long row_begin, long long ntiles,
                                                      float inv_count, float *grad, double *loss, int *err)
{
    extern __shared__ unsigned char smem_raw[];
    MlpTcSmem &S = tc_smem(smem_raw);
    const bool ok = mlptc_tiles<true>(S, P, x, yt, n, row_begin, ntiles, inv_count, nullptr, grad, loss);
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
}

// CTAs for ntiles tiles: one per multiprocessor at most (persistent)
int tile_grid(long long ntiles)
{
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return (int)std::max<long long>(1, std::min<long long>(ntiles, sms > 0 ? sms : 1));
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
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMlpTcSmemBytes) ==
                   cudaSuccess
               ? DES_OK
               : DES_ERR_CUDA;
}

// the kernels' time-out flag: DES_ERR_CUDA when a tensor-core wait gave up
int read_err(const int *derr)
{
    int e = 0;
    if (cudaMemcpy(&e, derr, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return DES_ERR_CUDA;
    return e ? DES_ERR_CUDA : DES_OK;
}

}  // namespace

extern "C" {

int des_mlp_forward(const des_mlp *net, const float *x, long long n, float *y)
{
    if (!net || !x || !y || n < 1) return DES_ERR_ARG;
    std::vector<float> P;
    pack(*net, P);
    DevBuf dP, dx, dy, de;
    if (dP.alloc(sizeof(float) * kNParams) || dx.alloc(sizeof(float) * n * kMlpIn) ||
        dy.alloc(sizeof(float) * n * kMlpOut) || de.alloc(sizeof(int)))
        return DES_ERR_NOMEM;
    if (smem_setup((const void *)k_mlp_forward)) return DES_ERR_CUDA;
    if (cudaMemcpy(dP.p, P.data(), sizeof(float) * kNParams, cudaMemcpyHostToDevice) ||
        cudaMemcpy(dx.p, x, sizeof(float) * n * kMlpIn, cudaMemcpyHostToDevice) ||
        cudaMemset(de.p, 0, sizeof(int)))
        return DES_ERR_CUDA;
    const int grid = tile_grid((n + kTile - 1) / kTile);
    k_mlp_forward<<<grid, kTcRows, kMlpTcSmemBytes>>>(dP.as<float>(), dx.as<float>(), n, dy.as<float>(),
                                                      de.as<int>());
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return DES_ERR_CUDA;
    if (int rc = read_err(de.as<int>())) return rc;
    return cudaMemcpy(y, dy.p, sizeof(float) * n * kMlpOut, cudaMemcpyDeviceToHost) == cudaSuccess ? DES_OK
                                                                                                    : DES_ERR_CUDA;
}

int des_mlp_loss_grad(const des_mlp *net, const float *x, const float *y, long long n, double *loss,
                      des_mlp *grad)
{
    if (!net || !x || !y || n < 1 || !loss || !grad) return DES_ERR_ARG;
    std::vector<float> P;
    pack(*net, P);
    DevBuf dP, dx, dy, dg, dl, de;
    if (dP.alloc(sizeof(float) * kNParams) || dx.alloc(sizeof(float) * n * kMlpIn) ||
        dy.alloc(sizeof(float) * n * kMlpOut) || dg.alloc(sizeof(float) * kNParams) || dl.alloc(sizeof(double)) ||
        de.alloc(sizeof(int)))
        return DES_ERR_NOMEM;
    if (smem_setup((const void *)k_mlp_grad)) return DES_ERR_CUDA;
    if (cudaMemcpy(dP.p, P.data(), sizeof(float) * kNParams, cudaMemcpyHostToDevice) ||
        cudaMemcpy(dx.p, x, sizeof(float) * n * kMlpIn, cudaMemcpyHostToDevice) ||
        cudaMemcpy(dy.p, y, sizeof(float) * n * kMlpOut, cudaMemcpyHostToDevice) ||
        cudaMemset(dg.p, 0, sizeof(float) * kNParams) || cudaMemset(dl.p, 0, sizeof(double)) ||
        cudaMemset(de.p, 0, sizeof(int)))
        return DES_ERR_CUDA;
    const long long ntiles = (n + kTile - 1) / kTile;
    k_mlp_grad<<<tile_grid(ntiles), kTcRows, kMlpTcSmemBytes>>>(dP.as<float>(), dx.as<float>(), dy.as<float>(),
                                                                n, 0, ntiles, 1.f / (float)n, dg.as<float>(), dl.as<double>(), de.as<int>());
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return DES_ERR_CUDA;
    if (int rc = read_err(de.as<int>())) return rc;
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
    DevBuf dP, dx, dy, dg, dm, dv, dl, de;
    if (dP.alloc(sizeof(float) * kNParams) || dx.alloc(sizeof(float) * n * kMlpIn) ||
        dy.alloc(sizeof(float) * n * kMlpOut) || dg.alloc(sizeof(float) * kNParams) ||
        dm.alloc(sizeof(float) * kNParams) || dv.alloc(sizeof(float) * kNParams) ||
        dl.alloc(sizeof(double) * (size_t)steps) || de.alloc(sizeof(int)))
        return DES_ERR_NOMEM;
    if (smem_setup((const void *)k_mlp_grad)) return DES_ERR_CUDA;
    if (cudaMemcpy(dP.p, P.data(), sizeof(float) * kNParams, cudaMemcpyHostToDevice) ||
        cudaMemcpy(dx.p, xs.data(), sizeof(float) * n * kMlpIn, cudaMemcpyHostToDevice) ||
        cudaMemcpy(dy.p, ys.data(), sizeof(float) * n * kMlpOut, cudaMemcpyHostToDevice) ||
        cudaMemset(dm.p, 0, sizeof(float) * kNParams) || cudaMemset(dv.p, 0, sizeof(float) * kNParams) ||
        cudaMemset(dl.p, 0, sizeof(double) * (size_t)steps) || cudaMemset(de.p, 0, sizeof(int)))
        return DES_ERR_CUDA;
    const long long nb = n / batch;
    const int ntiles = batch / kTile, grid = tile_grid(ntiles);
    for (int s = 0; s < steps; ++s) {
        long long begin = (long long)(s % nb) * batch;
        // cosine decay of the step size from lr to lr / 100
        const float lr_s = lr * (0.01f + 0.99f * 0.5f * (1.f + cosf(3.14159265f * (float)s / (float)steps)));
        cudaMemsetAsync(dg.p, 0, sizeof(float) * kNParams);
        k_mlp_grad<<<grid, kTcRows, kMlpTcSmemBytes>>>(dP.as<float>(), dx.as<float>(), dy.as<float>(), n,
                                                       begin, ntiles, 1.f / (float)batch, dg.as<float>(),
                                                       dl.as<double>() + s, de.as<int>());
        k_adam<<<(kNParams + 255) / 256, 256>>>(dP.as<float>(), dm.as<float>(), dv.as<float>(),
                                               dg.as<float>(), s + 1, lr_s);
    }
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return DES_ERR_CUDA;
    if (int rc = read_err(de.as<int>())) return rc;
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
