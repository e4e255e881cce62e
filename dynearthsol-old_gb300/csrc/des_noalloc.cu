// des_compute_dt_noalloc: the stable time step (compute_dt) for callers that
// cannot let a library allocate device memory.
//
// Who needs it: applications that own every byte of device memory through
// their own pool or budget, and code paths that must not call cudaMalloc or
// cudaFree because those calls can synchronise the whole device and stall
// other streams.  The des_gpu handle allocates its state when it is created;
// this entry point instead works directly on device arrays the caller already
// has, and keeps its only scratch -- one partial minimum per thread block and
// a completion counter -- in a fixed array compiled into the library.
//
// Limits and sharing:
//  * at most kMaxBlocks * kBlock = 16,777,216 elements per call (one thread
//    per element, one partial per block); larger meshes get DES_ERR_SIZE;
//  * the scratch array (1.5 MiB + 256 B) is held on every GPU that loads the
//    library until the process exits;
//  * all calls share it: calls that overlap on the GPU (different streams or
//    host threads without ordering) race and give wrong results; the counter
//    is cleared at the start of every call, the partials are rewritten by it.
//  * the first call on a device looks up the array's device address (a
//    set-up per device, done with that device current); make that first
//    call before any stream capture.  Every later call made while its stream
//    is not capturing looks the address up again, so a device reset (which
//    unloads the library's module and may place the array elsewhere when it
//    is loaded again) is followed by a fresh look-up; a call made during a
//    capture uses the address of the last call made outside one.
//  * dt <= 0, where compute_dt exits with code 11 (geometry.cxx:321-325),
//    is reported through the optional device status word, which every call
//    sets to DES_OK or DES_ERR_DT.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "des_device.cuh"
#include "des_gpu.h"

using namespace des;

namespace {

constexpr int kBlock = 256;
constexpr int kMaxBlocks = 65536;
constexpr long long kMaxElems = (long long)kBlock * kMaxBlocks;
constexpr int kCounter = 3 * kMaxBlocks;             // word index of the completion counter
constexpr int kWords = 3 * kMaxBlocks + 32;
constexpr int kMaxDevices = 64;

struct DtIn {
    double visc_min, therm_diff_max, max_vbc_val, inertial_scaling, dt_fraction;
    double shear_modulus, bulkm0, rho0;
    int is_qs, thermal;
};

}  // namespace

// Scratch of every call: [3 * block] partial minima (order bits of minh,
// dt_diffusion candidate, dt_maxwell candidate), then the counter.
static __device__ __align__(256) unsigned long long g_dt_scratch[kWords];

namespace {

__device__ __forceinline__ unsigned long long umin(unsigned long long a, unsigned long long b)
{
    return b < a ? b : a;
}

// min of three values over the block; result valid in thread 0
__device__ void block_min3(unsigned long long &a, unsigned long long &b, unsigned long long &m)
{
    __shared__ unsigned long long s[3][kBlock / 32];
    for (int o = 16; o > 0; o >>= 1) {
        a = umin(a, __shfl_down_sync(0xffffffffu, a, o));
        b = umin(b, __shfl_down_sync(0xffffffffu, b, o));
        m = umin(m, __shfl_down_sync(0xffffffffu, m, o));
    }
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        s[0][warp] = a;
        s[1][warp] = b;
        s[2][warp] = m;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kBlock / 32; ++w) {
            a = umin(a, s[0][w]);
            b = umin(b, s[1][w]);
            m = umin(m, s[2][w]);
        }
    }
    __syncthreads();
}

// geometry.cxx:270-325 over device arrays in the reference layout
__global__ void __launch_bounds__(kBlock) k_dt_noalloc(unsigned long long *scratch, int nelem,
                                                       const double *__restrict__ coord,
                                                       const int4 *__restrict__ conn,
                                                       const double *__restrict__ vol,
                                                       const double *__restrict__ shearm, DtIn c,
                                                       double *dt_out, int *status)
{
    __shared__ bool last;
    int e = blockIdx.x * kBlock + threadIdx.x;
    unsigned long long a = ~0ULL, b = ~0ULL, m = ~0ULL;
    if (e < nelem) {
        int4 q = conn[e];
        const int n[4] = {q.x, q.y, q.z, q.w};
        double X[4][3];
        for (int i = 0; i < 4; ++i)
            for (int k = 0; k < 3; ++k) X[i][k] = coord[3LL * n[i] + k];
        double minh = min_height(X, vol[e]);
        a = order_bits(minh);
        if (c.thermal) b = order_bits(0.5 * minh * minh / c.therm_diff_max);
        double sh = shearm ? shearm[e] : c.shear_modulus;
        m = order_bits(0.5 * c.visc_min / (1e-40 + sh));
    }
    block_min3(a, b, m);
    if (threadIdx.x == 0) {
        scratch[3 * blockIdx.x + 0] = a;
        scratch[3 * blockIdx.x + 1] = b;
        scratch[3 * blockIdx.x + 2] = m;
        __threadfence();
        unsigned long long done = atomicAdd(&scratch[kCounter], 1ULL);
        last = (done == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    a = b = m = ~0ULL;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += kBlock) {
        a = umin(a, __ldcg(&scratch[3 * i + 0]));
        b = umin(b, __ldcg(&scratch[3 * i + 1]));
        m = umin(m, __ldcg(&scratch[3 * i + 2]));
    }
    block_min3(a, b, m);
    if (threadIdx.x == 0) {
        double minl = from_order_bits(a);
        double dt_diffusion = c.thermal ? from_order_bits(b) : 1.7976931348623157e308;
        double dt_maxwell = from_order_bits(m);
        double dt_advection = 0.5 * minl / c.max_vbc_val;
        double dt_elastic = c.is_qs ? 0.5 * minl / (c.max_vbc_val * c.inertial_scaling)
                                    : 0.5 * minl / sqrt(c.bulkm0 / c.rho0);
        double dt = smin(smin(dt_elastic, dt_maxwell), smin(dt_advection, dt_diffusion)) * c.dt_fraction;
        *dt_out = dt;
        if (status) *status = (dt <= 0) ? DES_ERR_DT : DES_OK;
        scratch[kCounter] = 0;
    }
}

__global__ void k_dt_fixed(double *dt_out, double v, int *status)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        *dt_out = v;
        if (status) *status = DES_OK;     // compute_dt returns a fixed dt unchecked
    }
}

std::mutex g_setup_mutex;
unsigned long long *g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of g_dt_scratch on the current device.  Looked up (with the
// device current) on the first call and on every call whose stream is not
// capturing; a capturing call uses the address its device had last.
int scratch_address(cudaStream_t s, unsigned long long **out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return DES_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return DES_ERR_UNSUPPORTED;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusActive;
    bool capturing = true;
    if (cudaStreamIsCapturing(s, &cap) == cudaSuccess)
        capturing = cap != cudaStreamCaptureStatusNone;
    else
        (void)cudaGetLastError();   // the legacy stream while another captures: not sticky
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!capturing || !g_scratch_ptr[dev]) {
        if (capturing) return DES_ERR_UNSUPPORTED;   // no set-up outside a capture yet
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_dt_scratch) != cudaSuccess || !p) return DES_ERR_CUDA;
        g_scratch_ptr[dev] = static_cast<unsigned long long *>(p);
    }
    *out = g_scratch_ptr[dev];
    return DES_OK;
}

}  // namespace

extern "C" int des_compute_dt_noalloc(int nelem, const double *coord, const int *connectivity,
                                      const double *volume, const double *shearm,
                                      const des_dt_inputs *in, double *dt, int *status,
                                      void *stream)
{
    if (!in || !dt) return DES_ERR_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (in->fixed_dt != 0) {
        k_dt_fixed<<<1, 32, 0, s>>>(dt, in->fixed_dt, status);
        return cudaGetLastError() == cudaSuccess ? DES_OK : DES_ERR_CUDA;
    }
    if (nelem < 1 || !coord || !connectivity || !volume) return DES_ERR_ARG;
    if (reinterpret_cast<uintptr_t>(connectivity) % 16 != 0) return DES_ERR_ARG;
    if (nelem > kMaxElems) return DES_ERR_SIZE;
    unsigned long long *scratch = nullptr;
    int rc = scratch_address(s, &scratch);
    if (rc) return rc;
    if (cudaMemsetAsync(scratch + kCounter, 0, sizeof(unsigned long long), s) != cudaSuccess)
        return DES_ERR_CUDA;
    DtIn c;
    c.visc_min = in->visc_min;
    c.therm_diff_max = in->therm_diff_max;
    c.max_vbc_val = in->max_vbc_val;
    c.inertial_scaling = in->inertial_scaling;
    c.dt_fraction = in->dt_fraction;
    c.shear_modulus = in->shear_modulus;
    c.bulkm0 = in->bulkm0;
    c.rho0 = in->rho0;
    c.is_qs = in->is_quasi_static ? 1 : 0;
    c.thermal = in->has_thermal_diffusion ? 1 : 0;
    int grid = (int)((nelem + kBlock - 1) / kBlock);
    k_dt_noalloc<<<grid, kBlock, 0, s>>>(scratch, nelem, coord,
                                          reinterpret_cast<const int4 *>(connectivity), volume,
                                          shearm, c, dt, status);
    return cudaGetLastError() == cudaSuccess ? DES_OK : DES_ERR_CUDA;
}
