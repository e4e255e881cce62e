// The node -> element support lists (create_support, mesh.cxx:1703-1717) built
// on the device from the connectivity: for every node, the elements that hold
// it in ascending element order, as a CSR of (element << 2 | local slot).
// The step's node-side sums run over these lists in this order, which is the
// order of the reference's own node loops, so the sums are bit-identical.
//
//   count   one thread per (element, slot): atomicAdd into off[node + 1]
//   scan    inclusive scan of off[0..N] (off[0] = 0): 1024-entry blocks,
//           their totals scanned by one block, then added back
//   fill    one thread per (element, slot): a slot in its node's range from
//           a per-node cursor (order within a node is not yet defined)
//   sort    one thread per node: insertion sort of its range; an element
//           holds a node once, so sorting the packed entries sorts by element
//
// Connectivity entries must lie in [0, N) (des_gpu_create checks them on the
// host before these kernels run).
#pragma once

namespace des {

constexpr int kScanBlock = 1024;

__global__ void k_sup_count(long long nent, const int *__restrict__ conn, int *off)
{
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q < nent) atomicAdd(&off[conn[q] + 1], 1);
}

// inclusive scan of a[0..n) in blocks of kScanBlock; each block's total to sums
__global__ void __launch_bounds__(kScanBlock) k_scan_blocks(int *a, long long n, int *sums)
{
    __shared__ int warp_tot[kScanBlock / 32];
    const long long i = blockIdx.x * (long long)kScanBlock + threadIdx.x;
    int v = i < n ? a[i] : 0;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    if (lane == 31) warp_tot[w] = v;
    __syncthreads();
    if (w == 0) {
        int t = warp_tot[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        warp_tot[lane] = t;
    }
    __syncthreads();
    if (w > 0) v += warp_tot[w - 1];
    if (i < n) a[i] = v;
    if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = v;
}

// exclusive prefix of the block totals, in place, by one block
__global__ void __launch_bounds__(kScanBlock) k_scan_sums(int *sums, int nblocks)
{
    __shared__ int warp_tot[kScanBlock / 32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int base = 0; base < nblocks; base += kScanBlock) {
        const int i = base + threadIdx.x;
        const int x = i < nblocks ? sums[i] : 0;
        int v = x;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        if (lane == 31) warp_tot[w] = v;
        __syncthreads();
        if (w == 0) {
            int t = warp_tot[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            warp_tot[lane] = t;
        }
        __syncthreads();
        if (w > 0) v += warp_tot[w - 1];
        const int c = carry;
        if (i < nblocks) sums[i] = c + v - x;          // exclusive
        __syncthreads();
        if (threadIdx.x == kScanBlock - 1) carry = c + v;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kScanBlock) k_scan_add(int *a, long long n, const int *sums)
{
    const long long i = blockIdx.x * (long long)kScanBlock + threadIdx.x;
    if (i < n) a[i] += sums[blockIdx.x];
}

__global__ void k_sup_fill(long long nent, const int *__restrict__ conn, const int *__restrict__ off,
                           int *cursor, unsigned *ent)
{
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= nent) return;
    const int n = conn[q];
    const int p = off[n] + atomicAdd(&cursor[n], 1);
    ent[p] = ((unsigned)(q >> 2) << 2) | (unsigned)(q & 3);
}

__global__ void k_sup_sort(int nnode, const int *__restrict__ off, unsigned *ent)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nnode) return;
    const int a = off[n], b = off[n + 1];
    for (int k = a + 1; k < b; ++k) {
        const unsigned v = ent[k];
        int j = k - 1;
        while (j >= a && ent[j] > v) {
            ent[j + 1] = ent[j];
            --j;
        }
        ent[j + 1] = v;
    }
}

}  // namespace des
