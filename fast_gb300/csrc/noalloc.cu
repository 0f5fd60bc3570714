// Pore count that allocates nothing.
//
// Some callers cannot allocate device memory: a host application whose own
// allocator has reserved all of the GPU's memory (a caching allocator that
// owns the device, so a cudaMalloc from a library fails or fragments its
// pool), or a plug-in host that forbids its plug-ins to allocate device
// memory.  fast_porosity_device_noalloc serves them: the caller passes the
// device-resident mask and a host output, and the reduction's scratch (one
// partial count per block, an arrival counter and the total) lives in the
// file-scope array below instead of memory allocated per call.
//
// The array is part of the library's device image, so every GPU that loads
// the library holds it (kNoallocScratchBytes) until the process exits.  Every
// call shares it: calls whose work overlaps on the GPU (different streams or
// threads, no ordering between them) race on it and must be serialised by the
// caller.
//
// The first call on a device looks up the array's device address (with that
// device current) and keeps it for the life of the process; make one complete
// call on each device before any stream capture, which also loads the kernel
// under lazy module loading.  The kept address is not valid after a
// cudaDeviceReset of that device.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "fasttau.h"
#include "tau_errors.h"

namespace {

constexpr size_t kNoallocScratchBytes = 256 * 1024;  // 256 KiB
constexpr size_t kHeaderBytes = 256;                 // counter at 0, total at 8
constexpr int64_t kVoxelsPerBlock = 65536;
constexpr int kThreads = 256;
constexpr int64_t kMaxBlocks = (int64_t)((kNoallocScratchBytes - kHeaderBytes) / sizeof(unsigned long long));
// Largest volume the scratch can reduce: one partial slot per 65536 voxels.
constexpr int64_t kMaxVoxels = kMaxBlocks * kVoxelsPerBlock;

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

// Fixed-order block sum of one value per thread.
__device__ __forceinline__ unsigned long long block_sum_u64(unsigned long long v, unsigned long long *s_warp)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) s_warp[warp] = v;
    __syncthreads();
    unsigned long long t = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < kThreads / 32; w++) t += s_warp[w];
    __syncthreads();
    return t;  // valid in thread 0
}

// Counts zero bytes of mask[0..n); block b covers [b*65536, (b+1)*65536).
// The last block to finish sums the per-block counts in block order, writes
// the total and re-arms the counter.
__global__ void __launch_bounds__(kThreads) pore_count_noalloc_kernel(const uint8_t *__restrict__ mask, int64_t n,
                                                                      unsigned char *scratch)
{
    __shared__ unsigned long long s_warp[kThreads / 32];
    __shared__ int s_last;
    unsigned int *counter = reinterpret_cast<unsigned int *>(scratch);
    unsigned long long *total = reinterpret_cast<unsigned long long *>(scratch + 8);
    unsigned long long *part = reinterpret_cast<unsigned long long *>(scratch + kHeaderBytes);

    const int64_t base = (int64_t)blockIdx.x * kVoxelsPerBlock;
    const int64_t end = min(base + kVoxelsPerBlock, n);
    unsigned long long c = 0;
    for (int64_t i = base + threadIdx.x; i < end; i += kThreads) c += (__ldg(mask + i) == 0) ? 1ull : 0ull;
    const unsigned long long bsum = block_sum_u64(c, s_warp);
    if (threadIdx.x == 0) part[blockIdx.x] = bsum;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = (atomicAdd(counter, 1u) == gridDim.x - 1) ? 1 : 0;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    unsigned long long t = 0;
    for (unsigned int b = threadIdx.x; b < gridDim.x; b += kThreads) t += __ldcg(part + b);
    const unsigned long long all = block_sum_u64(t, s_warp);
    if (threadIdx.x == 0) {
        *total = all;
        *counter = 0u;
    }
}

namespace {

// Device address of the scratch array, looked up once per device with that
// device current (in host code the array's name is only a host-side stand-in).
std::mutex g_addr_mu;
unsigned char *g_addr[64] = {};

int scratch_address(int dev, unsigned char **out)
{
    std::lock_guard<std::mutex> lk(g_addr_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return ft_fail(FAST_CUDA_ERROR, "cudaGetSymbolAddress(no-allocation scratch) failed: %s",
                           cudaGetErrorString(e));
        g_addr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_addr[dev];
    return FAST_OK;
}

}  // namespace

extern "C" FAST_API int fast_porosity_device_noalloc(const uint8_t *d_mask, int64_t nx, int64_t ny, int64_t nz,
                                                     uint64_t *pore_count, double *porosity, void *stream)
{
    ft_clear_error();
    if (!d_mask) return ft_fail(FAST_NO_HOST_DATA, "mask is NULL");
    if (!pore_count) return ft_fail(FAST_BAD_ARG, "pore_count is NULL");
    if (nx <= 0 || ny <= 0 || nz <= 0) return ft_fail(FAST_BAD_ARG, "dimensions must be positive");
    if (nx > kMaxVoxels || ny > kMaxVoxels || nz > kMaxVoxels || nx * ny > kMaxVoxels || nx * ny * nz > kMaxVoxels)
        return ft_fail(FAST_BAD_ARG,
                       "volume of %lld x %lld x %lld voxels exceeds the no-allocation limit of %lld voxels "
                       "(%zu bytes of static scratch); use fast_porosity",
                       (long long)nx, (long long)ny, (long long)nz, (long long)kMaxVoxels, kNoallocScratchBytes);
    const int64_t n = nx * ny * nz;
    const unsigned int blocks = (unsigned int)((n + kVoxelsPerBlock - 1) / kVoxelsPerBlock);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return ft_fail(FAST_CUDA_ERROR, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return ft_fail(FAST_CUDA_ERROR, "device ordinal %d out of range", dev);
    unsigned char *scratch = nullptr;
    int st = scratch_address(dev, &scratch);
    if (st != FAST_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // The counter and the total must start at zero; the previous call's
    // partial counts are overwritten before they are read.
    e = cudaMemsetAsync(scratch, 0, kHeaderBytes, s);
    if (e != cudaSuccess) return ft_fail(FAST_CUDA_ERROR, "cudaMemsetAsync: %s", cudaGetErrorString(e));
    pore_count_noalloc_kernel<<<blocks, kThreads, 0, s>>>(d_mask, n, scratch);
    e = cudaGetLastError();
    if (e != cudaSuccess) return ft_fail(FAST_CUDA_ERROR, "pore count launch: %s", cudaGetErrorString(e));
    unsigned long long total = 0;
    e = cudaMemcpyAsync(&total, scratch + 8, sizeof(total), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return ft_fail(FAST_CUDA_ERROR, "pore count: %s", cudaGetErrorString(e));
    *pore_count = (uint64_t)total;
    if (porosity) *porosity = (double)total / (double)n;
    return FAST_OK;
}
