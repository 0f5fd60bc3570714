// Volume::binarize on uint8 volumes (fastlib/src/volume/Volume.cpp:478-486,
// kernelBinarizeUnsigned in fastlib/src/cuda/Volume.cu:157-183): the TIFF
// input of `fast tau` binarizes its slices with threshold 1.0, i.e.
// v < 255 -> 0, else 255 (fast/src/VolumeIOModule.h:57-63).
//
// A byte-wise HBM pass: 16 bytes per thread and iteration through a
// grid-stride loop over 8 resident blocks per SM, the compare done four bytes
// at a time with the per-byte unsigned SIMD compare (which yields 0xFF where
// v >= t, exactly the reference's 255).  A buffer that does not start on a
// 16-byte boundary has its first and last bytes done one at a time.
#include <cuda_runtime.h>

#include <cstdint>

#include "fasttau.h"
#include "tau_errors.h"

namespace {

constexpr int kThreads = 256;
constexpr int kBlocksPerSM = 8;

__global__ void __launch_bounds__(kThreads) binarize_kernel(uint8_t *v, uint64_t head, uint64_t nvec, uint64_t n,
                                                            uint32_t t4)
{
    const uint64_t tid = blockIdx.x * (uint64_t)kThreads + threadIdx.x;
    const uint64_t stride = (uint64_t)gridDim.x * kThreads;
    uint4 *body = reinterpret_cast<uint4 *>(v + head);
    for (uint64_t i = tid; i < nvec; i += stride) {
        uint4 w = body[i];
        w.x = __vcmpgeu4(w.x, t4);
        w.y = __vcmpgeu4(w.y, t4);
        w.z = __vcmpgeu4(w.z, t4);
        w.w = __vcmpgeu4(w.w, t4);
        body[i] = w;
    }
    const uint32_t t = t4 & 0xFFu;
    if (tid < head) v[tid] = v[tid] < t ? 0 : 255;
    const uint64_t j = head + nvec * 16 + tid;
    if (tid < 16 && j < n) v[j] = v[j] < t ? 0 : 255;
}

// uchar(threshold * 255) as kernelBinarizeUnsigned's caller forms it, with
// the threshold clamped to [0, 1] so the conversion is defined.
uint32_t threshold_byte(float threshold)
{
    const float c = !(threshold > 0.f) ? 0.f : (threshold > 1.f ? 1.f : threshold);
    return (uint32_t)(unsigned char)(c * 255.0f);
}

int launch_binarize(uint8_t *d, uint64_t n, float threshold, cudaStream_t s)
{
    if (n == 0) return FAST_OK;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return ft_fail(FAST_CUDA_ERROR, "device query: %s", cudaGetErrorString(e));
    const uint64_t mis = (uint64_t)(reinterpret_cast<uintptr_t>(d) & 15u);
    const uint64_t head = mis ? (16 - mis < n ? 16 - mis : n) : 0;
    const uint64_t nvec = (n - head) / 16;
    const uint64_t want = (nvec + kThreads - 1) / kThreads;
    uint64_t blocks = (uint64_t)sms * kBlocksPerSM;
    if (want < blocks) blocks = want;
    if (blocks == 0) blocks = 1;
    const uint32_t t = threshold_byte(threshold);
    binarize_kernel<<<(unsigned)blocks, kThreads, 0, s>>>(d, head, nvec, n, t * 0x01010101u);
    e = cudaGetLastError();
    if (e != cudaSuccess) return ft_fail(FAST_CUDA_ERROR, "binarize launch: %s", cudaGetErrorString(e));
    return FAST_OK;
}

}  // namespace

extern "C" {

FAST_API int fast_binarize_device(uint8_t *d_volume, uint64_t n, float threshold, void *stream)
{
    ft_clear_error();
    if (!d_volume && n) return ft_fail(FAST_NO_HOST_DATA, "volume is NULL");
    return launch_binarize(d_volume, n, threshold, (cudaStream_t)stream);
}

FAST_API int fast_binarize(uint8_t *volume, uint64_t n, float threshold)
{
    ft_clear_error();
    if (!volume && n) return ft_fail(FAST_NO_HOST_DATA, "volume is NULL");
    if (n == 0) return FAST_OK;
    cudaStream_t st = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e != cudaSuccess) return ft_fail(FAST_CUDA_ERROR, "stream: %s", cudaGetErrorString(e));
    uint8_t *d = nullptr;
    int s = FAST_OK;
    e = cudaMallocAsync((void **)&d, n, st);
    if (e != cudaSuccess) {
        s = ft_fail(FAST_NOMEM, "binarize buffer: %s", cudaGetErrorString(e));
    } else {
        e = cudaMemcpyAsync(d, volume, n, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) s = ft_fail(FAST_CUDA_ERROR, "binarize upload: %s", cudaGetErrorString(e));
        if (s == FAST_OK) s = launch_binarize(d, n, threshold, st);
        if (s == FAST_OK) {
            e = cudaMemcpyAsync(volume, d, n, cudaMemcpyDeviceToHost, st);
            if (e != cudaSuccess) s = ft_fail(FAST_CUDA_ERROR, "binarize download: %s", cudaGetErrorString(e));
        }
        cudaFreeAsync(d, st);
    }
    e = cudaStreamSynchronize(st);
    if (s == FAST_OK && e != cudaSuccess) s = ft_fail(FAST_CUDA_ERROR, "binarize: %s", cudaGetErrorString(e));
    cudaStreamDestroy(st);
    return s;
}

}  // extern "C"
