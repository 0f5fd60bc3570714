// Residual replacement, tau, stencil-code and initialisation kernels.
#include "tau_launch.h"
#include "tau_misc.cuh"

namespace ft {

constexpr int kStages = 3;

// The replacement slot runs at the head of every iteration and is idle in
// most: its kernels walk the tiles with one resident wave of blocks
// (sweep_kernel_tiles), sized here from the occupancy of each kernel.
int g_resident_bi = 0, g_resident_cg = 0;

void launch_replace(bool bicg, const Launch &L, cudaStream_t st)
{
    const int64_t resident = bicg ? g_resident_bi : g_resident_cg;
    const unsigned grid = (unsigned)(L.nblocks < resident ? L.nblocks : resident);
    if (bicg)
        sweep_kernel_tiles<OpReplaceBi2, kStages>
            <<<grid, NTHREADS, sweep_dyn_smem<OpReplaceBi2, kStages>(), st>>>(L);
    else
        sweep_kernel_tiles<OpReplace<false>, kStages>
            <<<grid, NTHREADS, sweep_dyn_smem<OpReplace<false>, kStages>(), st>>>(L);
}

template <class Op>
static cudaError_t configure_tiles(int &resident)
{
    cudaError_t e = cudaFuncSetAttribute(sweep_kernel_tiles<Op, kStages>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         sweep_dyn_smem<Op, kStages>());
    int per_sm = 0, dev = 0, sms = 0;
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_kernel_tiles<Op, kStages>, NTHREADS,
                                                          sweep_dyn_smem<Op, kStages>());
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    resident = (per_sm < 1 ? 1 : per_sm) * (sms < 1 ? 1 : sms);
    return e;
}

cudaError_t configure_misc()
{
    cudaError_t a = configure_tiles<OpReplaceBi2>(g_resident_bi);
    cudaError_t b = configure_tiles<OpReplace<false>>(g_resident_cg);
    return a != cudaSuccess ? a : b;
}

void launch_init64(const Launch &L, cudaStream_t st) { init64_kernel<<<(unsigned)L.nblocks, NTHREADS, 0, st>>>(L); }

void launch_code(const Launch &L, cudaStream_t st) { code_kernel<<<(unsigned)L.nblocks, NTHREADS, 0, st>>>(L); }

void launch_tau(int src, const Launch &L, cudaStream_t st)
{
    if (src == 1) tau_kernel<float><<<(unsigned)L.nblocks, NTHREADS, 0, st>>>(L, 0);
    else if (src == 2) tau_kernel<FF><<<(unsigned)L.nblocks, NTHREADS, 0, st>>>(L, 1);
    else tau_kernel<double><<<(unsigned)L.nblocks, NTHREADS, 0, st>>>(L, 0);
}

void launch_ff_to_double(const void *src, double *dst, int64_t n, cudaStream_t st)
{
    int64_t blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    if (blocks < 1) blocks = 1;
    ff_to_double_kernel<<<(unsigned)blocks, 256, 0, st>>>((const float2 *)src, dst, n);
}

}  // namespace ft
