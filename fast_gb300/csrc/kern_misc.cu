// Residual replacement, tau, stencil-code and initialisation kernels.
#include "tau_launch.h"
#include "tau_misc.cuh"

namespace ft {

constexpr int kStages = 3;

void launch_replace(bool bicg, const Launch &L, cudaStream_t st)
{
    if (bicg)
        sweep_kernel<OpReplaceBi2, kStages>
            <<<(unsigned)L.nblocks, NTHREADS, sweep_dyn_smem<OpReplaceBi2, kStages>(), st>>>(L);
    else
        sweep_kernel<OpReplace<false>, kStages>
            <<<(unsigned)L.nblocks, NTHREADS, sweep_dyn_smem<OpReplace<false>, kStages>(), st>>>(L);
}

cudaError_t configure_misc()
{
    cudaError_t a = cudaFuncSetAttribute(sweep_kernel<OpReplaceBi2, kStages>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         sweep_dyn_smem<OpReplaceBi2, kStages>());
    cudaError_t b = cudaFuncSetAttribute(sweep_kernel<OpReplace<false>, kStages>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         sweep_dyn_smem<OpReplace<false>, kStages>());
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
