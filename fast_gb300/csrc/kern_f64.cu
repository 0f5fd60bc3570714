// Pure FP64 solver kernels (the reference's `-p double`).
#include "tau_launch.h"
#include "tau_sweep.cuh"

namespace ft {

#ifndef FAST_TAU_STAGES_F64
#define FAST_TAU_STAGES_F64 3
#endif
// Depth of the TMA stage ring (planes of every operand in flight per block).
constexpr int kStages = FAST_TAU_STAGES_F64;

template <class Op>
static void go(const Launch &L, cudaStream_t st)
{
    constexpr int dyn = sweep_dyn_smem<Op, kStages>();
    sweep_kernel<Op, kStages><<<(unsigned)L.nblocks, sweep_threads<Op>(), dyn, st>>>(L);
}

template <class Op>
static cudaError_t cfg()
{
    return cudaFuncSetAttribute(sweep_kernel<Op, kStages>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                sweep_dyn_smem<Op, kStages>());
}

void launch_pure_f64(Step s, const Launch &L, cudaStream_t st)
{
    using T = double;
    switch (s) {
    case Step::INIT_CG: go<OpInit<T, T, false>>(L, st); break;
    case Step::INIT_BI: go<OpInit<T, T, true>>(L, st); break;
    case Step::CG1: go<OpCG1<T, T>>(L, st); break;
    case Step::CG2: go<OpCG2<T, T>>(L, st); break;
    case Step::BI_RESTART: go<OpBiRestart<T, T>>(L, st); break;
    case Step::BI1: go<OpBi1<T, T>>(L, st); break;
    case Step::BI2: go<OpBi2<T, T>>(L, st); break;
    case Step::BI3: go<OpBi3<T, T>>(L, st); break;
    default: break;  // replacement steps are MIXED-only (kern_misc.cu)
    }
}

cudaError_t configure_f64()
{
    using T = double;
    cudaError_t e = cudaSuccess, r;
    if ((r = cfg<OpInit<T, T, false>>()) != cudaSuccess) e = r;
    if ((r = cfg<OpInit<T, T, true>>()) != cudaSuccess) e = r;
    if ((r = cfg<OpCG1<T, T>>()) != cudaSuccess) e = r;
    if ((r = cfg<OpCG2<T, T>>()) != cudaSuccess) e = r;
    if ((r = cfg<OpBiRestart<T, T>>()) != cudaSuccess) e = r;
    if ((r = cfg<OpBi1<T, T>>()) != cudaSuccess) e = r;
    if ((r = cfg<OpBi2<T, T>>()) != cudaSuccess) e = r;
    if ((r = cfg<OpBi3<T, T>>()) != cudaSuccess) e = r;
    return e;
}

}  // namespace ft
