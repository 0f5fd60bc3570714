// FP32 solver kernels: the reference's `-p float` (float scalars) and the
// inner iterations of the MIXED solve (double scalars).
#include "tau_launch.h"
#include "tau_sweep.cuh"

namespace ft {

#ifndef FAST_TAU_STAGES_F32
#define FAST_TAU_STAGES_F32 4
#endif
// Depth of the TMA stage ring (planes of every operand in flight per block).
constexpr int kStages = FAST_TAU_STAGES_F32;

#ifndef FAST_TAU_STAGES_K1
#define FAST_TAU_STAGES_K1 3
#endif
// The two-sweep BiCGSTAB step 1 reads seven streams per plane: a 3-stage ring
// and a register bound of three blocks per SM fit three blocks (the compiler's
// own choice and a 4-stage ring fit two; measured 389 against 416 us per
// launch on the 256^3 x 3 workload).
constexpr int kStagesK1 = FAST_TAU_STAGES_K1;
#ifndef FAST_TAU_STAGES_CGF
#define FAST_TAU_STAGES_CGF 3
#endif
#ifndef FAST_TAU_BLOCKS_CGF
#define FAST_TAU_BLOCKS_CGF 2
#endif
constexpr int kStagesCGF = FAST_TAU_STAGES_CGF;
constexpr int kBlocksCGF = FAST_TAU_BLOCKS_CGF;
constexpr int kBlocksK1 = 3;

#ifndef FAST_TAU_STAGES_R2
#define FAST_TAU_STAGES_R2 2
#endif
#ifndef FAST_TAU_MINB_R2
#define FAST_TAU_MINB_R2 0
#endif
#ifndef FAST_TAU_STAGES_CG1
#define FAST_TAU_STAGES_CG1 3
#endif
#ifndef FAST_TAU_MINB_CG2
#define FAST_TAU_MINB_CG2 0
#endif
#ifndef FAST_TAU_MINB_K2
#define FAST_TAU_MINB_K2 7
#endif
// Ring depth and register bound of a sweep.  A sweep with two rows per
// thread runs half-size blocks, which the fixed shared memory of a block
// (plane buffers, tables) already limits to few per SM: its stage ring is
// shorter (FAST_TAU_STAGES_R2), and a minimum of blocks per SM > 0 bounds
// its registers.  Measured per sweep (MIXED): PCG step 1 with a 3-stage
// ring (six blocks per SM either way), PCG step 2 with 2 stages (a bound of
// 72 registers was faster at 256^3 but slower at the 1024^3 depth of 256
// planes), BiCGSTAB step 2 with 2 stages and the 72-register bound.
template <class Op>
struct SweepShape {
    static constexpr int stages = RowsPerThread<Op>::n == 2 ? FAST_TAU_STAGES_R2 : kStages;
    static constexpr int minb = RowsPerThread<Op>::n == 2 ? FAST_TAU_MINB_R2 : 0;
};
template <>
struct SweepShape<OpCG1<float, double>> {
    static constexpr int stages = RowsPerThread<OpCG1<float, double>>::n == 2 ? FAST_TAU_STAGES_CG1 : kStages;
    static constexpr int minb = 0;
};
template <>
struct SweepShape<OpCG2<float, double>> {
    static constexpr int stages = RowsPerThread<OpCG2<float, double>>::n == 2 ? FAST_TAU_STAGES_R2 : kStages;
    static constexpr int minb = RowsPerThread<OpCG2<float, double>>::n == 2 ? FAST_TAU_MINB_CG2 : 0;
};
template <>
struct SweepShape<OpBiK2> {
    static constexpr int stages = RowsPerThread<OpBiK2>::n == 2 ? FAST_TAU_STAGES_R2 : kStages;
    static constexpr int minb = RowsPerThread<OpBiK2>::n == 2 ? FAST_TAU_MINB_K2 : 0;
};

template <class Op>
constexpr int stages_of()
{
    return SweepShape<Op>::stages;
}
template <class Op>
constexpr int min_blocks_of()
{
    return SweepShape<Op>::minb;
}

template <class Op, int NS = stages_of<Op>()>
static void go(const Launch &L, cudaStream_t st)
{
    constexpr int dyn = sweep_dyn_smem<Op, NS>();
    constexpr int MB = min_blocks_of<Op>();
    if constexpr (MB > 0)
        sweep_kernel_mb<Op, NS, MB><<<(unsigned)L.nblocks, sweep_threads<Op>(), dyn, st>>>(L);
    else
        sweep_kernel<Op, NS><<<(unsigned)L.nblocks, sweep_threads<Op>(), dyn, st>>>(L);
}

template <class Op, int NS = stages_of<Op>()>
static cudaError_t cfg()
{
    constexpr int MB = min_blocks_of<Op>();
    if constexpr (MB > 0)
        return cudaFuncSetAttribute(sweep_kernel_mb<Op, NS, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    sweep_dyn_smem<Op, NS>());
    else
        return cudaFuncSetAttribute(sweep_kernel<Op, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    sweep_dyn_smem<Op, NS>());
}

template <typename ST>
static void dispatch(Step s, const Launch &L, cudaStream_t st)
{
    using T = float;
    switch (s) {
    case Step::INIT_CG: go<OpInit<T, ST, false>>(L, st); break;
    case Step::INIT_BI: go<OpInit<T, ST, true>>(L, st); break;
    case Step::CG1: go<OpCG1<T, ST>>(L, st); break;
    case Step::CG2: go<OpCG2<T, ST>>(L, st); break;
    case Step::BI_RESTART: go<OpBiRestart<T, ST>>(L, st); break;
    case Step::BI1: go<OpBi1<T, ST>>(L, st); break;
    case Step::BI2: go<OpBi2<T, ST>>(L, st); break;
    case Step::BI3: go<OpBi3<T, ST>>(L, st); break;
    default: break;  // replacement steps are MIXED-only (kern_misc.cu)
    }
}

template <typename ST>
static cudaError_t configure()
{
    using T = float;
    cudaError_t e = cudaSuccess, r;
    if ((r = cfg<OpInit<T, ST, false>>()) != cudaSuccess) e = r;
    if ((r = cfg<OpInit<T, ST, true>>()) != cudaSuccess) e = r;
    if ((r = cfg<OpCG1<T, ST>>()) != cudaSuccess) e = r;
    if ((r = cfg<OpCG2<T, ST>>()) != cudaSuccess) e = r;
    if ((r = cfg<OpBiRestart<T, ST>>()) != cudaSuccess) e = r;
    if ((r = cfg<OpBi1<T, ST>>()) != cudaSuccess) e = r;
    if ((r = cfg<OpBi2<T, ST>>()) != cudaSuccess) e = r;
    if ((r = cfg<OpBi3<T, ST>>()) != cudaSuccess) e = r;
    return e;
}

cudaError_t configure_f32()
{
    cudaError_t a = configure<float>(), b = configure<double>();
    cudaError_t c = cudaFuncSetAttribute(sweep_kernel_mb<OpBiK1, kStagesK1, kBlocksK1>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         sweep_dyn_smem<OpBiK1, kStagesK1>());
    cudaError_t d = cfg<OpBiK2>();
    cudaError_t f = cudaFuncSetAttribute(sweep_kernel_mb<OpCGF, kStagesCGF, kBlocksCGF>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         sweep_dyn_smem<OpCGF, kStagesCGF>());
    if (a != cudaSuccess) return a;
    if (b != cudaSuccess) return b;
    if (f != cudaSuccess) return f;
    return c != cudaSuccess ? c : d;
}

void launch_pure_f32(Step s, const Launch &L, cudaStream_t st) { dispatch<float>(s, L, st); }
void launch_mixed_inner(Step s, const Launch &L, cudaStream_t st)
{
    if (s == Step::BI_K1)
        sweep_kernel_mb<OpBiK1, kStagesK1, kBlocksK1>
            <<<(unsigned)L.nblocks, sweep_threads<OpBiK1>(), sweep_dyn_smem<OpBiK1, kStagesK1>(), st>>>(L);
    else if (s == Step::BI_K2) go<OpBiK2>(L, st);
    else if (s == Step::CG_F)
        sweep_kernel_mb<OpCGF, kStagesCGF, kBlocksCGF>
            <<<(unsigned)L.nblocks, sweep_threads<OpCGF>(), sweep_dyn_smem<OpCGF, kStagesCGF>(), st>>>(L);
    else dispatch<double>(s, L, st);
}

}  // namespace ft
