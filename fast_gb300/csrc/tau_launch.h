// Host-side launchers of the device kernels (one translation unit per
// precision family so the build compiles them in parallel).
#pragma once
#include <cuda_runtime.h>
#include "tau_types.h"

namespace ft {

enum class Step {
    INIT_CG, INIT_BI, CG1, CG2, BI_RESTART, BI1, BI2, BI3, REPLACE_CG, REPLACE_BI, BI_K1, BI_K2, CG_F,
    REPLACE_CG_FF, REPLACE_BI_FF  // the replacement with a float-float iterate (opt-in)
};

// Pure-precision solves: `f64` selects double, otherwise float (scalars in
// the solve precision, as the reference's T).
void launch_pure_f64(Step s, const Launch &L, cudaStream_t st);
void launch_pure_f32(Step s, const Launch &L, cudaStream_t st);
// FP32 iterations of a MIXED solve (scalars in double); BI_K1/BI_K2 are the
// two-sweep BiCGSTAB steps, MIXED only.
void launch_mixed_inner(Step s, const Launch &L, cudaStream_t st);
// Residual replacement of a MIXED solve (a no-op launch unless the solve
// asked for one): FP64 iterate, or float-float with `ff`.
void launch_replace(bool bicg, bool ff, const Launch &L, cudaStream_t st);
void launch_init64(const Launch &L, cudaStream_t st);
void launch_code(const Launch &L, cudaStream_t st);
// tau flux sum: src 0 = double x, 1 = float x, 2 = the current MIXED iterate
// as float-float pairs, 3 = the current MIXED iterate as doubles.
void launch_tau(int src, const Launch &L, cudaStream_t st);
// n float-float pairs at src -> n doubles at dst (device).
void launch_ff_to_double(const void *src, double *dst, int64_t n, cudaStream_t st);
// Raise the dynamic shared-memory limit of every sweep kernel (once per device).
cudaError_t configure_f64();
cudaError_t configure_f32();
cudaError_t configure_misc();

}  // namespace ft
