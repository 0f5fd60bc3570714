// Internal types shared by the host orchestration and the device kernels.
#pragma once
#include <cuda.h>
#include <stdint.h>

namespace ft {

// Tile of one thread block: TX x TY columns marching over ZC planes in z.
// Each thread owns two neighbouring x columns (LANES), so a row of TX
// voxels is TPR threads; NTHREADS = 256 threads cover the TX * TY = 512
// columns with one row each (a sweep with two rows per thread runs
// NTHREADS / 2).
#ifndef FAST_TAU_TX
#define FAST_TAU_TX 64
#endif
constexpr int TX = FAST_TAU_TX;
constexpr int LANES = 2;
constexpr int TPR = TX / LANES;
constexpr int TY = 256 / TPR;
constexpr int NTHREADS = TPR * TY;
static_assert(NTHREADS == 256 && TX % 16 == 0, "tile must be 256 threads, 16-element aligned in x");
constexpr int HY = TY + 2;   // tile rows + one halo row on each side
constexpr int NPART = 4;     // partial sums per block per kernel

// Stencil code byte: bit d (d = 0..5, Dir order X_POS, X_NEG, Y_POS, Y_NEG,
// Z_POS, Z_NEG) = neighbour d is solid; bit 6 = the voxel itself is solid;
// bit 7 = the voxel lies on a face of the domain (some neighbour is outside).
// Out-of-domain neighbours repeat the voxel's own bit (the reference's
// clamped neighbour, fastlib/src/solver/Diffusion.cpp:51-62).
constexpr int SELF_BIT = 6;
constexpr int BND_BIT = 7;

enum SolveState : int32_t {
    RUNNING = 0,
    CONVERGED = 1,
    MAXITER = 2,
    DIVERGED = 3,
    ZERO_RHS = 4,
    FAULT = 6,     // a bounded device-side wait ran out (tile loads did not arrive)
};

// Tensor maps of a job's arrays (TMA descriptors), by array.
enum TensorMapId : int {
    TM_CODE = 0, TM_X = 1, TM_R = 2 /* +parity */, TM_R0 = 4, TM_P = 5 /* +parity */, TM_V = 7 /* +parity */,
    TM_X64 = 9 /* +parity */, TM_T = 11,
    // the same arrays with the TX x TY tile as the box (streams read only at
    // a block's own points): x, r[0], r0
    TM_XI = 12, TM_RI = 13, TM_R0I = 14, NTM = 15
};

// Per right-hand-side solver scalars, resident in device memory and updated
// by the last block of each kernel ("finisher").
struct Scalars {
    double rhs_sq;      // |b|^2 of the system being iterated
    double tol2;        // tol^2 |b|^2 (in solve precision)
    double tol;         // relative tolerance of the system being iterated
    double rsq;         // |r|^2 (recursive)
    double zr;          // CG: r.z
    double alpha, beta; // CG/BiCGSTAB
    double rho, omega;  // BiCGSTAB
    double rho_old;     // BiCGSTAB rho of the previous iteration (for a restart)
    double r0_sq;       // BiCGSTAB |r0|^2
    double div_thresh;  // divergence threshold on rsq (1e11 scaled to h=1 units)
    double eps2;        // BiCGSTAB restart threshold eps(T)^2
    uint64_t iter;      // iterations, reference counting
    uint64_t max_iter;  // iteration limit
    uint64_t restarts;
    int32_t state;      // SolveState
    int32_t restart;    // BiCGSTAB: restart pending before the next iteration
    // MIXED: FP32 iterations on the correction e of an FP64 iterate x64, with
    // the recursive residual replaced by fp32(b - A (x64 + e)) computed in
    // FP64 (x64 += e, e = 0) whenever `replace` is set.
    double tol_outer;   // requested relative tolerance on the FP64 residual
    double r64_sq;      // |b - A x64|^2 at the last replacement
    double b64_sq;      // |b|^2 in FP64
    double rsq_max;     // largest recursive |r|^2 since the last replacement
    double delta2;      // replace once |r|^2 < delta2 * rsq_max
    double cos2_min;    // BiCGSTAB: restart once (r0.r)^2 < cos2_min |r0|^2 |r|^2
    int32_t replace;    // 0: none pending, 1: residual replacement, 2: replacement + Krylov restart
    int32_t e_reset;    // 1: the next step-1 kernel zeroes e
    int32_t outer_steps;    // residual replacements done
    int32_t x64_cur;        // which x64 buffer holds the current iterate
    int32_t inner_mode;     // 1: MIXED solve
    int32_t k1_mode;        // two-sweep BiCGSTAB: 1 = the next step 1 takes r from t (just replaced), e = 0;
                            // one-sweep CG: 1 = the next sweep restarts from the replaced residual
    int32_t cg_fused;       // 1: MIXED CG runs as one sweep per iteration (OpCGF)
    int32_t oob;            // bounds-check builds: first failing access site (0 = none)
    int32_t test_withhold;  // test-hook builds: withhold one tile load of the next sweep (see tau_sweep.cuh)
    int32_t pad_hook;
    // reductions for tau and porosity
    double flux_sum;    // sum over voxels of the tau flux term
    uint64_t pores;     // number of zero (pore) voxels
    double dbg[4];      // the last kernel's reduced dot products (tracing)
};

// One right-hand side (a direction of a volume) inside a launch.  Arrays
// are x-fastest with a row pitch of `pitch` elements (nx rounded up to 16) so
// every row starts on a 16-byte boundary, as TMA requires.
struct Job {
    CUtensorMap tm[NTM];         // TMA descriptors of the arrays below
    int32_t pitch;               // row pitch in elements (all arrays of the volume)
    int32_t nx, ny, nz;
    int32_t dir;                 // 0..5
    int32_t tiles_x, tiles_y, tiles_z;
    int32_t zc;                  // planes per block
    int64_t tile_base;           // first block index of this job in the launch
    int64_t ntiles;
    const uint8_t *code;         // stencil codes, N bytes
    const uint8_t *mask;         // raw mask (tau and porosity)
    void *x;                     // solution (T); MIXED: FP32 correction e
    void *r[2];                  // residual ping-pong (T)
    void *r0;                    // BiCGSTAB shadow residual (T)
    void *p[2];                  // search direction ping-pong (T)
    void *v[2];                  // BiCGSTAB v ping-pong (T)
    void *t;                     // MIXED BiCGSTAB: t = A s, kept from step 2 to step 1 (FP32)
    void *x64[2];                // MIXED extended-precision iterate ping-pong: double, or float-float
                                 // (hi, lo) pairs when x64_ff is set
    Scalars *sc;
    double *part;                // ntiles * NPART partial sums
    uint32_t *counter;           // finisher arrival counter
    // Coefficients in h = 1 units (the reference's values divided by the
    // cell size h; tau and x are invariant to a common scale of A and b).
    double dface[2][2];          // face coefficient by (self solid, neighbour solid)
    double dcell[2];             // cell diffusivity by solid bit (pore, solid)
    float fface[2][2];
    float fdiag_b[7][128];       // FP32 diagonal by (boundary count + 2, code 7 bits)
    float finv_b[7][128];        // 1/diag, FP32
    double ddiag_int[128];       // interior diagonal, FP64
    double dinv_int[128];        // 1/diag, FP64
    // MIXED residual replacement in float-float (x64_ff): the FP64 values
    // above as pairs (value = hi + lo), the diagonal by (boundary count + 2, code).
    float xdiag_hi[7][128], xdiag_lo[7][128];
    float xface[2][2][2];        // [self solid][neighbour solid][hi, lo]
    float xcell2[2][2];          // 2*D by solid bit, [hi, lo]
    float c_tau[2];              // tau cell coefficients (float coeffs of the reference)
    int32_t x64_ff;              // MIXED: 1 = x64 holds float-float pairs, 0 = doubles
    int32_t pad0;
};

struct Launch {
    Job *jobs;          // device array
    int32_t njobs;
    int32_t pad;
    int64_t nblocks;    // total blocks = sum of job tiles
    // MIXED: one device word, nonzero while a residual replacement is
    // pending for some right-hand side of the launch (null otherwise).  The
    // replacement kernel's blocks leave at once while it is zero; the first
    // sweep after the slot clears it and any sweep that asks sets it.
    uint32_t *gate;
};

}  // namespace ft
