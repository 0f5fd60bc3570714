// Device building blocks of the matrix-free tortuosity solvers.
//
// The operator is the reference's 7-point finite-volume diffusion system
// (fastlib/src/cuda/Diffusion.cuh:54-148) evaluated on the fly from a one-byte
// stencil code per voxel instead of 7 stored coefficient arrays
// (fastlib/src/cuda/Diffusion.cu:30-71 writes those).  All coefficients are in
// h = 1 units: the reference's coefficients are Dface*h^2/dist = Dface*h for
// interior faces and 2*D*h for the two Dirichlet faces; dividing A and b by h
// leaves x, every solver scalar ratio and tau unchanged.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <type_traits>
#include "tau_types.h"

namespace ft {

// ---------------------------------------------------------------------------
// Coefficient tables, staged in shared memory at block start.
//
// The FP32 iterations of a MIXED solve look up the diagonal of EVERY voxel in
// a table indexed by its
// stencil code and its boundary count bc = (missing secondary-axis
// neighbours) - (missing primary-axis neighbours), bc in [-2, 4]: a missing
// neighbour's code bit repeats the voxel's own bit, so the interior entry
// counts D_self for it, which a zero-flux face must give back (+D_self) and a
// Dirichlet face must double (-D_self: 2*D_self in all).  The count is fixed
// per thread in x and y for a whole slab and changes only on the first and
// last plane in z, so the lookup has no branch.  FP64 solves and the
// reference's FP32 mode keep the coordinate-aware evaluation in the
// reference's subtraction order for voxels on a domain face (row 2 of the FP32
// table is the interior diagonal they use).
// ---------------------------------------------------------------------------
constexpr int NBC = 7;  // boundary counts -2..4

// FAST_TAU_BOUNDS_CHECK=1 builds check every global access that TMA does not
// bound (the plain loads and stores): an index outside its array records the
// site in the right-hand side's scalars (the first one to fail) and the access
// is skipped; the host reports the record as FAST_CUDA_ERROR.  Off (and free)
// by default.
#ifndef FAST_TAU_BOUNDS_CHECK
#define FAST_TAU_BOUNDS_CHECK 0
#endif
enum OobSite { OOB_SWEEP_STORE = 1, OOB_PARTIALS = 2, OOB_CODE = 3, OOB_INIT = 4, OOB_TAU = 5 };

// [lo, hi] inside [0, n)?
__device__ __forceinline__ bool ft_in(const Job &J, int64_t lo, int64_t hi, int64_t n, int site)
{
#if FAST_TAU_BOUNDS_CHECK
    if (lo >= 0 && hi < n) return true;
    atomicCAS(&J.sc->oob, 0, site);
    return false;
#else
    (void)J; (void)lo; (void)hi; (void)n; (void)site;
    return true;
#endif
}

// Float-float number: value = hi + lo, |lo| <= ulp(hi) / 2, about 48
// significant bits.  The MIXED residual replacement keeps its iterate and
// evaluates b - A x in this form with FP32 instructions (error-free
// transformations: Knuth's two-sum, Dekker's product through a fused
// multiply-add), because FP64 throughput on this GPU is a small fraction of
// FP32's.
struct FF {
    float hi, lo;
    FF() = default;
    __host__ __device__ constexpr FF(int v) : hi((float)v), lo(0.f) {}
    __host__ __device__ constexpr FF(float h, float l) : hi(h), lo(l) {}
};

template <typename T>
struct Coef {
    static constexpr int NB = sizeof(T) == 4 ? NBC : 1;
    T face[2][2];      // face coefficient by (self solid, neighbour solid)
    T cell2[2];        // 2*D: the half-cell Dirichlet face (dist = h/2)
    T diag_b[NB][128]; // diagonal by (boundary count + 2, code); FP64: interior row only
    T inv_b[NB][128];  // its reciprocal
};

// FP32: the diagonal and its inverse interleaved, {diag, 1/diag}, so that
// a voxel that needs both reads one 8-byte entry.
#ifndef FAST_TAU_FACE_TABLE
#define FAST_TAU_FACE_TABLE 1
#endif

template <>
struct Coef<float> {
    static constexpr int NB = NBC;
    float face[2][2];
    float cell2[2];
    float2 di[NBC][128];  // {diag, 1/diag} by (boundary count + 2, code)
};

// The six face coefficients of each stencil code (X+, X-, Y+, Y-, Z+, Z-):
// face[self solid][neighbour solid] selected by the code's bits.  Shared
// memory of the sweeps that read it (FAST_TAU_FACE_TABLE), not of the others.
struct FaceTable {
    float4 fxy[128];
    float2 fz[128];
};

// Fills the table (blocks of at least 128 threads).
__device__ __forceinline__ void load_face_table(FaceTable &t, const Job &J, int tid)
{
    if (tid < 128) {
        const int self = (tid >> SELF_BIT) & 1;
        auto f = [&](int d) { return J.fface[self][(tid >> d) & 1]; };
        t.fxy[tid] = make_float4(f(0), f(1), f(2), f(3));
        t.fz[tid] = make_float2(f(4), f(5));
    }
}

// Fills the block's coefficient tables; nt = the block's threads.
template <typename T>
__device__ __forceinline__ void load_coef(Coef<T> &C, const Job &J, int tid, int nt = NTHREADS)
{
    if constexpr (sizeof(T) == 8) {
        if (tid < 128) {
            C.diag_b[0][tid] = J.ddiag_int[tid];
            C.inv_b[0][tid] = J.dinv_int[tid];
        }
        if (tid < 4) C.face[tid >> 1][tid & 1] = J.dface[tid >> 1][tid & 1];
        if (tid < 2) C.cell2[tid] = 2.0 * J.dcell[tid];
    } else {
        for (int k = tid; k < NBC * 128; k += nt)
            C.di[k >> 7][k & 127] = make_float2(J.fdiag_b[k >> 7][k & 127], J.finv_b[k >> 7][k & 127]);
        if (tid < 4) C.face[tid >> 1][tid & 1] = J.fface[tid >> 1][tid & 1];
        if (tid < 2) C.cell2[tid] = (float)(2.0 * J.dcell[tid]);
    }
}

// The replacement's tables: the FP64 coefficients as float-float pairs.
template <>
struct Coef<FF> {
    static constexpr int NB = NBC;
    FF face[2][2];
    FF cell2[2];
    float dhi[NBC][128], dlo[NBC][128];  // diagonal by (boundary count + 2, code)
};

template <>
__device__ __forceinline__ void load_coef<FF>(Coef<FF> &C, const Job &J, int tid, int nt)
{
    for (int k = tid; k < NBC * 128; k += nt) {
        C.dhi[k >> 7][k & 127] = J.xdiag_hi[k >> 7][k & 127];
        C.dlo[k >> 7][k & 127] = J.xdiag_lo[k >> 7][k & 127];
    }
    if (tid < 4) C.face[tid >> 1][tid & 1] = FF(J.xface[tid >> 1][tid & 1][0], J.xface[tid >> 1][tid & 1][1]);
    if (tid < 2) C.cell2[tid] = FF(J.xcell2[tid][0], J.xcell2[tid][1]);
}

// Face coefficients of a solve, held in registers by every thread.
template <typename T>
struct Faces {
    T a0, b0, a1, b1;  // (self pore: neighbour pore, solid), (self solid: pore, solid)
};

template <typename T>
__device__ __forceinline__ Faces<T> faces_of(const Job &J)
{
    if constexpr (std::is_same<T, FF>::value) {
        auto f = [&](int s, int n) { return FF(J.xface[s][n][0], J.xface[s][n][1]); };
        return Faces<T>{f(0, 0), f(0, 1), f(1, 0), f(1, 1)};
    } else if constexpr (sizeof(T) == 8) {
        return Faces<T>{J.dface[0][0], J.dface[0][1], J.dface[1][0], J.dface[1][1]};
    } else {
        return Faces<T>{J.fface[0][0], J.fface[0][1], J.fface[1][0], J.fface[1][1]};
    }
}

// A voxel of a sweep: coordinates and its boundary count (see above).
struct Pos {
    int x, y, z, bc;
};

struct Geo {
    int nx, ny, nz;
    int k;     // primary axis
    int sgn;   // +1 for *_POS, -1 for *_NEG
    int P;     // row pitch of the state arrays, elements
    __device__ __forceinline__ bool in(int x, int y, int z) const
    {
        return (unsigned)x < (unsigned)nx && (unsigned)y < (unsigned)ny && (unsigned)z < (unsigned)nz;
    }
    __device__ __forceinline__ bool interior(int x, int y, int z) const
    {
        return x > 0 && y > 0 && z > 0 && x < nx - 1 && y < ny - 1 && z < nz - 1;
    }
    __device__ __forceinline__ int64_t idx(int x, int y, int z) const
    {
        return (int64_t)x + (int64_t)P * ((int64_t)y + (int64_t)ny * (int64_t)z);
    }
    __device__ __forceinline__ int coord(int x, int y, int z) const { return k == 0 ? x : (k == 1 ? y : z); }
    __device__ __forceinline__ int extent() const { return k == 0 ? nx : (k == 1 ? ny : nz); }
};

// Boundary count contributions: in x and y (fixed per thread for a slab)
// and in z (per plane).
__device__ __forceinline__ int boundary_count_xy(const Geo &g, int x, int y)
{
    const int mx = (x == 0) + (x == g.nx - 1), my = (y == 0) + (y == g.ny - 1);
    return (g.k == 0 ? -mx : mx) + (g.k == 1 ? -my : my);
}

__device__ __forceinline__ int boundary_count_z(const Geo &g, int z)
{
    const int mz = (z == 0) + (z == g.nz - 1);
    return g.k == 2 ? -mz : mz;
}

// Diagonal of voxel (x,y,z): 0 - c(X+) - c(X-) - c(Y+) - c(Y-) - c(Z+) - c(Z-),
// the subtraction order of getSystemTopKernel (Diffusion.cuh:85-105).  A
// face to an in-domain neighbour contributes its face coefficient; a domain
// face on the primary axis contributes the half-cell Dirichlet term 2*D; a
// domain face on a secondary axis is zero-flux and contributes nothing.
template <typename T>
__device__ __forceinline__ T diag_general(const Coef<T> &C, const Geo &g, uint32_t code, int x, int y, int z)
{
    const int self = (code >> SELF_BIT) & 1;
    T d = T(0);
    if (x + 1 < g.nx) d -= C.face[self][code & 1];        else if (g.k == 0) d -= C.cell2[self];
    if (x > 0)        d -= C.face[self][(code >> 1) & 1]; else if (g.k == 0) d -= C.cell2[self];
    if (y + 1 < g.ny) d -= C.face[self][(code >> 2) & 1]; else if (g.k == 1) d -= C.cell2[self];
    if (y > 0)        d -= C.face[self][(code >> 3) & 1]; else if (g.k == 1) d -= C.cell2[self];
    if (z + 1 < g.nz) d -= C.face[self][(code >> 4) & 1]; else if (g.k == 2) d -= C.cell2[self];
    if (z > 0)        d -= C.face[self][(code >> 5) & 1]; else if (g.k == 2) d -= C.cell2[self];
    return d;
}

// Diagonal and its inverse of the voxel at p.  FAST (the FP32 iterations of
// a MIXED solve): the boundary-count table, no branch.  Otherwise (FP64 and
// the reference's FP32 mode): the interior table, or the coordinate-aware
// evaluation in the reference's subtraction order for a voxel on a domain
// face (BND_BIT of its code).
template <typename T>
__host__ __device__ constexpr int interior_row() { return Coef<T>::NB == 1 ? 0 : 2; }

// Interior entries of the tables: row `row` (FP32 boundary-count row, or
// the single FP64 row), diagonal and inverse.
template <typename T>
__device__ __forceinline__ T tab_diag(const Coef<T> &C, int row, uint32_t code)
{
    if constexpr (std::is_same<T, float>::value) return C.di[row][code & 127].x;
    else return C.diag_b[row][code & 127];
}

template <typename T>
__device__ __forceinline__ T tab_inv(const Coef<T> &C, int row, uint32_t code)
{
    if constexpr (std::is_same<T, float>::value) return C.di[row][code & 127].y;
    else return C.inv_b[row][code & 127];
}

template <typename T, bool FAST>
__device__ __forceinline__ T diag_of(const Coef<T> &C, const Geo &g, uint32_t code, const Pos &p)
{
    if constexpr (FAST) {
        return tab_diag(C, p.bc + 2, code);
    } else {
        if (code & (1u << BND_BIT)) return diag_general(C, g, code, p.x, p.y, p.z);
        return tab_diag(C, interior_row<T>(), code);
    }
}

// {diagonal, inverse} of the voxel at p (FP32).
template <bool FAST>
__device__ __forceinline__ float2 dinv_of(const Coef<float> &C, const Geo &g, uint32_t code, const Pos &p);

// The diagonal and its inverse together: one table entry in FP32.
template <typename T, bool FAST>
__device__ __forceinline__ void diag_inv(const Coef<T> &C, const Geo &g, uint32_t code, const Pos &p, T &d, T &inv);

// {diagonal, inverse} of the voxel at p (FP32).
template <bool FAST>
__device__ __forceinline__ float2 dinv_of(const Coef<float> &C, const Geo &g, uint32_t code, const Pos &p)
{
    if constexpr (FAST) {
        return C.di[p.bc + 2][code & 127];
    } else {
        if (code & (1u << BND_BIT)) {
            const float d = diag_general(C, g, code, p.x, p.y, p.z);
            return make_float2(d, 1.0f / d);
        }
        return C.di[interior_row<float>()][code & 127];
    }
}

template <typename T, bool FAST>
__device__ __forceinline__ T inv_from_diag(const Coef<T> &C, uint32_t code, const Pos &p, T d);

template <typename T, bool FAST>
__device__ __forceinline__ void diag_inv(const Coef<T> &C, const Geo &g, uint32_t code, const Pos &p, T &d, T &inv)
{
    if constexpr (std::is_same<T, float>::value) {
        const float2 di = dinv_of<FAST>(C, g, code, p);
        d = di.x;
        inv = di.y;
    } else {
        d = diag_of<T, FAST>(C, g, code, p);
        inv = inv_from_diag<T, FAST>(C, code, p, d);
    }
}

template <typename T, bool FAST>
__device__ __forceinline__ T inv_of(const Coef<T> &C, const Geo &g, uint32_t code, const Pos &p)
{
    if constexpr (FAST) {
        return tab_inv(C, p.bc + 2, code);
    } else {
        if (code & (1u << BND_BIT)) return T(1) / diag_general(C, g, code, p.x, p.y, p.z);
        return tab_inv(C, interior_row<T>(), code);
    }
}

// The inverse when the diagonal d of the voxel is already at hand.
template <typename T, bool FAST>
__device__ __forceinline__ T inv_from_diag(const Coef<T> &C, uint32_t code, const Pos &p, T d)
{
    if constexpr (FAST) {
        return tab_inv(C, p.bc + 2, code);
    } else {
        return (code & (1u << BND_BIT)) ? T(1) / d : tab_inv(C, interior_row<T>(), code);
    }
}

// Right-hand side b (Diffusion.cuh:108-122): on the first plane of the
// primary axis b = -2D * cBegin, else on the last plane b = -2D * cEnd, with
// cBegin = 1, cEnd = 0 for a positive direction and the reverse for a negative
// one.  `else if`: a one-plane axis only gets the cBegin term.
template <typename T>
__device__ __forceinline__ T rhs_at(const Coef<T> &C, const Geo &g, uint32_t code, int x, int y, int z)
{
    const int c = g.coord(x, y, z);
    const int self = (code >> SELF_BIT) & 1;
    if (c == 0) return (g.sgn > 0) ? -C.cell2[self] : T(0);
    if (c == g.extent() - 1) return (g.sgn > 0) ? T(0) : -C.cell2[self];
    return T(0);
}

// Initial guess (Diffusion.cuh:127-131): linear profile along the primary axis.
template <typename T>
__device__ __forceinline__ T x0_at(const Geo &g, int x, int y, int z)
{
    const int c = g.coord(x, y, z);
    const T q = T(c) / T(g.extent() + 1);
    return (g.sgn > 0) ? (T(1.0f) - q) : q;
}

// y = A f at a voxel given the field at the voxel and its 6 neighbours, in
// the reference's summation order X+,X-,Y+,Y-,Z+,Z-,diag
// (LinearSystemDevice.cuh:67-80).  A neighbour outside the domain carries a
// field value of exactly 0 (the sweep writes 0 there), which drops its term
// just as the reference's zeroed boundary coefficient does; no bounds test is
// needed.
template <typename T>
__device__ __forceinline__ T stencil7(const Faces<T> &F, uint32_t code, T fc, T fxp, T fxm, T fyp, T fym, T fzp,
                                      T fzm, T diag)
{
    const bool solid = (code >> SELF_BIT) & 1;
    const T a = solid ? F.a1 : F.a0, b = solid ? F.b1 : F.b0;
    T s = fxp * ((code & 1) ? b : a);
    s += fxm * ((code & 2) ? b : a);
    s += fyp * ((code & 4) ? b : a);
    s += fym * ((code & 8) ? b : a);
    s += fzp * ((code & 16) ? b : a);
    s += fzm * ((code & 32) ? b : a);
    s += fc * diag;
    return s;
}

// The stencil with the six face coefficients of the code taken from one
// shared-memory table entry (FP32) instead of selected by its code bits: the
// same products in the same order, so the same result.  Measured per kernel:
// faster for the BiCGSTAB sweeps, slower for the PCG sweeps, which keep the
// bit selects (stencil7).
template <typename T>
__device__ __forceinline__ T stencil7t(const FaceTable &t, uint32_t code, T fc, T fxp, T fxm, T fyp, T fym, T fzp,
                                       T fzm, T diag)
{
    static_assert(std::is_same<T, float>::value, "FP32 table");
    {
        const float4 q = t.fxy[code & 127];
        const float2 r = t.fz[code & 127];
        T s = fxp * q.x;
        s += fxm * q.y;
        s += fyp * q.z;
        s += fym * q.w;
        s += fzp * r.x;
        s += fzm * r.y;
        s += fc * diag;
        return s;
    }
}

// The same stencil in float-float arithmetic (the MIXED residual
// replacement), same summation order; `diag` from the float-float table.
__device__ __forceinline__ FF stencil7_ff(const Faces<FF> &F, uint32_t code, FF fc, FF fxp, FF fxm, FF fyp, FF fym,
                                          FF fzp, FF fzm, FF diag);

// ---------------------------------------------------------------------------
// Dot-product accumulation.  FP64 solves accumulate in double.  FP32 solves
// accumulate each thread's products in FP32 (at most one slab column, a few
// dozen terms), combine the threads of a block with compensated (two-sum)
// FP32 arithmetic, and hand each block's (sum, error) pair to the grid level
// as a double.  Every level has a fixed order, so reductions are
// deterministic run to run.
// ---------------------------------------------------------------------------
template <typename T>
struct Acc;

template <>
struct Acc<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double v) { s += v; }
    __device__ __forceinline__ void add_prod(double a, double b) { s = fma(a, b, s); }
    __device__ __forceinline__ double hi() const { return s; }
    __device__ __forceinline__ double lo() const { return 0.0; }
};

template <>
struct Acc<float> {
    float s = 0.f;
    __device__ __forceinline__ void add(float v) { s += v; }
    __device__ __forceinline__ void add_prod(float a, float b) { s = fmaf(a, b, s); }
    __device__ __forceinline__ float hi() const { return s; }
    __device__ __forceinline__ float lo() const { return 0.f; }
};

// Error-free transformation a + b = s + e (Knuth's two-sum).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}

// (s, c) += (s2, c2), compensated.
__device__ __forceinline__ void pair_add(float &s, float &c, float s2, float c2)
{
    float t, e;
    two_sum(s, s2, t, e);
    s = t;
    c = __fadd_rn(__fadd_rn(c, c2), e);
}

// Float-float arithmetic (value = hi + lo).
// (s, e) -> (hi, lo) with hi = fl(s + e); a full two-sum, since near a
// converged residual e need not be smaller than s.
__device__ __forceinline__ FF ff_renorm(float s, float e)
{
    float h, l;
    two_sum(s, e, h, l);
    return FF(h, l);
}

__device__ __forceinline__ FF ff_add(FF a, FF b)
{
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    return ff_renorm(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ FF ff_add_f(FF a, float b)
{
    float s, e;
    two_sum(a.hi, b, s, e);
    return ff_renorm(s, __fadd_rn(e, a.lo));
}

__device__ __forceinline__ FF ff_neg(FF a) { return FF(-a.hi, -a.lo); }
__device__ __forceinline__ FF operator-(FF a) { return ff_neg(a); }

__device__ __forceinline__ float ff_to_float(FF a) { return __fadd_rn(a.hi, a.lo); }

// Accumulator of a sum of float-float products: hi parts in an error-free
// two-sum chain, every error and low-order term in one float, normalised once.
struct FFSum {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add_prod(FF a, FF b)
    {
        const float p = __fmul_rn(a.hi, b.hi);
        float pl = __fmaf_rn(a.hi, b.hi, -p);  // exact error of the product
        pl = __fmaf_rn(a.hi, b.lo, pl);
        pl = __fmaf_rn(a.lo, b.hi, pl);
        float t, e;
        two_sum(s, p, t, e);
        s = t;
        c = __fadd_rn(c, __fadd_rn(e, pl));
    }
    __device__ __forceinline__ FF value() const { return ff_renorm(s, c); }
};

__device__ __forceinline__ FF stencil7_ff(const Faces<FF> &F, uint32_t code, FF fc, FF fxp, FF fxm, FF fyp, FF fym,
                                          FF fzp, FF fzm, FF diag)
{
    const bool solid = (code >> SELF_BIT) & 1;
    const FF a = solid ? F.a1 : F.a0, b = solid ? F.b1 : F.b0;
    FFSum s;
    s.add_prod(fxp, (code & 1) ? b : a);
    s.add_prod(fxm, (code & 2) ? b : a);
    s.add_prod(fyp, (code & 4) ? b : a);
    s.add_prod(fym, (code & 8) ? b : a);
    s.add_prod(fzp, (code & 16) ? b : a);
    s.add_prod(fzm, (code & 32) ? b : a);
    s.add_prod(fc, diag);
    return s.value();
}

__device__ __forceinline__ FF diag_ff(const Coef<FF> &C, uint32_t code, const Pos &p)
{
    return FF(C.dhi[p.bc + 2][code & 127], C.dlo[p.bc + 2][code & 127]);
}

// Sum NV per-thread values over the block (fixed tree) and store the block
// totals, as doubles, to out[0..NV).  FP32 values are combined as
// compensated (sum, error) pairs.  NT = the block's threads.
template <int NV, typename V, int NT = NTHREADS>
__device__ __forceinline__ void block_sum_store(const V (&v)[NV], double *out, double *s_red /* [NV][2*NT/32] */)
{
    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    constexpr int NW = NT / 32;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        if constexpr (sizeof(V) == 8) {
            double a = (double)v[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
            if (lane == 0) s_red[k * 2 * NW + warp] = a;
        } else {
            float a = (float)v[k], c = 0.f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float a2 = __shfl_down_sync(0xffffffffu, a, o);
                const float c2 = __shfl_down_sync(0xffffffffu, c, o);
                pair_add(a, c, a2, c2);
            }
            if (lane == 0) {
                s_red[k * 2 * NW + warp] = (double)a;
                s_red[k * 2 * NW + NW + warp] = (double)c;
            }
        }
    }
    __syncthreads();
    if (tid < NV) {
        double a = 0.0;
        if constexpr (sizeof(V) == 8) {
#pragma unroll
            for (int w = 0; w < NW; w++) a += s_red[tid * 2 * NW + w];
        } else {
            float s = 0.f, c = 0.f;
#pragma unroll
            for (int w = 0; w < NW; w++) pair_add(s, c, (float)s_red[tid * 2 * NW + w], (float)s_red[tid * 2 * NW + NW + w]);
            a = (double)s + (double)c;
        }
        out[tid] = a;
    }
}

// Arrival of a block at the end of a kernel.  Returns true (block-uniform)
// in the last block to arrive for this job; that block then sums all
// partials of the job, in a fixed order.
__device__ __forceinline__ bool arrive_last(uint32_t *counter, int64_t ntiles, int *s_flag)
{
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t prev = atomicAdd(counter, 1u);
        *s_flag = (prev == (uint32_t)(ntiles - 1)) ? 1 : 0;
    }
    __syncthreads();
    return *s_flag != 0;
}

template <int NV, int NT = NTHREADS>
__device__ __forceinline__ void sum_partials(const double *part, int64_t ntiles, double (&tot)[NV], double *s_red)
{
    const int tid = threadIdx.x;
    __threadfence();
    double v[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) v[k] = 0.0;
    for (int64_t t = tid; t < ntiles; t += NT) {
#pragma unroll
        for (int k = 0; k < NV; k++) v[k] += __ldcg(part + t * NPART + k);
    }
    __shared__ double s_tot[NV];
    block_sum_store<NV, double, NT>(v, s_tot, s_red);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; k++) tot[k] = s_tot[k];
}

// Locate the job of this block (jobs are laid out back to back by tile_base).
__device__ __forceinline__ int find_job(const Launch &L, int64_t b)
{
    int lo = 0, hi = L.njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (L.jobs[mid].tile_base <= b) lo = mid; else hi = mid - 1;
    }
    return lo;
}

}  // namespace ft
