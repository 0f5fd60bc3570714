// MIXED FP64 residual replacement, tau flux reduction, stencil-code build
// and porosity count.
#pragma once
#include <type_traits>
#include "fp_convert.h"
#include "tau_sweep.cuh"

namespace ft {

// ===========================================================================
// Arithmetic of the MIXED iterate x64, by its storage type XT (8 bytes per
// voxel either way): double (the default: the iterate, the correction update
// and the true residual b - A x in FP64, the stencil and diagonal exactly as
// the FP64 solver evaluates them) or FF, a float-float pair (an opt-in: about
// 48 significant bits from error-free FP32 transformations, for when FP64
// throughput bounds the replacement).
// ===========================================================================
template <typename XT>
struct XArith;

// The replacement's float <-> double conversions: integer instructions
// (fp_convert.h) by default, the conversion instructions with
// FAST_TAU_INT_CVT=0.
#ifndef FAST_TAU_INT_CVT
#define FAST_TAU_INT_CVT 1
#endif

__device__ __forceinline__ double to_d(float f)
{
#if FAST_TAU_INT_CVT
    return widen_f(f);
#else
    return (double)f;
#endif
}

__device__ __forceinline__ float to_f(double d)
{
#if FAST_TAU_INT_CVT
    return narrow_d(d);
#else
    return (float)d;
#endif
}

template <>
struct XArith<double> {
    using Tab = Coef<double>;
    __device__ static double add_f(double x, float e) { return x + to_d(e); }
    __device__ static double stencil(const Faces<double> &F, const Tab &C, const Geo &g, uint32_t code,
                                     const Pos &ps, double fc, double fxp, double fxm, double fyp, double fym,
                                     double fzp, double fzm)
    {
        return stencil7<double>(F, code, fc, fxp, fxm, fyp, fym, fzp, fzm, diag_of<double, false>(C, g, code, ps));
    }
    // fp32(b - A x) and fp32(b).  b is nonzero only on the first and last
    // plane of the primary axis (where it is exact in FP32); elsewhere the
    // residual is -A x, with no FP64 subtraction and no conversion of b (the
    // FP64 pipe bounds this kernel).
    __device__ static void residual(const Tab &C, const Geo &g, uint32_t code, const Pos &ps, double ax, float &r32,
                                    float &b32)
    {
        const int c = g.coord(ps.x, ps.y, ps.z);
        if (c == 0 || c == g.extent() - 1) {
            const double b = rhs_at<double>(C, g, code, ps.x, ps.y, ps.z);
            r32 = to_f(b - ax);
            b32 = to_f(b);
        } else {
            r32 = to_f(-ax);
            b32 = 0.f;
        }
    }
};

template <>
struct XArith<FF> {
    using Tab = Coef<FF>;
    __device__ static FF add_f(FF x, float e) { return ff_add_f(x, e); }
    __device__ static FF stencil(const Faces<FF> &F, const Tab &C, const Geo &, uint32_t code, const Pos &ps,
                                 FF fc, FF fxp, FF fxm, FF fyp, FF fym, FF fzp, FF fzm)
    {
        return stencil7_ff(F, code, fc, fxp, fxm, fyp, fym, fzp, fzm, diag_ff(C, code, ps));
    }
    __device__ static void residual(const Tab &C, const Geo &g, uint32_t code, const Pos &ps, FF ax, float &r32,
                                    float &b32)
    {
        const FF b = rhs_at<FF>(C, g, code, ps.x, ps.y, ps.z);
        r32 = ff_to_float(ff_add(b, ff_neg(ax)));
        b32 = ff_to_float(b);
    }
};

// ===========================================================================
// MIXED residual replacement.  The FP32 iterations work on a correction e of
// an extended-precision iterate x64 (FP64 by default, a float-float pair on
// request; XArith above); when one of them asks for it (`replace`), this step
// folds e into x64 (x64' = x64 + e, e is zeroed by the next step-1 kernel),
// recomputes the residual b - A x64' in that precision and hands
// fp32 of it to the recursion in place of the recursive residual, keeping
// the Krylov vectors (replace = 1) or restarting them from it (replace = 2,
// also the first step of a solve).  The true residual decides convergence.
// Dots, accumulated in FP32 per thread (they steer the iteration and test
// convergence; they need no more than FP32 accuracy): |fp32(r64)|^2, |b|^2
// and, for BiCGSTAB, r0.fp32(r64) (r0 = fp32(r64) itself on a restart), for
// CG fp32(r64).z.  Streams: x64, e, code (+ r0 for BiCGSTAB).
// ===========================================================================
template <bool BICG, typename XT>
struct OpReplace {
    using T = XT;
    using X = XArith<XT>;
    using R = double;
    using SL = typename std::conditional<BICG, Streams<8, 4, 1, 4>, Streams<8, 4, 1>>::type;
    static constexpr int NV = 3;
    using Shared = Coef<float>;
    struct Vals { XT x; float e; uint32_t code; float r0; };
    struct Own { uint32_t code; float r0; };
    struct Out { XT x; float r; };
    const CUtensorMap *tmap[SL::N];
    Faces<T> F;
    XT *x64n;
    float *r, *r0, *p, *v;
    bool restart;
    Acc<float> a_rr, a_bb, a_d;

    __device__ static bool active(const Scalars &sc) { return sc.state == RUNNING && sc.replace != 0; }
    __device__ static void load_shared(Shared &S, const Job &J, int tid) { load_coef<float>(S, J, tid); }
    __device__ static void load2(const unsigned char *st, const Pt &p_, Vals &a, Vals &b)
    {
        sv2<XT, SL, 0>(st, p_, a.x, b.x);
        sv2<float, SL, 1>(st, p_, a.e, b.e);
        load_code2<SL, 2>(st, p_, a.code, b.code);
        if constexpr (BICG) sv2<float, SL, 3>(st, p_, a.r0, b.r0);
    }
    __device__ static void load1(const unsigned char *st, const Pt &p_, Vals &a)
    {
        a.x = sv<XT, SL, 0>(st, p_);
        a.e = sv<float, SL, 1>(st, p_);
    }
    __device__ void init(const Job &J, Shared &)
    {
        F = faces_of<T>(J);
        const Scalars &sc = *J.sc;
        const int cur = sc.x64_cur;
        // the residual goes where the next kernel reads it: r[iter & 1] for
        // BiCGSTAB and the one-sweep CG, r[0] for the two-sweep CG
        const int par = (BICG || sc.cg_fused) ? (int)(sc.iter & 1) : 0;
        tmap[0] = &J.tm[TM_X64 + cur];
        tmap[1] = &J.tm[TM_X];
        tmap[2] = &J.tm[TM_CODE];
        if constexpr (BICG) tmap[3] = &J.tm[TM_R0];
        x64n = (XT *)J.x64[cur ^ 1];
        r = (float *)J.r[par];
        r0 = (float *)J.r0;
        p = (float *)J.p[(int)(sc.iter & 1)];
        v = BICG ? (float *)J.v[par] : nullptr;
        restart = sc.replace == 2;
    }
    __device__ XT field(const Geo &, const typename X::Tab &, Shared &, const Vals &a, const Pos &) const
    {
        return X::add_f(a.x, a.e);
    }
    __device__ Own own(const Geo &, const typename X::Tab &, Shared &, const Vals &a, const Pos &, XT &f) const
    {
        f = X::add_f(a.x, a.e);
        return Own{a.code, a.r0};
    }
    __device__ Out apply(const Geo &g, const typename X::Tab &C, Shared &S, const Own &o, const Pos &ps, XT fc,
                         XT fxp, XT fxm, XT fyp, XT fym, XT fzp, XT fzm)
    {
        const XT ax = X::stencil(F, C, g, o.code, ps, fc, fxp, fxm, fyp, fym, fzp, fzm);
        float r32, b32;
        X::residual(C, g, o.code, ps, ax, r32, b32);
        a_rr.add_prod(r32, r32);
        a_bb.add_prod(b32, b32);
        if constexpr (BICG) {
            a_d.add_prod(restart ? r32 : o.r0, r32);
        } else {
            const float inv = inv_of<float, true>(S, g, o.code, ps);
            a_d.add_prod(r32, r32 * inv);
        }
        return Out{fc, r32};
    }
    __device__ void store(int64_t i, const Out &a, const Out &b, bool v0_, bool v1_)
    {
        store2<XT>(x64n, i, a.x, b.x, v0_, v1_);
        store2<float>(r, i, a.r, b.r, v0_, v1_);
        if (restart) {
            store2<float>(p, i, 0.f, 0.f, v0_, v1_);
            if constexpr (BICG) {
                store2<float>(r0, i, a.r, b.r, v0_, v1_);
                store2<float>(v, i, 0.f, 0.f, v0_, v1_);
            }
        }
    }
    __device__ void partials(double (&t)[NV]) const
    {
        t[0] = (double)a_rr.hi(); t[1] = (double)a_bb.hi(); t[2] = (double)a_d.hi();
    }
    __device__ static void finish(Scalars &sc, const double (&t)[NV])
    {
        const int mode = sc.replace;
        sc.replace = 0;
        sc.b64_sq = t[1];
        if (t[1] == 0.0) { sc.state = ZERO_RHS; return; }
        sc.x64_cur ^= 1;
        sc.e_reset = 1;
        sc.outer_steps += 1;
        sc.r64_sq = t[0];
        const double tol2 = sc.tol_outer * sc.tol_outer * t[1];
        sc.tol2 = tol2;
        sc.rhs_sq = t[1];
        if (t[0] <= tol2) { sc.state = CONVERGED; return; }
        if (!(t[0] <= sc.div_thresh)) { sc.state = DIVERGED; return; }  // also NaN
        if (sc.iter >= sc.max_iter) { sc.state = MAXITER; return; }
        sc.rsq = t[0];
        sc.rsq_max = t[0];
        if (sc.cg_fused) {
            // the one-sweep CG restarts from the replaced residual
            sc.k1_mode = 1;
            return;
        }
        if (mode == 2) {
            // Fresh Krylov space from the true residual: p (and v) are zero,
            // so the next step-1 kernel forms p = r (CG: p = z).
            sc.beta = 0.0;
            if (BICG) {
                sc.r0_sq = t[0];
                sc.rho = t[2];
                sc.rho_old = 1.0;
                sc.alpha = 1.0;
                sc.omega = 1.0;
            } else {
                sc.zr = t[2];
            }
        } else if (BICG) {
            // rho_old, alpha and omega are those of the iteration just done.
            sc.rho = t[2];
            sc.beta = (t[2] / sc.rho_old) * (sc.alpha / sc.omega);
        } else {
            // rho_old holds r.z of the previous iteration (set by CG step 2).
            sc.beta = t[2] / sc.rho_old;
            sc.zr = t[2];
        }
    }
};

// ===========================================================================
// MIXED two-sweep BiCGSTAB: the FP64 residual replacement at the head of an
// iteration.  The updates of the last iteration are still pending (step 1
// applies them), so the iterate is formed on the fly,
//   e_k = e + a y + w z, y = p/diag, z = (r - a v)/diag   (FP32, as step 1),
//   x = x64 + e_k                                          (FP64),
// at every tile and halo point; then r64 = b - A x in FP64.  x64' = x is
// stored, fp32(r64) goes to t, from which step 1 takes r_k (k1_mode = 1, e =
// 0); on a restart it also becomes the shadow residual r0 and beta = 0 makes
// p_k = r_k.  Dots (FP32-accumulated): |fp32(r64)|^2, |b|^2, r0.fp32(r64).
// x64 and b - A x are FP64 by default, float-float on request (XArith).
// Streams: x64, e, p, r, v, r0, code.
// ===========================================================================
template <typename XT>
struct OpReplaceBi2 {
    using T = XT;
    using X = XArith<XT>;
    using R = double;
    using SL = Streams<8, 4, 4, 4, 4, 4, 1>;
    static constexpr int NV = 3;
    using Shared = Coef<float>;
    struct Vals { XT x; float e, p, r, v, r0; uint32_t code; };
    struct Own { uint32_t code; float r0; };
    struct Out { XT x; float r; };
    const CUtensorMap *tmap[SL::N];
    Faces<T> F;
    XT *x64n;
    float *t, *r0;
    float alpha, omega;
    bool restart;
    Acc<float> a_rr, a_bb, a_d;

    __device__ static bool active(const Scalars &sc) { return sc.state == RUNNING && sc.replace != 0; }
    __device__ static void load_shared(Shared &S, const Job &J, int tid) { load_coef<float>(S, J, tid); }
    __device__ static void load2(const unsigned char *st, const Pt &p_, Vals &a, Vals &b)
    {
        sv2<XT, SL, 0>(st, p_, a.x, b.x);
        sv2<float, SL, 1>(st, p_, a.e, b.e);
        sv2<float, SL, 2>(st, p_, a.p, b.p);
        sv2<float, SL, 3>(st, p_, a.r, b.r);
        sv2<float, SL, 4>(st, p_, a.v, b.v);
        sv2<float, SL, 5>(st, p_, a.r0, b.r0);
        load_code2<SL, 6>(st, p_, a.code, b.code);
    }
    __device__ static void load1(const unsigned char *st, const Pt &p_, Vals &a)
    {
        a.x = sv<XT, SL, 0>(st, p_);
        a.e = sv<float, SL, 1>(st, p_);
        a.p = sv<float, SL, 2>(st, p_);
        a.r = sv<float, SL, 3>(st, p_);
        a.v = sv<float, SL, 4>(st, p_);
        a.code = sv<uint8_t, SL, 6>(st, p_);
    }
    __device__ void init(const Job &J, Shared &)
    {
        F = faces_of<T>(J);
        const Scalars &sc = *J.sc;
        const int cur = sc.x64_cur;
        const int par = (int)(sc.iter & 1);
        tmap[0] = &J.tm[TM_X64 + cur];
        tmap[1] = &J.tm[TM_X];
        tmap[2] = &J.tm[TM_P + par];
        tmap[3] = &J.tm[TM_R + par];
        tmap[4] = &J.tm[TM_V + par];
        tmap[5] = &J.tm[TM_R0];
        tmap[6] = &J.tm[TM_CODE];
        x64n = (XT *)J.x64[cur ^ 1];
        t = (float *)J.t;
        r0 = (float *)J.r0;
        alpha = (float)sc.alpha;
        omega = (float)sc.omega;
        restart = sc.replace == 2;
    }
    __device__ XT iterate(const Geo &g, Shared &S, const Vals &a, const Pos &ps) const
    {
        const float inv = inv_of<float, true>(S, g, a.code, ps);
        const float ek = a.e + alpha * (a.p * inv) + omega * ((a.r - alpha * a.v) * inv);
        return X::add_f(a.x, ek);
    }
    __device__ XT field(const Geo &g, const typename X::Tab &, Shared &S, const Vals &a, const Pos &ps) const
    {
        return iterate(g, S, a, ps);
    }
    __device__ Own own(const Geo &g, const typename X::Tab &, Shared &S, const Vals &a, const Pos &ps, XT &f) const
    {
        f = iterate(g, S, a, ps);
        return Own{a.code, a.r0};
    }
    __device__ Out apply(const Geo &g, const typename X::Tab &C, Shared &, const Own &o, const Pos &ps, XT fc,
                         XT fxp, XT fxm, XT fyp, XT fym, XT fzp, XT fzm)
    {
        const XT ax = X::stencil(F, C, g, o.code, ps, fc, fxp, fxm, fyp, fym, fzp, fzm);
        float r32, b32;
        X::residual(C, g, o.code, ps, ax, r32, b32);
        a_rr.add_prod(r32, r32);
        a_bb.add_prod(b32, b32);
        a_d.add_prod(restart ? r32 : o.r0, r32);
        return Out{fc, r32};
    }
    __device__ void store(int64_t i, const Out &a, const Out &b, bool v0_, bool v1_)
    {
        store2<XT>(x64n, i, a.x, b.x, v0_, v1_);
        store2<float>(t, i, a.r, b.r, v0_, v1_);
        if (restart) store2<float>(r0, i, a.r, b.r, v0_, v1_);
    }
    __device__ void partials(double (&v)[NV]) const
    {
        v[0] = (double)a_rr.hi(); v[1] = (double)a_bb.hi(); v[2] = (double)a_d.hi();
    }
    __device__ static void finish(Scalars &sc, const double (&t)[NV])
    {
        const int mode = sc.replace;
        sc.replace = 0;
        sc.b64_sq = t[1];
        if (t[1] == 0.0) { sc.state = ZERO_RHS; return; }
        sc.x64_cur ^= 1;
        sc.k1_mode = 1;
        sc.outer_steps += 1;
        sc.r64_sq = t[0];
        const double tol2 = sc.tol_outer * sc.tol_outer * t[1];
        sc.tol2 = tol2;
        sc.rhs_sq = t[1];
        if (t[0] <= tol2) { sc.state = CONVERGED; return; }
        if (!(t[0] <= sc.div_thresh)) { sc.state = DIVERGED; return; }  // also NaN
        if (sc.iter >= sc.max_iter) { sc.state = MAXITER; return; }
        sc.rsq = t[0];
        sc.rsq_max = t[0];
        if (mode == 2) {  // new shadow residual r0 = r: rho = |r|^2, p_k = r_k
            sc.r0_sq = t[0];
            sc.rho = t[0];
            sc.beta = 0.0;
        } else {          // rho_old, alpha, omega are those of the last iteration
            sc.rho = t[2];
            sc.beta = (t[2] / sc.rho_old) * (sc.alpha / sc.omega);
        }
    }
};

// ===========================================================================
// Pointwise kernels on the same tiling (two x columns per thread): stencil
// codes + pore count, the MIXED x64 = x0 initialisation, and the tau flux.
// ===========================================================================
struct TileCoords {
    int x0, y0, z0, z1, gx, gy;
    bool v[2];
    int64_t local;
};

__device__ __forceinline__ TileCoords tile_coords(const Job &J, int tid)
{
    TileCoords t;
    t.local = (int64_t)blockIdx.x - J.tile_base;
    const int tx_t = (int)(t.local % J.tiles_x);
    const int ty_t = (int)((t.local / J.tiles_x) % J.tiles_y);
    const int tz_t = (int)(t.local / ((int64_t)J.tiles_x * J.tiles_y));
    t.x0 = tx_t * TX;
    t.y0 = ty_t * TY;
    t.z0 = tz_t * J.zc;
    t.z1 = min(t.z0 + J.zc, J.nz);
    t.gx = t.x0 + 2 * (tid % TPR);
    t.gy = t.y0 + tid / TPR;
    t.v[0] = t.gx < J.nx && t.gy < J.ny;
    t.v[1] = t.gx + 1 < J.nx && t.gy < J.ny;
    return t;
}

// Stencil code of every voxel (bit d: neighbour d solid, clamped at the domain
// faces; bit 6: self solid; bit 7: on a domain face) and the number of pore
// (zero) voxels, as Volume::sumZeroElems counts them
// (fastlib/src/volume/Volume.cpp:261-272).
__global__ void __launch_bounds__(NTHREADS) code_kernel(Launch L)
{
    __shared__ int s_job, s_flag;
    __shared__ double s_red[2 * (NTHREADS / 32)];
    const int tid = threadIdx.x;
    if (tid == 0) s_job = find_job(L, (int64_t)blockIdx.x);
    __syncthreads();
    const Job &J = L.jobs[s_job];
    const TileCoords t = tile_coords(J, tid);
    const int nx = J.nx, ny = J.ny, nz = J.nz;
    uint8_t *code = const_cast<uint8_t *>(J.code);
    const uint8_t *m = J.mask;  // unpadded
    const int64_t sy = nx, sz = (int64_t)nx * ny;
    uint32_t pores = 0;
    for (int k = 0; k < 2; k++) {
        if (!t.v[k]) continue;
        const int x = t.gx + k, y = t.gy;
        for (int z = t.z0; z < t.z1; ++z) {
            const int64_t i = (int64_t)x + sy * y + sz * z;
            const int64_t ic = (int64_t)x + (int64_t)J.pitch * ((int64_t)y + (int64_t)ny * z);
            if (!ft_in(J, i, i, sz * nz, OOB_CODE) || !ft_in(J, ic, ic, (int64_t)J.pitch * ny * nz, OOB_CODE)) continue;
            const uint32_t self = __ldg(m + i) != 0;
            pores += self ? 0u : 1u;
            uint32_t c = self << SELF_BIT;
            c |= (x + 1 < nx ? (__ldg(m + i + 1) != 0) : self) << 0;
            c |= (x > 0 ? (__ldg(m + i - 1) != 0) : self) << 1;
            c |= (y + 1 < ny ? (__ldg(m + i + sy) != 0) : self) << 2;
            c |= (y > 0 ? (__ldg(m + i - sy) != 0) : self) << 3;
            c |= (z + 1 < nz ? (__ldg(m + i + sz) != 0) : self) << 4;
            c |= (z > 0 ? (__ldg(m + i - sz) != 0) : self) << 5;
            const bool bnd = x == 0 || y == 0 || z == 0 || x == nx - 1 || y == ny - 1 || z == nz - 1;
            c |= (bnd ? 1u : 0u) << BND_BIT;
            code[ic] = (uint8_t)c;
        }
    }
    double v[1] = {(double)pores};
    block_sum_store<1>(v, J.part + t.local * NPART, s_red);
    if (arrive_last(J.counter, J.ntiles, &s_flag)) {
        double tot[1];
        sum_partials<1>(J.part, J.ntiles, tot, s_red);
        if (tid == 0) {
            J.sc->pores = (uint64_t)tot[0];
            *J.counter = 0u;
        }
    }
}

// MIXED: x64[0] = x0 (the reference's initial guess; its precision does not
// matter to the converged iterate, so it is formed in FP32), e = 0 (and the
// two-sweep BiCGSTAB vectors r, p, v, t = 0).
__global__ void __launch_bounds__(NTHREADS) init64_kernel(Launch L)
{
    __shared__ int s_job;
    const int tid = threadIdx.x;
    if (tid == 0) s_job = find_job(L, (int64_t)blockIdx.x);
    __syncthreads();
    const Job &J = L.jobs[s_job];
    const TileCoords t = tile_coords(J, tid);
    const Geo g{J.nx, J.ny, J.nz, J.dir >> 1, (J.dir & 1) ? -1 : 1, J.pitch};
    void *x64 = J.x64[0];
    const bool ff = J.x64_ff != 0;
    float *e = (float *)J.x;
    // Two-sweep BiCGSTAB: the first replacement reads r, p, v (scaled by
    // alpha = omega = 0) and step 1 reads t; all start at zero.
    float *zr = (float *)J.r[0], *zp = (float *)J.p[0], *zv = (float *)J.v[0], *zt = (float *)J.t;
    for (int k = 0; k < 2; k++) {
        if (!t.v[k]) continue;
        for (int z = t.z0; z < t.z1; ++z) {
            const int64_t i = g.idx(t.gx + k, t.gy, z);
            if (!ft_in(J, i, i, (int64_t)J.pitch * J.ny * J.nz, OOB_INIT)) continue;
            const float x0 = x0_at<float>(g, t.gx + k, t.gy, z);
            if (ff) ((FF *)x64)[i] = FF(x0, 0.f);
            else ((double *)x64)[i] = (double)x0;
            e[i] = 0.f;
            if (zt) {
                zr[i] = 0.f;
                zp[i] = 0.f;
                zv[i] = 0.f;
                zt[i] = 0.f;
            }
        }
    }
}

// tau flux (fastlib/src/volume/VolumeMeasures.cpp:208-257): for every voxel
// D_cell * (c - c_next) / dx with c_next the neighbour one step along the
// direction, or 0 with dx = 0.5 past the last plane.  D_cell is the float
// coefficient of the voxel's phase.  Summed in FP64.
template <typename TC>
__device__ __forceinline__ double conc_at(const TC *c, int64_t i)
{
    if constexpr (std::is_same<TC, FF>::value) {
        const float2 v = __ldg(reinterpret_cast<const float2 *>(c) + i);
        return (double)v.x + (double)v.y;
    } else {
        return (double)__ldg(c + i);
    }
}

// The MIXED iterate as FP64 values (for the concentration output).
__global__ void ff_to_double_kernel(const float2 *src, double *dst, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 v = src[i];
        dst[i] = (double)v.x + (double)v.y;
    }
}

template <typename TC>
__global__ void __launch_bounds__(NTHREADS) tau_kernel(Launch L, int use_x64)
{
    __shared__ int s_job, s_flag;
    __shared__ double s_red[2 * (NTHREADS / 32)];
    const int tid = threadIdx.x;
    if (tid == 0) s_job = find_job(L, (int64_t)blockIdx.x);
    __syncthreads();
    const Job &J = L.jobs[s_job];
    const TileCoords t = tile_coords(J, tid);
    const Geo g{J.nx, J.ny, J.nz, J.dir >> 1, (J.dir & 1) ? -1 : 1, J.pitch};
    const TC *c = use_x64 ? (const TC *)J.x64[J.sc->x64_cur] : (const TC *)J.x;
    const double cc[2] = {(double)J.c_tau[0], (double)J.c_tau[1]};
    const int64_t step = g.k == 0 ? 1 : (g.k == 1 ? (int64_t)g.P : (int64_t)g.P * g.ny);
    const int64_t sstep = g.sgn > 0 ? step : -step;
    const int ext = g.extent();
    Acc<double> acc;
    for (int k = 0; k < 2; k++) {
        if (!t.v[k]) continue;
        const int x = t.gx + k;
        for (int z = t.z0; z < t.z1; ++z) {
            const int64_t i = g.idx(x, t.gy, z);
            const int kn = g.coord(x, t.gy, z) + g.sgn;
            const int64_t np = (int64_t)g.P * g.ny * g.nz;
            if (!ft_in(J, i, i, np, OOB_TAU)) continue;
            const double here = conc_at(c, i);
            double prev = 0.0, rdx = 2.0;  // 1/dx: dx = 0.5 past the last plane
            if (kn >= 0 && kn < ext && ft_in(J, i + sstep, i + sstep, np, OOB_TAU)) {
                prev = conc_at(c, i + sstep);
                rdx = 1.0;
            }
            const int self = (__ldg(J.code + i) >> SELF_BIT) & 1;
            acc.add(cc[self] * (here - prev) * rdx);  // == / dx exactly (dx is 1 or 1/2)
        }
    }
    double v[1] = {acc.hi()};
    block_sum_store<1>(v, J.part + t.local * NPART, s_red);
    if (arrive_last(J.counter, J.ntiles, &s_flag)) {
        double tot[1];
        sum_partials<1>(J.part, J.ntiles, tot, s_red);
        if (tid == 0) {
            J.sc->flux_sum = tot[0];
            *J.counter = 0u;
        }
    }
}

}  // namespace ft
