// FP64 iterative refinement step, tau flux reduction, stencil-code build and
// porosity count.
#pragma once
#include "tau_sweep.cuh"

namespace ft {

// ===========================================================================
// MIXED refinement step (FP64): x64' = x64 + e (e = the FP32 correction of
// the previous inner solve), r64 = b - A x64' in FP64, and the next inner
// system A e = fp32(r64) set up with e = 0 and zeroed Krylov vectors.
// Dots (FP64): |r64|^2, |b|^2, |fp32(r64)|^2, fp32(r64).z.
// Streams: x64, e, code.
// ===========================================================================
template <bool BICG>
struct OpRefine {
    using T = double;
    using SL = Streams<8, 4, 1>;
    static constexpr int NV = 4;
    using Shared = Coef<float>;
    struct Vals { double x; float e; uint32_t code; };
    struct Own { uint32_t code; };
    struct Out { double x; float r; };
    const CUtensorMap *tmap[SL::N];
    double *x64n;
    float *r, *r0, *p0, *v0;
    Acc<double> a_r64, a_bb, a_r32, a_rz;

    __device__ static bool active(const Scalars &sc) { return sc.outer_state == RUNNING; }
    __device__ static void load_shared(Shared &S, const Job &J, int tid) { load_coef<float>(S, J, tid); }
    __device__ static void load2(const unsigned char *st, const Pt &p, Vals &a, Vals &b)
    {
        sv2<double, SL, 0>(st, p, a.x, b.x);
        sv2<float, SL, 1>(st, p, a.e, b.e);
        load_code2<SL, 2>(st, p, a.code, b.code);
    }
    __device__ static void load1(const unsigned char *st, const Pt &p, Vals &a)
    {
        a.x = sv<double, SL, 0>(st, p);
        a.e = sv<float, SL, 1>(st, p);
    }
    __device__ void init(const Job &J, Shared &)
    {
        const int cur = J.sc->x64_cur;
        tmap[0] = &J.tm[TM_X64 + cur];
        tmap[1] = &J.tm[TM_X];
        tmap[2] = &J.tm[TM_CODE];
        x64n = J.x64[cur ^ 1];
        r = (float *)J.r[0];
        r0 = (float *)J.r0;
        p0 = (float *)J.p[0];
        v0 = (float *)J.v[0];
    }
    __device__ double field(const Geo &, const Coef<double> &, Shared &, const Vals &v, int, int, int) const
    {
        return v.x + (double)v.e;
    }
    __device__ Own own(const Geo &, const Coef<double> &, Shared &, const Vals &v, int, int, int, double &f) const
    {
        f = v.x + (double)v.e;
        return Own{v.code};
    }
    __device__ Out apply(const Geo &g, const Coef<double> &C, Shared &S, const Own &o, int x_, int y_, int z_,
                         double fc, double fxp, double fxm, double fyp, double fym, double fzp, double fzm)
    {
        const double d = diag_of<double>(C, g, o.code, x_, y_, z_);
        const double ax = stencil7<double>(C, o.code, fc, fxp, fxm, fyp, fym, fzp, fzm, d);
        const double b = rhs_at<double>(C, g, o.code, x_, y_, z_);
        const double res = b - ax;
        const float r32 = (float)res;
        const float inv = inv_of<float>(S, g, o.code, x_, y_, z_);
        a_r64.add_prod(res, res);
        a_bb.add_prod(b, b);
        a_r32.add_prod((double)r32, (double)r32);
        a_rz.add_prod((double)r32, (double)(r32 * inv));
        return Out{fc, r32};
    }
    __device__ void store(int64_t i, const Out &a, const Out &b, bool v0_, bool v1_)
    {
        store2<double>(x64n, i, a.x, b.x, v0_, v1_);
        store2<float>(r, i, a.r, b.r, v0_, v1_);
        store2<float>(p0, i, 0.f, 0.f, v0_, v1_);
        if (BICG) {
            store2<float>(r0, i, a.r, b.r, v0_, v1_);
            store2<float>(v0, i, 0.f, 0.f, v0_, v1_);
        }
    }
    __device__ void partials(double (&v)[NV]) const
    {
        v[0] = a_r64.hi(); v[1] = a_bb.hi(); v[2] = a_r32.hi(); v[3] = a_rz.hi();
    }
    __device__ static void finish(Scalars &sc, const double (&t)[NV])
    {
        sc.total_iter += sc.iter;
        sc.iter = 0;
        sc.state = CONVERGED;  // no inner solve unless set up below
        sc.b64_sq = t[1];
        if (t[1] == 0.0) { sc.outer_state = ZERO_RHS; return; }
        // Keep a correction only if it lowered the true FP64 residual.  A
        // rejected one leaves x64 as it was; the host zeroes e and this step
        // runs again, which re-evaluates x64 and sets up the same inner solve
        // bit for bit (every reduction has a fixed order).  That replay stops
        // at the iteration where the rejected solve had its smallest
        // residual, so it returns the best correction the solve passed by.
        if (sc.outer_steps > 0 && !sc.reject_pending && !(t[0] < sc.r64_sq)) {
            sc.rejects += 1;
            const uint64_t best = sc.iter_min;
            if (best == 0 || sc.replay_iters != 0 || sc.rejects > 8 || sc.total_iter >= sc.max_total) {
                sc.outer_state = MAXITER;
                return;
            }
            sc.replay_iters = best;
            sc.reject_pending = 1;
            return;
        }
        const uint64_t replay = sc.reject_pending ? sc.replay_iters : 0;
        if (!sc.reject_pending) sc.replay_iters = 0;
        sc.reject_pending = 0;
        sc.x64_cur ^= 1;
        sc.r64_sq = t[0];
        sc.rsq = t[0];
        if (t[0] <= sc.tol_outer * sc.tol_outer * t[1]) { sc.outer_state = CONVERGED; return; }
        if (t[0] > sc.div_thresh) { sc.outer_state = DIVERGED; return; }
        if (sc.total_iter >= sc.max_total) { sc.outer_state = MAXITER; return; }
        // Ask the FP32 inner solve for the residual reduction still needed
        // (with a factor 2 margin), but no less than it can deliver.
        const double rel = sqrt(t[0] / t[1]);
        double tin = 0.5 * sc.tol_outer / rel;
        if (tin < sc.inner_floor) tin = sc.inner_floor;
        if (tin > 0.5) tin = 0.5;
        sc.tol = tin;
        sc.rhs_sq = t[2];
        sc.tol2 = tin * tin * t[2];
        sc.rsq = t[2];
        sc.zr = t[3];
        sc.beta = 0.0;
        sc.alpha = 1.0;
        sc.omega = 1.0;
        sc.rho = t[2];
        sc.rho_old = 1.0;
        sc.r0_sq = t[2];
        if (BICG) sc.beta = t[2];  // (rho/1)*(1/1)
        sc.restarts = 0;
        sc.restart = 0;
        sc.max_iter = sc.max_total - sc.total_iter;
        if (replay != 0 && replay < sc.max_iter) sc.max_iter = replay;
        sc.rsq_min = t[2];
        sc.iter_min = 0;
        sc.outer_steps += 1;
        sc.state = (t[2] > sc.tol2) ? RUNNING : CONVERGED;
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

// MIXED: x64[0] = x0 (the reference's initial guess, in FP64), e = 0.
__global__ void __launch_bounds__(NTHREADS) init64_kernel(Launch L)
{
    __shared__ int s_job;
    const int tid = threadIdx.x;
    if (tid == 0) s_job = find_job(L, (int64_t)blockIdx.x);
    __syncthreads();
    const Job &J = L.jobs[s_job];
    const TileCoords t = tile_coords(J, tid);
    const Geo g{J.nx, J.ny, J.nz, J.dir >> 1, (J.dir & 1) ? -1 : 1, J.pitch};
    double *x64 = J.x64[0];
    float *e = (float *)J.x;
    for (int k = 0; k < 2; k++) {
        if (!t.v[k]) continue;
        for (int z = t.z0; z < t.z1; ++z) {
            const int64_t i = g.idx(t.gx + k, t.gy, z);
            x64[i] = x0_at<double>(g, t.gx + k, t.gy, z);
            e[i] = 0.f;
        }
    }
}

// tau flux (fastlib/src/volume/VolumeMeasures.cpp:208-257): for every voxel
// D_cell * (c - c_next) / dx with c_next the neighbour one step along the
// direction, or 0 with dx = 0.5 past the last plane.  D_cell is the float
// coefficient of the voxel's phase.  Summed in FP64.
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
            const double here = (double)__ldg(c + i);
            double prev = 0.0, dx = 0.5;
            if (kn >= 0 && kn < ext) {
                prev = (double)__ldg(c + i + sstep);
                dx = 1.0;
            }
            const int self = (__ldg(J.code + i) >> SELF_BIT) & 1;
            acc.add(cc[self] * (here - prev) / dx);
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
