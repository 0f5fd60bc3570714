// The z-marching stencil sweep shared by every solver kernel, and the
// operations (Op) that plug into it.
//
// One thread block owns a TX x TY column tile of one right-hand side and
// marches the planes z0..z1-1 of its slab; each thread owns two neighbouring
// x columns of one row (or of two rows, for the operations that name
// RPT = 2).  The state vectors an operation reads arrive through TMA: for
// every plane, one thread issues one cp.async.bulk.tensor tile load per vector
// (the tile plus a one-voxel x/y halo, widened in x to the 16-byte TMA
// alignment) into a ring of NSTAGE shared-memory stages, each completed on
// its own mbarrier, so NSTAGE-1 planes of every vector are in flight while
// the block computes.  From a stage the block forms the operand field of the
// plane (p = z + beta p, y = p/diag, ...) for its tile and halo into a shared
// plane buffer (paired vector stores); the z neighbours of a thread's own
// columns stay in registers.  The operator is applied one plane behind the
// loads.  Points outside the domain hold exactly 0 in the plane buffers and
// registers, so the stencil needs no bounds tests.  Dot products accumulate
// per thread, reduce per block into a partial slot, and the last block of
// each right-hand side to arrive sums the partials in a fixed order and
// advances that right-hand side's scalars.
//
// Every mbarrier wait is bounded (%globaltimer, 2 s).  A block whose tile
// loads do not arrive drains its own copies in flight (again bounded), marks
// its job FAULT and returns; the host reports FAST_TIMEOUT.
#pragma once
#include "tau_device.cuh"

namespace ft {

// ---------------------------------------------------------------------------
// TMA / mbarrier primitives (inline PTX).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// HINT > 0: the wait may suspend the thread for up to HINT ns while the
// phase is incomplete (a suspended thread issues nothing) instead of
// returning at once to the polling loop.  Which is better depends on the
// kernel (an operation names its hint as wait_hint_ns; default 0).
template <uint32_t HINT = 0>
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    if constexpr (HINT > 0) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(bar), "r"(parity), "r"(HINT)
            : "memory");
    } else {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
    }
    return ok != 0;
}

__device__ __forceinline__ uint64_t global_timer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Limit of every bounded wait; test builds shorten it.
#ifndef FAST_TAU_WAIT_LIMIT_NS
#define FAST_TAU_WAIT_LIMIT_NS 2000000000ull  // 2 s
#endif
constexpr uint64_t kWaitLimitNs = FAST_TAU_WAIT_LIMIT_NS;

// FAST_TAU_TEST_HOOKS=1 builds (tests only) honour Scalars::test_withhold: the
// first sweep of an armed right-hand side does not issue the tile loads of
// plane 1 in its first tile, so that block's bounded wait runs out and the
// solve fails with FAST_TIMEOUT.  Compiled out by default.
#ifndef FAST_TAU_TEST_HOOKS
#define FAST_TAU_TEST_HOOKS 0
#endif

// Waits for phase `parity` of the mbarrier, giving up after kWaitLimitNs.
template <uint32_t HINT = 0>
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity)
{
    if (mbar_try_wait<HINT>(bar, parity)) return true;
    const uint64_t t0 = global_timer_ns();
    while (!mbar_try_wait<HINT>(bar, parity)) {
        if (global_timer_ns() - t0 > kWaitLimitNs) return false;
    }
    return true;
}

#ifndef FAST_TAU_HINT_CG
#define FAST_TAU_HINT_CG 0
#endif

// An operation's wait hint: Op::wait_hint_ns when it names one, else 0.
template <class Op, class = void>
struct WaitHint {
    static constexpr uint32_t ns = 0;
};
template <class Op>
struct WaitHint<Op, std::void_t<decltype(Op::wait_hint_ns)>> {
    static constexpr uint32_t ns = Op::wait_hint_ns;
};

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *tm, int x, int y, int z, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(dst), "l"(tm), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void prefetch_tmap(const CUtensorMap *tm)
{
    asm volatile("prefetch.tensormap [%0];" ::"l"(tm) : "memory");
}

// ---------------------------------------------------------------------------
// Shared-memory stage layout.  A stream of element size ES is loaded as a box
// of box_w(ES) x HY elements starting at (x0 - 16/ES, y0 - 1): the box start
// and width in x are multiples of 16 bytes, and the element of x = x0 + 2k
// sits at an even offset, so a thread's two columns load as one vector.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int box_off(int es) { return 16 / es; }
__host__ __device__ constexpr int box_w(int es) { return TX + 2 * box_off(es); }
__host__ __device__ constexpr int box_bytes(int es) { return box_w(es) * HY * es; }
__host__ __device__ constexpr int box_alloc(int es) { return (box_bytes(es) + 127) / 128 * 128; }

// A stream is named by its element size; a negative size marks a stream the
// operation reads only at its own points (never at the halo): it is loaded
// as the TX x TY tile alone (its tensor map has that box), which saves the
// halo's shared memory and L2 reads.
template <int... ES>
struct Streams {
    static constexpr int N = sizeof...(ES);
    __host__ __device__ static constexpr int raw(int s)
    {
        constexpr int a[N] = {ES...};
        return a[s];
    }
    __host__ __device__ static constexpr int esz(int s) { return raw(s) < 0 ? -raw(s) : raw(s); }
    __host__ __device__ static constexpr bool interior(int s) { return raw(s) < 0; }
    __host__ __device__ static constexpr int bytes(int s) { return interior(s) ? TX * TY * esz(s) : box_bytes(esz(s)); }
    __host__ __device__ static constexpr int off(int s)
    {
        int o = 0;
        for (int t = 0; t < s; ++t) o += (bytes(t) + 127) / 128 * 128;
        return o;
    }
    __host__ __device__ static constexpr int stage_bytes() { return off(N); }
    __host__ __device__ static constexpr int tx_bytes()
    {
        int b = 0;
        for (int t = 0; t < N; ++t) b += bytes(t);
        return b;
    }
};

// A point of the stage tile: tile row (0..HY-1) and x offset xr = x - x0
// (-1..TX).
struct Pt {
    int row, xr;
};

template <typename E, class SL, int S>
__device__ __forceinline__ const E *sp(const unsigned char *stage, const Pt &p)
{
    constexpr int es = (int)sizeof(E);
    static_assert(SL::esz(S) == es, "stream element size");
    if constexpr (SL::interior(S))  // own points only: tile rows 1..TY, x 0..TX-1
        return reinterpret_cast<const E *>(stage + SL::off(S)) + (p.row - 1) * TX + p.xr;
    else
        return reinterpret_cast<const E *>(stage + SL::off(S)) + p.row * box_w(es) + p.xr + box_off(es);
}

// Element of stream S at point p.
template <typename E, class SL, int S>
__device__ __forceinline__ E sv(const unsigned char *stage, const Pt &p)
{
    return *sp<E, SL, S>(stage, p);
}

// The two elements of stream S at p and p + 1 (p.xr even), as one load.
template <typename E, class SL, int S>
__device__ __forceinline__ void sv2(const unsigned char *stage, const Pt &p, E &a, E &b)
{
    const E *q = sp<E, SL, S>(stage, p);
    if constexpr (std::is_same<E, FF>::value) {
        const float4 v = *reinterpret_cast<const float4 *>(q);
        a = FF(v.x, v.y);
        b = FF(v.z, v.w);
    } else if constexpr (sizeof(E) == 4) {
        const float2 v = *reinterpret_cast<const float2 *>(q);
        a = v.x;
        b = v.y;
    } else if constexpr (sizeof(E) == 8) {
        const double2 v = *reinterpret_cast<const double2 *>(q);
        a = v.x;
        b = v.y;
    } else {
        const unsigned short v = *reinterpret_cast<const unsigned short *>(q);
        a = (E)(v & 0xff);
        b = (E)(v >> 8);
    }
}

template <typename T>
struct alignas(2 * sizeof(T)) Pair {
    T a, b;
};

// Stores a lane pair to p[i], p[i+1] (i even): one vector store when both
// lanes are inside the domain.
template <typename T>
__device__ __forceinline__ void store2(T *p, int64_t i, T a, T b, bool v0, bool v1)
{
    if (v0 && v1) {
        *reinterpret_cast<Pair<T> *>(p + i) = Pair<T>{a, b};
    } else {
        if (v0) p[i] = a;
        if (v1) p[i + 1] = b;
    }
}

// Dynamic shared memory of a sweep: the stage ring plus 128 bytes to align
// its base to 128 bytes.
template <class Op, int NSTAGE>
__host__ __device__ constexpr int sweep_dyn_smem()
{
    return NSTAGE * Op::SL::stage_bytes() + 128;
}

// Plane buffer: row stride PW elements; x = x0 + k sits at column k + 2, so
// thread pairs start at even columns; column 1 holds x0 - 1, column TX + 2
// holds x0 + TX.
constexpr int PW = TX + 4;

// Type of an operation's per-thread partial sums: Op::R when it names one,
// else its field type.
template <class Op, class = void>
struct RedType {
    using type = typename Op::T;
};
template <class Op>
struct RedType<Op, std::void_t<typename Op::R>> {
    using type = typename Op::R;
};

// FAST_TAU_INTERIOR=0 loads every stream with its halo (the interior-only
// boxes off).
#ifndef FAST_TAU_INTERIOR
#define FAST_TAU_INTERIOR 1
#endif
__host__ __device__ constexpr int own_only(int es) { return FAST_TAU_INTERIOR ? -es : es; }

// A lane pair of halo points: Op::load2h when the operation has streams it
// reads only at its own points (they are not in the stage at the halo),
// else Op::load2.
template <class Op, class = void>
struct HaloLoad {
    template <class V>
    __device__ static void pair(const unsigned char *st, const Pt &p, V &a, V &b) { Op::load2(st, p, a, b); }
};
template <class Op>
struct HaloLoad<Op, std::void_t<decltype(&Op::load2h)>> {
    template <class V>
    __device__ static void pair(const unsigned char *st, const Pt &p, V &a, V &b) { Op::load2h(st, p, a, b); }
};

// Operations that run first after the MIXED replacement slot clear the
// launch's gate word (Op::clears_gate).
template <class Op, class = void>
struct GateRole {
    static constexpr bool clears = false;
};
template <class Op>
struct GateRole<Op, std::void_t<decltype(Op::clears_gate)>> {
    static constexpr bool clears = Op::clears_gate;
};

// The sweep of one tile `blk` (a block index of the launch), shared by the
// kernel entries below.  `qb` counts the planes this block has taken through
// its stage ring so far (ring slot and mbarrier phase continue from it), and
// `ready` tells whether the block's mbarriers are initialised; both carry
// over when one block sweeps several tiles.  Returns SWEEP_DONE, SWEEP_IDLE
// (the tile's right-hand side is not active; *idle_end = its last tile + 1)
// or SWEEP_FAULT.
enum { SWEEP_DONE = 0, SWEEP_IDLE = 1, SWEEP_FAULT = 2 };

// Rows per thread: an operation that names RPT = 2 sweeps its TX x TY tile
// with half the threads, each owning two neighbouring rows of its two
// columns (four points per plane).  The per-plane work that does not depend
// on the point (ring slot and phase, the wait, plane indices, the barrier,
// store addresses) is then spread over twice the points, and the y
// neighbour inside a thread's row pair comes from its registers.  For the
// sweeps whose few bytes per point leave them bound by instruction issue.
template <class Op, class = void>
struct RowsPerThread {
    static constexpr int n = 1;
};
template <class Op>
struct RowsPerThread<Op, std::void_t<decltype(Op::RPT)>> {
    static constexpr int n = Op::RPT;
};

// Threads of an operation's sweep blocks.
template <class Op>
__host__ __device__ constexpr int sweep_threads()
{
    return NTHREADS / RowsPerThread<Op>::n;
}

#ifndef FAST_TAU_FULL_TILE
#define FAST_TAU_FULL_TILE 1
#endif

template <class Op, int NSTAGE>
__device__ __forceinline__ int sweep_body(const Launch &L, int64_t blk, int &qb, bool &ready, int64_t *idle_end)
{
    using T = typename Op::T;
    using SL = typename Op::SL;
    using V = typename Op::Vals;
    constexpr int NV = Op::NV;
    constexpr int SB = SL::stage_bytes();
    constexpr int RPT = RowsPerThread<Op>::n;
    constexpr int NT = sweep_threads<Op>();
    static_assert((RPT == 1 || RPT == 2) && TY % RPT == 0, "one or two rows per thread");
    static_assert(NT >= 2 * TPR + 2 * TY && NT % 32 == 0, "halo roles need 2 TPR + 2 TY threads");
    // The stage refill: the first thread of the last warp (the first warps
    // also form the halo rows).
    constexpr int kRefillThread = NT - 32;
    extern __shared__ __align__(128) unsigned char dsm[];
    __shared__ __align__(8) uint64_t bars[NSTAGE];
    __shared__ int s_job, s_go, s_flag, s_err;
    __shared__ Coef<T> C;
    __shared__ __align__(16) T fb[3][HY][PW];
    __shared__ double s_red[2 * NV * (NT / 32)];
    __shared__ typename Op::Shared S;

    const int tid = threadIdx.x;
    // The first sweep after the replacement slot re-arms the launch's gate
    // (before any block of it can arrive at the finisher, which may set it).
    if (GateRole<Op>::clears && L.gate != nullptr && blk == 0 && tid == 0) *L.gate = 0u;
    __syncthreads();  // the previous tile of this block is done with the shared state
    if (tid == 0) {
        s_job = find_job(L, blk);
        s_go = Op::active(*L.jobs[s_job].sc) ? 1 : 0;
        s_err = 0;
    }
    __syncthreads();
    if (!s_go) {
        *idle_end = L.jobs[s_job].tile_base + L.jobs[s_job].ntiles;
        return SWEEP_IDLE;
    }
    const Job &J = L.jobs[s_job];
    load_coef<T>(C, J, tid, NT);
    Op::load_shared(S, J, tid);

    const Geo g{J.nx, J.ny, J.nz, J.dir >> 1, (J.dir & 1) ? -1 : 1, J.pitch};
    const int64_t local = blk - J.tile_base;
    const int tx_t = (int)(local % J.tiles_x);
    const int ty_t = (int)((local / J.tiles_x) % J.tiles_y);
    const int tz_t = (int)(local / ((int64_t)J.tiles_x * J.tiles_y));
    const int x0 = tx_t * TX, y0 = ty_t * TY;
    const int z0 = tz_t * J.zc;
    const int z1 = min(z0 + J.zc, g.nz);
    const int pa = max(z0 - 1, 0), pb = min(z1, g.nz - 1);
    const int NP = pb - pa + 1;
    // A thread's points: columns gx, gx + 1 of tile rows ly0 .. ly0 + RPT - 1.
    const int lp = tid % TPR, ly0 = (tid / TPR) * RPT;
    const int gx = x0 + 2 * lp;
    bool v0[RPT], v1[RPT];
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
        v0[r] = gx < g.nx && y0 + ly0 + r < g.ny;
        v1[r] = gx + 1 < g.nx && y0 + ly0 + r < g.ny;
    }
    const bool any_v = v0[0] || v1[0] || (RPT == 2 && (v0[RPT - 1] || v1[RPT - 1]));
    const int64_t plane = (int64_t)g.P * g.ny;
    const int64_t i_col = (int64_t)gx + (int64_t)g.P * (y0 + ly0);

    Op op;
    op.init(J, S);

    const uint32_t raw0 = smem_u32(dsm);
    const uint32_t stage0 = (raw0 + 127u) & ~127u;
    unsigned char *const sbase = dsm + (stage0 - raw0);
    if (tid == 0) {
        if (!ready)
            for (int s = 0; s < NSTAGE; ++s) mbar_init(smem_u32(&bars[s]), 1);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
#pragma unroll
        for (int s = 0; s < SL::N; ++s) prefetch_tmap(op.tmap[s]);
    }
    ready = true;
    __syncthreads();
    // Tile loads of plane pa+q into ring slot (qb + q) % NSTAGE (one thread:
    // thread 0 for the first NSTAGE planes, the refill thread after).
    auto issue = [&](int q) {
#if FAST_TAU_TEST_HOOKS
        if (q == 1 && local == 0 && atomicExch(&J.sc->test_withhold, 0) != 0) return;
#endif
        const int st = (qb + q) % NSTAGE;
        const uint32_t bar = smem_u32(&bars[st]);
        mbar_arrive_expect_tx(bar, (uint32_t)SL::tx_bytes());
#pragma unroll
        for (int s = 0; s < SL::N; ++s) {
            if (SL::interior(s))
                tma_load_3d(stage0 + st * SB + SL::off(s), op.tmap[s], x0, y0, pa + q, bar);
            else
                tma_load_3d(stage0 + st * SB + SL::off(s), op.tmap[s], x0 - box_off(SL::esz(s)), y0 - 1, pa + q, bar);
        }
    };
    if (tid == 0) {
        const int n0 = min(NSTAGE, NP);
        for (int q = 0; q < n0; ++q) issue(q);
    }

    // Halo roles: threads 0..TPR-1 the row above the tile, TPR..2TPR-1 the
    // row below (pairs), then TY threads the column left of the tile and TY
    // the column right of it (single points).  Corners are never read.
    int hrow = 0, hcol = 0, hgx = 0, hgy = 0, hkind = 0;
    if (tid < 2 * TPR) {
        const int t = tid % TPR;
        hkind = 1;
        hrow = tid < TPR ? 0 : HY - 1;
        hgx = x0 + 2 * t;
        hgy = tid < TPR ? y0 - 1 : y0 + TY;
        hcol = 2 * t + 2;
    } else if (tid < 2 * TPR + 2 * TY) {
        const int t = tid - 2 * TPR;
        hkind = 2;
        hrow = 1 + (t % TY);
        hgy = y0 + (t % TY);
        hgx = t < TY ? x0 - 1 : x0 + TX;
        hcol = t < TY ? 1 : TX + 2;
    }
    const bool hin_y = (unsigned)hgy < (unsigned)g.ny;
    const bool h0 = hin_y && (unsigned)hgx < (unsigned)g.nx;
    const bool h1 = hin_y && (unsigned)(hgx + 1) < (unsigned)g.nx;
    const Pt p_halo{hrow, hgx - x0};
    // Boundary counts in x and y of the thread's own columns and halo points
    // (fixed for the slab); the z part is added per plane.
    int bc0[RPT], bc1[RPT];
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
        bc0[r] = boundary_count_xy(g, gx, y0 + ly0 + r);
        bc1[r] = boundary_count_xy(g, gx + 1, y0 + ly0 + r);
    }
    const int hbc0 = boundary_count_xy(g, hgx, hgy), hbc1 = boundary_count_xy(g, hgx + 1, hgy);

    // The field of the thread's points in the planes below (m), at (c) and
    // above (p) the plane the operator is applied to, and the own-point
    // state of the planes c and p.
    T fm0[RPT], fm1[RPT], fc0[RPT], fc1[RPT], fp0[RPT], fp1[RPT];
    typename Op::Own oc0[RPT], oc1[RPT], op0[RPT], op1[RPT];
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
        fm0[r] = fm1[r] = fc0[r] = fc1[r] = fp0[r] = fp1[r] = T(0);
        oc0[r] = oc1[r] = op0[r] = op1[r] = typename Op::Own{};
    }
    // A tile inside the domain in x and y (most tiles) runs the plane loop
    // with every point valid as a compile-time fact, which removes the
    // per-point validity branches; edge tiles test each point.
    // FAST_TAU_FULL_TILE=0 tests the points of every tile.
    const bool full = FAST_TAU_FULL_TILE && x0 + TX <= g.nx && y0 + TY <= g.ny;
    int q = 0;
    auto march = [&](auto full_c) {
        constexpr bool FULL = decltype(full_c)::value;
        auto ok0 = [&](int r) { return FULL || v0[r]; };
        auto ok1 = [&](int r) { return FULL || v1[r]; };
        // The operator at plane zs on the thread's points, from the plane
        // buffer (x and y neighbours; the y neighbour inside the thread's
        // row pair from its registers) and the field of the planes below
        // (fm) and above (u0, u1: 0 past the last plane); stores the outputs.
        auto apply_at = [&](int zs, const T(&u0)[RPT], const T(&u1)[RPT]) {
            const int bczs = boundary_count_z(g, zs);
            const T(*P)[PW] = fb[(unsigned)zs % 3u];
#pragma unroll
            for (int r = 0; r < RPT; ++r) {
                if (!(ok0(r) || ok1(r))) continue;
                const int row = ly0 + r + 1;
                const Pair<T> left = *reinterpret_cast<const Pair<T> *>(&P[row][2 * lp]);
                const Pair<T> right = *reinterpret_cast<const Pair<T> *>(&P[row][2 * lp + 4]);
                T up0, up1, dn0, dn1;
                if (r + 1 < RPT) {
                    up0 = fc0[r + 1];
                    up1 = fc1[r + 1];
                } else {
                    const Pair<T> up = *reinterpret_cast<const Pair<T> *>(&P[row + 1][2 * lp + 2]);
                    up0 = up.a;
                    up1 = up.b;
                }
                if (r > 0) {
                    dn0 = fc0[r - 1];
                    dn1 = fc1[r - 1];
                } else {
                    const Pair<T> dn = *reinterpret_cast<const Pair<T> *>(&P[row - 1][2 * lp + 2]);
                    dn0 = dn.a;
                    dn1 = dn.b;
                }
                const int gy = y0 + ly0 + r;
                const int64_t i = i_col + (int64_t)r * g.P + plane * zs;
                typename Op::Out o0{}, o1{};
                if (ok0(r))
                    o0 = op.apply(g, C, S, oc0[r], Pos{gx, gy, zs, bc0[r] + bczs}, fc0[r], fc1[r], left.b, up0, dn0,
                                  u0[r], fm0[r]);
                if (ok1(r))
                    o1 = op.apply(g, C, S, oc1[r], Pos{gx + 1, gy, zs, bc1[r] + bczs}, fc1[r], right.a, fc0[r], up1,
                                  dn1, u1[r], fm1[r]);
                if (ft_in(J, i, i + 1, plane * g.nz, OOB_SWEEP_STORE)) op.store(i, o0, o1, ok0(r), ok1(r));
            }
        };
        for (; q < NP; ++q) {
            const int zq = pa + q;
            // ring slot and phase (plane counts are never negative)
            const int st = (int)((unsigned)(qb + q) % (unsigned)NSTAGE);
            const uint32_t par = ((unsigned)(qb + q) / (unsigned)NSTAGE) & 1u;
            const unsigned zb = (unsigned)zq % 3u;  // plane-buffer slot
            if (!mbar_wait_bounded<WaitHint<Op>::ns>(smem_u32(&bars[st]), par)) s_err = 1;
            const unsigned char *stage = sbase + st * SB;
            const bool out_plane = zq >= z0 && zq < z1;
            const int bcz = boundary_count_z(g, zq);
#pragma unroll
            for (int r = 0; r < RPT; ++r) {
                const int gy = y0 + ly0 + r;
                V a, b;
                Op::load2(stage, Pt{ly0 + r + 1, 2 * lp}, a, b);
                fp0[r] = T(0);
                fp1[r] = T(0);
                if (out_plane) {
                    if (ok0(r)) op0[r] = op.own(g, C, S, a, Pos{gx, gy, zq, bc0[r] + bcz}, fp0[r]);
                    if (ok1(r)) op1[r] = op.own(g, C, S, b, Pos{gx + 1, gy, zq, bc1[r] + bcz}, fp1[r]);
                    *reinterpret_cast<Pair<T> *>(&fb[zb][ly0 + r + 1][2 * lp + 2]) = Pair<T>{fp0[r], fp1[r]};
                } else {
                    if (ok0(r)) fp0[r] = op.field(g, C, S, a, Pos{gx, gy, zq, bc0[r] + bcz});
                    if (ok1(r)) fp1[r] = op.field(g, C, S, b, Pos{gx + 1, gy, zq, bc1[r] + bcz});
                }
            }
            if (out_plane && hkind == 1) {
                V a, b;
                HaloLoad<Op>::pair(stage, p_halo, a, b);
                const T f0 = h0 ? op.field(g, C, S, a, Pos{hgx, hgy, zq, hbc0 + bcz}) : T(0);
                const T f1 = h1 ? op.field(g, C, S, b, Pos{hgx + 1, hgy, zq, hbc1 + bcz}) : T(0);
                *reinterpret_cast<Pair<T> *>(&fb[zb][hrow][hcol]) = Pair<T>{f0, f1};
            } else if (out_plane && hkind == 2) {
                V a;
                Op::load1(stage, p_halo, a);
                fb[zb][hrow][hcol] = h0 ? op.field(g, C, S, a, Pos{hgx, hgy, zq, hbc0 + bcz}) : T(0);
            }
            __syncthreads();
            if (s_err) break;
            // Every thread is done with this stage: refill it with plane
            // q+NSTAGE.  The last warp issues (the first warps also load the
            // halo rows).
            if (tid == kRefillThread && q + NSTAGE < NP) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue(q + NSTAGE);
            }
            const int zs = zq - 1;
            if (zs >= z0 && zs < z1 && (FULL || any_v)) apply_at(zs, fp0, fp1);
#pragma unroll
            for (int r = 0; r < RPT; ++r) {
                fm0[r] = fc0[r];
                fm1[r] = fc1[r];
                fc0[r] = fp0[r];
                fc1[r] = fp1[r];
                oc0[r] = op0[r];
                oc1[r] = op1[r];
            }
        }
        // The last plane of the volume has no z+1 neighbour: apply it here.
        if (!s_err && pb == z1 - 1 && (FULL || any_v)) {
            T zero[RPT];
#pragma unroll
            for (int r = 0; r < RPT; ++r) zero[r] = T(0);
            apply_at(z1 - 1, zero, zero);
        }
    };
    if (full)
        march(std::true_type{});
    else
        march(std::false_type{});

    if (s_err) {
        // Tile loads did not arrive in time.  Wait (bounded) for the copies
        // this block issued and has not consumed, then fail the job.
        if (tid == 0) {
            const int issued = min(q + NSTAGE, NP);
            for (int k = q; k < issued; ++k)
                mbar_wait_bounded(smem_u32(&bars[(qb + k) % NSTAGE]), (uint32_t)(((qb + k) / NSTAGE) & 1));
            atomicExch(&J.sc->state, (int32_t)FAULT);
        }
        return SWEEP_FAULT;
    }
    qb += NP;

    using RT = typename RedType<Op>::type;
    RT v[NV];
    op.partials(v);
    if (!ft_in(J, local * NPART, local * NPART + NPART - 1, J.ntiles * NPART, OOB_PARTIALS)) return SWEEP_FAULT;
    block_sum_store<NV, RT, NT>(v, J.part + local * NPART, s_red);
    if (arrive_last(J.counter, J.ntiles, &s_flag)) {
        double tot[NV];
        sum_partials<NV, NT>(J.part, J.ntiles, tot, s_red);
        if (tid == 0) {
            for (int k = 0; k < NV && k < 4; k++) J.sc->dbg[k] = tot[k];
            Op::finish(*J.sc, tot);
            *J.counter = 0u;
            if (L.gate != nullptr && J.sc->replace != 0 && J.sc->state == RUNNING) *L.gate = 1u;
        }
    }
    return SWEEP_DONE;
}

// Kernel entries: one tile per block with the compiler's own register
// choice, or (for an operation that is otherwise held to two blocks per SM)
// a bound that fits MB blocks.
template <class Op, int NSTAGE>
__global__ void __launch_bounds__(sweep_threads<Op>()) sweep_kernel(Launch L)
{
    int qb = 0;
    bool ready = false;
    int64_t idle_end;
    sweep_body<Op, NSTAGE>(L, (int64_t)blockIdx.x, qb, ready, &idle_end);
}

template <class Op, int NSTAGE, int MB>
__global__ void __launch_bounds__(sweep_threads<Op>(), MB) sweep_kernel_mb(Launch L)
{
    int qb = 0;
    bool ready = false;
    int64_t idle_end;
    sweep_body<Op, NSTAGE>(L, (int64_t)blockIdx.x, qb, ready, &idle_end);
}

// A resident grid that walks the launch's tiles (tile = blockIdx.x +
// k * gridDim.x) and skips the rest of a right-hand side it finds inactive:
// for operations that most launches leave idle (the residual replacement
// slot of every iteration), so an idle launch costs one wave of blocks.
template <class Op, int NSTAGE>
__global__ void __launch_bounds__(sweep_threads<Op>()) sweep_kernel_tiles(Launch L)
{
    // No replacement pending in the whole launch: leave without touching
    // the job table.
    if (L.gate != nullptr && __ldcg(L.gate) == 0u) return;
    int qb = 0;
    bool ready = false;
    for (int64_t blk = blockIdx.x; blk < L.nblocks;) {
        int64_t idle_end = 0;
        const int r = sweep_body<Op, NSTAGE>(L, blk, qb, ready, &idle_end);
        if (r == SWEEP_FAULT) {
            // The stage ring of this block is unusable now: the right-hand
            // sides of the tiles it leaves undone cannot finish this step
            // either, so they fail too (no partial reduction reaches them).
            if (threadIdx.x == 0)
                for (int64_t b = blk + gridDim.x; b < L.nblocks; b += gridDim.x)
                    atomicExch(&L.jobs[find_job(L, b)].sc->state, (int32_t)FAULT);
            return;
        }
        if (r == SWEEP_IDLE && idle_end > blk + gridDim.x) {
            // first tile >= idle_end that belongs to this block
            blk += ((idle_end - blk + gridDim.x - 1) / gridDim.x) * gridDim.x;
        } else {
            blk += gridDim.x;
        }
    }
}

// ---------------------------------------------------------------------------
// Operation interface.  An op names its streams (SL, code last), loads one
// point's stream values (Vals) for a lane pair (load2) or a single point
// (load1), forms the operand field at a point (field), the same plus what the
// point's own update needs (own -> Own), applies the update from the
// stencil of the field (apply -> Out, accumulating its dot products), and
// writes a lane pair's outputs (store).
// ---------------------------------------------------------------------------
struct NoShared {};
struct NoOut {};

// Shared memory of the sweeps that take the face coefficients of a point
// from the per-code table (FAST_TAU_FACE_TABLE=1; else they select them by
// the code's bits and hold nothing), and their stencil.
#if FAST_TAU_FACE_TABLE
using FaceShared = FaceTable;
__device__ __forceinline__ void load_faces(FaceTable &t, const Job &J, int tid) { load_face_table(t, J, tid); }
#else
using FaceShared = NoShared;
__device__ __forceinline__ void load_faces(NoShared &, const Job &, int) {}
#endif

__device__ __forceinline__ float stencil7s(const Faces<float> &F, const FaceShared &S, uint32_t code, float fc,
                                           float fxp, float fxm, float fyp, float fym, float fzp, float fzm, float diag)
{
#if FAST_TAU_FACE_TABLE
    (void)F;
    return stencil7t<float>(S, code, fc, fxp, fxm, fyp, fym, fzp, fzm, diag);
#else
    (void)S;
    return stencil7<float>(F, code, fc, fxp, fxm, fyp, fym, fzp, fzm, diag);
#endif
}

template <class SL, int S>
__device__ __forceinline__ void load_code2(const unsigned char *st, const Pt &p, uint32_t &a, uint32_t &b)
{
    uint8_t ca, cb;
    sv2<uint8_t, SL, S>(st, p, ca, cb);
    a = ca;
    b = cb;
}

// ===========================================================================
// Setup of a pure-precision solve (F64 or F32): x = x0, r = b - A x0, and the
// Krylov vectors zeroed.  Dots: |b|^2, |r|^2, r.z.
// CG_Solve setup: CG.cu:38-63.  BICG_Solve setup: BICGSTAB.cu:49-91.
// Streams: code.
// ===========================================================================
template <typename TT, typename ST, bool BICG>
struct OpInit {
    using T = TT;
    static constexpr bool FB = sizeof(TT) == 4 && sizeof(ST) == 8;  // MIXED FP32 iterations
    using SL = Streams<1>;
    static constexpr int NV = 3;
    using Shared = NoShared;
    struct Vals { uint32_t code; };
    struct Own { uint32_t code; };
    struct Out { T x, r; };
    const CUtensorMap *tmap[SL::N];
    Faces<T> F;
    T *x, *r, *r0, *p0, *v0;
    Acc<T> bb, rr, rz;

    __device__ static bool active(const Scalars &sc) { return sc.state == RUNNING; }
    __device__ static void load_shared(Shared &, const Job &, int) {}
    __device__ static void load2(const unsigned char *st, const Pt &p, Vals &a, Vals &b)
    {
        load_code2<SL, 0>(st, p, a.code, b.code);
    }
    __device__ static void load1(const unsigned char *st, const Pt &p, Vals &a) { a.code = sv<uint8_t, SL, 0>(st, p); }
    __device__ void init(const Job &J, Shared &)
    {
        F = faces_of<T>(J);
        tmap[0] = &J.tm[TM_CODE];
        x = (T *)J.x; r = (T *)J.r[0]; r0 = (T *)J.r0; p0 = (T *)J.p[0]; v0 = (T *)J.v[0];
    }
    __device__ T field(const Geo &g, const Coef<T> &, Shared &, const Vals &, const Pos &ps) const
    {
        return x0_at<T>(g, ps.x, ps.y, ps.z);
    }
    __device__ Own own(const Geo &g, const Coef<T> &, Shared &, const Vals &v, const Pos &ps, T &f) const
    {
        f = x0_at<T>(g, ps.x, ps.y, ps.z);
        return Own{v.code};
    }
    __device__ Out apply(const Geo &g, const Coef<T> &C, Shared &, const Own &o, const Pos &ps, T fc,
                         T fxp, T fxm, T fyp, T fym, T fzp, T fzm)
    {
        const T d = diag_of<T, FB>(C, g, o.code, ps);
        const T ax = stencil7<T>(F, o.code, fc, fxp, fxm, fyp, fym, fzp, fzm, d);
        const T b = rhs_at<T>(C, g, o.code, ps.x, ps.y, ps.z);
        const T res = b - ax;
        const T inv = inv_from_diag<T, FB>(C, o.code, ps, d);
        bb.add_prod(b, b);
        rr.add_prod(res, res);
        rz.add_prod(res, res * inv);
        return Out{fc, res};
    }
    __device__ void store(int64_t i, const Out &a, const Out &b, bool v0_, bool v1_)
    {
        store2<T>(x, i, a.x, b.x, v0_, v1_);
        store2<T>(r, i, a.r, b.r, v0_, v1_);
        store2<T>(p0, i, T(0), T(0), v0_, v1_);
        if (BICG) {
            store2<T>(r0, i, a.r, b.r, v0_, v1_);
            store2<T>(v0, i, T(0), T(0), v0_, v1_);
        }
    }
    __device__ void partials(T (&v)[NV]) const { v[0] = bb.hi(); v[1] = rr.hi(); v[2] = rz.hi(); }
    __device__ static void finish(Scalars &sc, const double (&t)[NV])
    {
        const ST rhs = (ST)t[0];
        sc.rhs_sq = rhs;
        sc.iter = 0;
        sc.restarts = 0;
        sc.restart = 0;
        if (rhs == ST(0)) {  // CG.cu:41-44, BICGSTAB.cu:66-69
            sc.state = ZERO_RHS;
            return;
        }
        const ST tol = (ST)sc.tol;
        const ST tol2 = tol * tol * rhs;
        sc.tol2 = tol2;
        const ST rsq = (ST)t[1];
        sc.rsq = rsq;
        if (!BICG) {
            sc.zr = (ST)t[2];
            sc.beta = 0.0;
        } else {
            // First pass of the loop head: rho_old = 1, rho = r0.r = |r0|^2,
            // alpha = w = 1, beta = (rho/rho_old)*(alpha/w) (BICGSTAB.cu:71-112).
            sc.r0_sq = rsq;
            sc.alpha = 1.0;
            sc.omega = 1.0;
            const ST rho = rsq;
            sc.rho = rho;
            sc.beta = (double)((rho / ST(1)) * (ST(1) / ST(1)));
        }
        if (!(rsq > tol2)) sc.state = CONVERGED;
        else if (sc.max_iter == 0) sc.state = MAXITER;
        else sc.state = RUNNING;
    }
};

// ===========================================================================
// MIXED iteration control (FP32 vectors, FP64 scalars).  The recursive
// residual of the FP32 iteration stands for b - A (x64 + e); it is replaced
// by the true one (OpReplace) once it has fallen by delta below the largest
// value seen since the last replacement (so the rounding gap between the two,
// proportional to that largest value, stays small against it), when it
// claims convergence (the true residual then decides), and with a Krylov
// restart when the recursion breaks down (BiCGSTAB: r0.r small against
// |r0||r|, or a non-finite or exploding residual).
// ===========================================================================
// mode: what a requested replacement does with the Krylov vectors -- 1 keeps
// them (CG), 2 restarts them from the true residual (BiCGSTAB: a fresh
// shadow residual r0 = r; measured faster on the benchmark than keeping the
// old r0, 6.24 against 6.08 solves/s, with the same accuracy).
__device__ __forceinline__ void mixed_request(Scalars &sc, double rsq, int mode = 1)
{
    if (rsq > sc.rsq_max) sc.rsq_max = rsq;
    if (rsq <= sc.tol2 || rsq < sc.delta2 * sc.rsq_max) sc.replace = mode;
    else if (sc.iter >= sc.max_iter) sc.state = MAXITER;
}

__device__ __forceinline__ void mixed_cg_finish(Scalars &sc, double rsq, double zr_new)
{
    sc.rsq = rsq;
    sc.iter += 1;
    if (!(rsq <= sc.div_thresh)) {  // non-finite or exploding: restart from the true residual
        sc.restarts += 1;
        sc.replace = 2;
        return;
    }
    sc.rho_old = sc.zr;  // r.z of this iteration's start, for a replacement
    sc.beta = zr_new / sc.zr;
    sc.zr = zr_new;
    mixed_request(sc, rsq);
}

__device__ __forceinline__ void mixed_bicg_finish(Scalars &sc, double r0r, double rsq)
{
    sc.rsq = rsq;
    sc.iter += 1;
    if (!(rsq <= sc.div_thresh)) {
        sc.restarts += 1;
        sc.replace = 2;
        return;
    }
    const double rho_old = sc.rho;
    sc.rho_old = rho_old;
    sc.rho = r0r;
    // The shadow residual r0 has become (numerically) orthogonal to r: in
    // FP32, r0.r is noise well before |rho| reaches eps^2 |r0|^2.
    if (fabs(r0r) < sc.eps2 * sc.r0_sq || r0r * r0r < sc.cos2_min * sc.r0_sq * rsq) {
        sc.restarts += 1;
        sc.replace = 2;
        return;
    }
    sc.beta = (r0r / rho_old) * (sc.alpha / sc.omega);
    mixed_request(sc, rsq);
}

// ===========================================================================
// CG step 1: p <- z + beta p (z = r/diag on the fly), q = A p, dot p.q.
// CG.cu:113-135 (z, beta, p update of the previous iteration) + :70-81.
// Streams: r, p_old, code.
// ===========================================================================
// Rows per thread of the MIXED FP32 sweeps (the PCG steps and BiCGSTAB
// step 2); the other sweeps own one row per thread.
#ifndef FAST_TAU_RPT_CG1
#define FAST_TAU_RPT_CG1 2
#endif
#ifndef FAST_TAU_RPT_CG2
#define FAST_TAU_RPT_CG2 2
#endif
#ifndef FAST_TAU_RPT_K2
#define FAST_TAU_RPT_K2 2
#endif

template <typename TT, typename ST>
struct OpCG1 {
    using T = TT;
    static constexpr bool FB = sizeof(TT) == 4 && sizeof(ST) == 8;  // MIXED FP32 iterations
    static constexpr int RPT = FB ? FAST_TAU_RPT_CG1 : 1;
    static constexpr bool clears_gate = FB;
    static constexpr uint32_t wait_hint_ns = FB ? FAST_TAU_HINT_CG : 0;
    using SL = Streams<sizeof(TT), sizeof(TT), 1>;
    static constexpr int NV = 1;
    using Shared = NoShared;
    struct Vals { T r, p; uint32_t code; };
    struct Own { uint32_t code; T d; };
    struct Out { T p; };
    const CUtensorMap *tmap[SL::N];
    Faces<T> F;
    T *pnew;
    T *ezero;  // MIXED: e to zero after a residual replacement, else null
    T beta;
    Acc<T> pap;

    __device__ static bool active(const Scalars &sc) { return sc.state == RUNNING; }
    __device__ static void load_shared(Shared &, const Job &, int) {}
    __device__ static void load2(const unsigned char *st, const Pt &p, Vals &a, Vals &b)
    {
        sv2<T, SL, 0>(st, p, a.r, b.r);
        sv2<T, SL, 1>(st, p, a.p, b.p);
        load_code2<SL, 2>(st, p, a.code, b.code);
    }
    __device__ static void load1(const unsigned char *st, const Pt &p, Vals &a)
    {
        a.r = sv<T, SL, 0>(st, p);
        a.p = sv<T, SL, 1>(st, p);
        a.code = sv<uint8_t, SL, 2>(st, p);
    }
    __device__ void init(const Job &J, Shared &)
    {
        F = faces_of<T>(J);
        const int par = (int)(J.sc->iter & 1);
        tmap[0] = &J.tm[TM_R];
        tmap[1] = &J.tm[TM_P + par];
        tmap[2] = &J.tm[TM_CODE];
        pnew = (T *)J.p[par ^ 1];
        ezero = J.sc->e_reset ? (T *)J.x : nullptr;
        beta = (T)J.sc->beta;
    }
    __device__ T field(const Geo &g, const Coef<T> &C, Shared &, const Vals &v, const Pos &ps) const
    {
        const T zi = v.r * inv_of<T, FB>(C, g, v.code, ps);
        return v.p * beta + zi;  // __aAddAlphaBKernel: p = p*beta + z
    }
    __device__ Own own(const Geo &g, const Coef<T> &C, Shared &, const Vals &v, const Pos &ps, T &f) const
    {
        T d, inv;
        diag_inv<T, FB>(C, g, v.code, ps, d, inv);
        f = v.p * beta + v.r * inv;  // as field()
        return Own{v.code, d};
    }
    __device__ Out apply(const Geo &, const Coef<T> &C, Shared &, const Own &o, const Pos &, T fc,
                         T fxp, T fxm, T fyp, T fym, T fzp, T fzm)
    {
        const T q = stencil7<T>(F, o.code, fc, fxp, fxm, fyp, fym, fzp, fzm, o.d);
        pap.add_prod(fc, q);
        return Out{fc};
    }
    __device__ void store(int64_t i, const Out &a, const Out &b, bool v0, bool v1)
    {
        store2<T>(pnew, i, a.p, b.p, v0, v1);
        if (ezero) store2<T>(ezero, i, T(0), T(0), v0, v1);
    }
    __device__ void partials(T (&v)[NV]) const { v[0] = pap.hi(); }
    __device__ static void finish(Scalars &sc, const double (&t)[NV])
    {
        sc.alpha = (double)((ST)sc.zr / (ST)t[0]);  // CG.cu:79-81
        sc.e_reset = 0;
    }
};

// ===========================================================================
// CG step 2: q = A p (recomputed), x += alpha p, r -= alpha q, z = r/diag,
// dots |r|^2 and r.z; convergence, beta and the iteration count.
// CG.cu:87-154.  Streams: p, x, r, code.
// ===========================================================================
template <typename TT, typename ST>
struct OpCG2 {
    using T = TT;
    static constexpr bool FB = sizeof(TT) == 4 && sizeof(ST) == 8;  // MIXED FP32 iterations
    static constexpr int RPT = FB ? FAST_TAU_RPT_CG2 : 1;
    static constexpr uint32_t wait_hint_ns = FB ? FAST_TAU_HINT_CG : 0;
    // p (halo), x and r (own points only), code
    using SL = Streams<sizeof(TT), own_only(sizeof(TT)), own_only(sizeof(TT)), 1>;
    static constexpr int NV = 2;
    using Shared = NoShared;
    struct Vals { T p, x, r; uint32_t code; };
    struct Own { uint32_t code; T x, r; };
    struct Out { T x, r; };
    const CUtensorMap *tmap[SL::N];
    Faces<T> F;
    T *x, *r;
    T alpha;
    Acc<T> rr, rz;

    __device__ static bool active(const Scalars &sc) { return sc.state == RUNNING; }
    __device__ static void load_shared(Shared &, const Job &, int) {}
    __device__ static void load2(const unsigned char *st, const Pt &p, Vals &a, Vals &b)
    {
        sv2<T, SL, 0>(st, p, a.p, b.p);
        sv2<T, SL, 1>(st, p, a.x, b.x);
        sv2<T, SL, 2>(st, p, a.r, b.r);
        load_code2<SL, 3>(st, p, a.code, b.code);
    }
    __device__ static void load2h(const unsigned char *st, const Pt &p, Vals &a, Vals &b)
    {
        sv2<T, SL, 0>(st, p, a.p, b.p);
    }
    __device__ static void load1(const unsigned char *st, const Pt &p, Vals &a) { a.p = sv<T, SL, 0>(st, p); }
    __device__ void init(const Job &J, Shared &)
    {
        F = faces_of<T>(J);
        const int par = (int)(J.sc->iter & 1);
        tmap[0] = &J.tm[TM_P + (par ^ 1)];
        tmap[1] = &J.tm[FAST_TAU_INTERIOR ? TM_XI : TM_X];
        tmap[2] = &J.tm[FAST_TAU_INTERIOR ? TM_RI : TM_R];
        tmap[3] = &J.tm[TM_CODE];
        x = (T *)J.x;
        r = (T *)J.r[0];
        alpha = (T)J.sc->alpha;
    }
    __device__ T field(const Geo &, const Coef<T> &, Shared &, const Vals &v, const Pos &) const { return v.p; }
    __device__ Own own(const Geo &, const Coef<T> &, Shared &, const Vals &v, const Pos &, T &f) const
    {
        f = v.p;
        return Own{v.code, v.x, v.r};
    }
    __device__ Out apply(const Geo &g, const Coef<T> &C, Shared &, const Own &o, const Pos &ps, T fc,
                         T fxp, T fxm, T fyp, T fym, T fzp, T fzm)
    {
        T d, inv;
        diag_inv<T, FB>(C, g, o.code, ps, d, inv);
        const T q = stencil7<T>(F, o.code, fc, fxp, fxm, fyp, fym, fzp, fzm, d);
        const T xn = o.x + alpha * fc;        // __aAddBetaBKernel(x, p, alpha)
        const T rn = o.r + (-alpha) * q;      // __aAddBetaBKernel(r, ap, -alpha)
        rr.add_prod(rn, rn);
        rz.add_prod(rn, rn * inv);
        return Out{xn, rn};
    }
    __device__ void store(int64_t i, const Out &a, const Out &b, bool v0, bool v1)
    {
        store2<T>(x, i, a.x, b.x, v0, v1);
        store2<T>(r, i, a.r, b.r, v0, v1);
    }
    __device__ void partials(T (&v)[NV]) const { v[0] = rr.hi(); v[1] = rz.hi(); }
    __device__ static void finish(Scalars &sc, const double (&t)[NV])
    {
        if (sc.inner_mode) {
            mixed_cg_finish(sc, t[0], t[1]);
            return;
        }
        const ST rsq = (ST)t[0];
        sc.rsq = rsq;
        if (rsq <= (ST)sc.tol2) {  // CG.cu:108-110: converging iteration not counted
            sc.state = CONVERGED;
            return;
        }
        const ST zr_new = (ST)t[1];
        sc.beta = (double)(zr_new / (ST)sc.zr);  // CG.cu:121-123
        sc.zr = zr_new;
        sc.iter += 1;                            // CG.cu:144
        if (rsq > (ST)sc.div_thresh) sc.state = DIVERGED;  // CG.cu:152
        else if (sc.iter >= sc.max_iter) sc.state = MAXITER;
    }
};

// ===========================================================================
// BiCGSTAB restart (BICGSTAB.cu:103-110): when |rho| < eps^2 |r0|^2 the
// residual is recomputed from x and becomes the new shadow residual.  Runs
// as a no-op kernel unless a restart is pending.  Streams: x, code.
// ===========================================================================
template <typename TT, typename ST>
struct OpBiRestart {
    using T = TT;
    static constexpr bool FB = sizeof(TT) == 4 && sizeof(ST) == 8;  // MIXED FP32 iterations
    using SL = Streams<sizeof(TT), 1>;
    static constexpr int NV = 1;
    using Shared = NoShared;
    struct Vals { T x; uint32_t code; };
    struct Own { uint32_t code; };
    struct Out { T r; };
    const CUtensorMap *tmap[SL::N];
    Faces<T> F;
    T *r, *r0;
    Acc<T> rr;

    __device__ static bool active(const Scalars &sc) { return sc.state == RUNNING && sc.restart != 0; }
    __device__ static void load_shared(Shared &, const Job &, int) {}
    __device__ static void load2(const unsigned char *st, const Pt &p, Vals &a, Vals &b)
    {
        sv2<T, SL, 0>(st, p, a.x, b.x);
        load_code2<SL, 1>(st, p, a.code, b.code);
    }
    __device__ static void load1(const unsigned char *st, const Pt &p, Vals &a) { a.x = sv<T, SL, 0>(st, p); }
    __device__ void init(const Job &J, Shared &)
    {
        F = faces_of<T>(J);
        const int par = (int)(J.sc->iter & 1);
        tmap[0] = &J.tm[TM_X];
        tmap[1] = &J.tm[TM_CODE];
        r = (T *)J.r[par];
        r0 = (T *)J.r0;
    }
    __device__ T field(const Geo &, const Coef<T> &, Shared &, const Vals &v, const Pos &) const { return v.x; }
    __device__ Own own(const Geo &, const Coef<T> &, Shared &, const Vals &v, const Pos &, T &f) const
    {
        f = v.x;
        return Own{v.code};
    }
    __device__ Out apply(const Geo &g, const Coef<T> &C, Shared &, const Own &o, const Pos &ps, T fc,
                         T fxp, T fxm, T fyp, T fym, T fzp, T fzm)
    {
        const T d = diag_of<T, FB>(C, g, o.code, ps);
        const T ax = stencil7<T>(F, o.code, fc, fxp, fxm, fyp, fym, fzp, fzm, d);
        const T res = rhs_at<T>(C, g, o.code, ps.x, ps.y, ps.z) - ax;
        rr.add_prod(res, res);
        return Out{res};
    }
    __device__ void store(int64_t i, const Out &a, const Out &b, bool v0, bool v1)
    {
        store2<T>(r, i, a.r, b.r, v0, v1);
        store2<T>(r0, i, a.r, b.r, v0, v1);
    }
    __device__ void partials(T (&v)[NV]) const { v[0] = rr.hi(); }
    __device__ static void finish(Scalars &sc, const double (&t)[NV])
    {
        const ST rho = (ST)t[0];
        sc.r0_sq = rho;
        sc.rho = rho;
        sc.restarts += 1;
        sc.restart = 0;
        const ST rho_old = (ST)sc.rho_old;
        sc.beta = (double)((rho / rho_old) * ((ST)sc.alpha / (ST)sc.omega));
    }
};

// ===========================================================================
// BiCGSTAB step 1: p <- r + beta (p - w v), y = p/diag, v = A y, dot r0.v.
// BICGSTAB.cu:112-147.  Streams: r, p_old, v_old, r0, code.
// ===========================================================================
template <typename TT, typename ST>
struct OpBi1 {
    using T = TT;
    static constexpr bool FB = sizeof(TT) == 4 && sizeof(ST) == 8;  // MIXED FP32 iterations
    using SL = Streams<sizeof(TT), sizeof(TT), sizeof(TT), sizeof(TT), 1>;
    static constexpr int NV = 1;
    using Shared = NoShared;
    struct Vals { T r, p, v, r0; uint32_t code; };
    struct Own { uint32_t code; T p, r0; };
    struct Out { T p, v; };
    const CUtensorMap *tmap[SL::N];
    Faces<T> F;
    T *pnew, *vnew;
    T *ezero;  // MIXED: e to zero after a residual replacement, else null
    T beta, nw;
    Acc<T> r0v;

    __device__ static bool active(const Scalars &sc) { return sc.state == RUNNING; }
    __device__ static void load_shared(Shared &, const Job &, int) {}
    __device__ static void load2(const unsigned char *st, const Pt &p, Vals &a, Vals &b)
    {
        sv2<T, SL, 0>(st, p, a.r, b.r);
        sv2<T, SL, 1>(st, p, a.p, b.p);
        sv2<T, SL, 2>(st, p, a.v, b.v);
        sv2<T, SL, 3>(st, p, a.r0, b.r0);
        load_code2<SL, 4>(st, p, a.code, b.code);
    }
    __device__ static void load1(const unsigned char *st, const Pt &p, Vals &a)
    {
        a.r = sv<T, SL, 0>(st, p);
        a.p = sv<T, SL, 1>(st, p);
        a.v = sv<T, SL, 2>(st, p);
        a.code = sv<uint8_t, SL, 4>(st, p);
    }
    __device__ void init(const Job &J, Shared &)
    {
        F = faces_of<T>(J);
        const int par = (int)(J.sc->iter & 1);
        tmap[0] = &J.tm[TM_R + par];
        tmap[1] = &J.tm[TM_P + par];
        tmap[2] = &J.tm[TM_V + par];
        tmap[3] = &J.tm[TM_R0];
        tmap[4] = &J.tm[TM_CODE];
        pnew = (T *)J.p[par ^ 1];
        vnew = (T *)J.v[par ^ 1];
        ezero = J.sc->e_reset ? (T *)J.x : nullptr;
        beta = (T)J.sc->beta;
        nw = (T)(-J.sc->omega);
    }
    // __aPlusBetaBGammaPlusCKernel: p = beta*(p + (-w)*v) + r
    __device__ __forceinline__ T pval(const Vals &v) const { return beta * (v.p + nw * v.v) + v.r; }
    __device__ T field(const Geo &g, const Coef<T> &C, Shared &, const Vals &v, const Pos &ps) const
    {
        return pval(v) * inv_of<T, FB>(C, g, v.code, ps);
    }
    __device__ Own own(const Geo &g, const Coef<T> &C, Shared &, const Vals &v, const Pos &ps, T &f) const
    {
        const T pn = pval(v);
        f = pn * inv_of<T, FB>(C, g, v.code, ps);
        return Own{v.code, pn, v.r0};
    }
    __device__ Out apply(const Geo &g, const Coef<T> &C, Shared &, const Own &o, const Pos &ps, T fc,
                         T fxp, T fxm, T fyp, T fym, T fzp, T fzm)
    {
        const T d = diag_of<T, FB>(C, g, o.code, ps);
        const T vn = stencil7<T>(F, o.code, fc, fxp, fxm, fyp, fym, fzp, fzm, d);
        r0v.add_prod(o.r0, vn);
        return Out{o.p, vn};
    }
    __device__ void store(int64_t i, const Out &a, const Out &b, bool v0, bool v1)
    {
        store2<T>(pnew, i, a.p, b.p, v0, v1);
        store2<T>(vnew, i, a.v, b.v, v0, v1);
        if (ezero) store2<T>(ezero, i, T(0), T(0), v0, v1);
    }
    __device__ void partials(T (&v)[NV]) const { v[0] = r0v.hi(); }
    __device__ static void finish(Scalars &sc, const double (&t)[NV])
    {
        sc.alpha = (double)((ST)sc.rho / (ST)t[0]);  // BICGSTAB.cu:147
        sc.e_reset = 0;
    }
};

// ===========================================================================
// BiCGSTAB step 2: s = r - alpha v, z = s/diag, t = A z, dots t.s, t.t.
// BICGSTAB.cu:149-183.  Streams: r, v_new, code.
// ===========================================================================
template <typename TT, typename ST>
struct OpBi2 {
    using T = TT;
    static constexpr bool FB = sizeof(TT) == 4 && sizeof(ST) == 8;  // MIXED FP32 iterations
    using SL = Streams<sizeof(TT), sizeof(TT), 1>;
    static constexpr int NV = 2;
    using Shared = NoShared;
    struct Vals { T r, v; uint32_t code; };
    struct Own { uint32_t code; T s; };
    using Out = NoOut;
    const CUtensorMap *tmap[SL::N];
    Faces<T> F;
    T nalpha;
    Acc<T> ts, tt;

    __device__ static bool active(const Scalars &sc) { return sc.state == RUNNING; }
    __device__ static void load_shared(Shared &, const Job &, int) {}
    __device__ static void load2(const unsigned char *st, const Pt &p, Vals &a, Vals &b)
    {
        sv2<T, SL, 0>(st, p, a.r, b.r);
        sv2<T, SL, 1>(st, p, a.v, b.v);
        load_code2<SL, 2>(st, p, a.code, b.code);
    }
    __device__ static void load1(const unsigned char *st, const Pt &p, Vals &a)
    {
        a.r = sv<T, SL, 0>(st, p);
        a.v = sv<T, SL, 1>(st, p);
        a.code = sv<uint8_t, SL, 2>(st, p);
    }
    __device__ void init(const Job &J, Shared &)
    {
        F = faces_of<T>(J);
        const int par = (int)(J.sc->iter & 1);
        tmap[0] = &J.tm[TM_R + par];
        tmap[1] = &J.tm[TM_V + (par ^ 1)];
        tmap[2] = &J.tm[TM_CODE];
        nalpha = (T)(-J.sc->alpha);
    }
    __device__ __forceinline__ T sval(const Vals &v) const { return v.r + nalpha * v.v; }  // s = r + (-alpha) v
    __device__ T field(const Geo &g, const Coef<T> &C, Shared &, const Vals &v, const Pos &ps) const
    {
        return sval(v) * inv_of<T, FB>(C, g, v.code, ps);
    }
    __device__ Own own(const Geo &g, const Coef<T> &C, Shared &, const Vals &v, const Pos &ps, T &f) const
    {
        const T s = sval(v);
        f = s * inv_of<T, FB>(C, g, v.code, ps);
        return Own{v.code, s};
    }
    __device__ Out apply(const Geo &g, const Coef<T> &C, Shared &, const Own &o, const Pos &ps, T fc,
                         T fxp, T fxm, T fyp, T fym, T fzp, T fzm)
    {
        const T d = diag_of<T, FB>(C, g, o.code, ps);
        const T t = stencil7<T>(F, o.code, fc, fxp, fxm, fyp, fym, fzp, fzm, d);
        ts.add_prod(t, o.s);
        tt.add_prod(t, t);
        return Out{};
    }
    __device__ void store(int64_t, const Out &, const Out &, bool, bool) {}
    __device__ void partials(T (&v_)[NV]) const { v_[0] = ts.hi(); v_[1] = tt.hi(); }
    __device__ static void finish(Scalars &sc, const double (&t)[NV])
    {
        const ST tmp = (ST)t[1];
        sc.omega = (tmp > ST(0)) ? (double)((ST)t[0] / tmp) : 0.0;  // BICGSTAB.cu:175-183
    }
};

// ===========================================================================
// BiCGSTAB step 3: t recomputed, x += alpha y + w z, r = s - w t, dots r0.r and
// |r|^2; divergence, iteration count, convergence, next rho/beta or a
// restart.  BICGSTAB.cu:187-212 + the loop head :93-112.
// Streams: r, v_new, p_new, x, r0, code.
// ===========================================================================
template <typename TT, typename ST>
struct OpBi3 {
    using T = TT;
    static constexpr bool FB = sizeof(TT) == 4 && sizeof(ST) == 8;  // MIXED FP32 iterations
    using SL = Streams<sizeof(TT), sizeof(TT), sizeof(TT), sizeof(TT), sizeof(TT), 1>;
    static constexpr int NV = 2;
    using Shared = NoShared;
    struct Vals { T r, v, p, x, r0; uint32_t code; };
    struct Own { uint32_t code; T s, x, y, r0; };
    struct Out { T x, r; };
    const CUtensorMap *tmap[SL::N];
    Faces<T> F;
    T *x, *rnew;
    T alpha, omega, nalpha, nomega;
    Acc<T> r0r, rr;

    __device__ static bool active(const Scalars &sc) { return sc.state == RUNNING; }
    __device__ static void load_shared(Shared &, const Job &, int) {}
    __device__ static void load2(const unsigned char *st, const Pt &p, Vals &a, Vals &b)
    {
        sv2<T, SL, 0>(st, p, a.r, b.r);
        sv2<T, SL, 1>(st, p, a.v, b.v);
        sv2<T, SL, 2>(st, p, a.p, b.p);
        sv2<T, SL, 3>(st, p, a.x, b.x);
        sv2<T, SL, 4>(st, p, a.r0, b.r0);
        load_code2<SL, 5>(st, p, a.code, b.code);
    }
    __device__ static void load1(const unsigned char *st, const Pt &p, Vals &a)
    {
        a.r = sv<T, SL, 0>(st, p);
        a.v = sv<T, SL, 1>(st, p);
        a.code = sv<uint8_t, SL, 5>(st, p);
    }
    __device__ void init(const Job &J, Shared &)
    {
        F = faces_of<T>(J);
        const int par = (int)(J.sc->iter & 1);
        tmap[0] = &J.tm[TM_R + par];
        tmap[1] = &J.tm[TM_V + (par ^ 1)];
        tmap[2] = &J.tm[TM_P + (par ^ 1)];
        tmap[3] = &J.tm[TM_X];
        tmap[4] = &J.tm[TM_R0];
        tmap[5] = &J.tm[TM_CODE];
        x = (T *)J.x;
        rnew = (T *)J.r[par ^ 1];
        alpha = (T)J.sc->alpha;
        omega = (T)J.sc->omega;
        nalpha = -alpha;
        nomega = -omega;
    }
    __device__ __forceinline__ T sval(const Vals &v) const { return v.r + nalpha * v.v; }
    __device__ T field(const Geo &g, const Coef<T> &C, Shared &, const Vals &v, const Pos &ps) const
    {
        return sval(v) * inv_of<T, FB>(C, g, v.code, ps);
    }
    __device__ Own own(const Geo &g, const Coef<T> &C, Shared &, const Vals &v, const Pos &ps, T &f) const
    {
        const T s = sval(v);
        const T inv = inv_of<T, FB>(C, g, v.code, ps);
        f = s * inv;
        return Own{v.code, s, v.x, v.p * inv, v.r0};
    }
    __device__ Out apply(const Geo &g, const Coef<T> &C, Shared &, const Own &o, const Pos &ps, T fc,
                         T fxp, T fxm, T fyp, T fym, T fzp, T fzm)
    {
        const T d = diag_of<T, FB>(C, g, o.code, ps);
        const T t = stencil7<T>(F, o.code, fc, fxp, fxm, fyp, fym, fzp, fzm, d);
        const T xn = o.x + (alpha * o.y + omega * fc);   // __ABC_BetaGammaKernel: x += a*y + w*z
        const T rn = o.s + nomega * t;                   // __aPlusBetaBKernel(s, t, r, -w)
        r0r.add_prod(o.r0, rn);
        rr.add_prod(rn, rn);
        return Out{xn, rn};
    }
    __device__ void store(int64_t i, const Out &a, const Out &b, bool v0, bool v1)
    {
        store2<T>(x, i, a.x, b.x, v0, v1);
        store2<T>(rnew, i, a.r, b.r, v0, v1);
    }
    __device__ void partials(T (&v_)[NV]) const { v_[0] = r0r.hi(); v_[1] = rr.hi(); }
    __device__ static void finish(Scalars &sc, const double (&t)[NV])
    {
        if (sc.inner_mode) {
            mixed_bicg_finish(sc, t[0], t[1]);
            return;
        }
        const ST rsq = (ST)t[1];
        sc.rsq = rsq;
        if (rsq > (ST)sc.div_thresh) {  // BICGSTAB.cu:206-209, before ++i
            sc.state = DIVERGED;
            return;
        }
        sc.iter += 1;  // BICGSTAB.cu:211
        if (!(rsq > (ST)sc.tol2)) { sc.state = CONVERGED; return; }
        if (sc.iter >= sc.max_iter) { sc.state = MAXITER; return; }
        // Loop head of the next iteration (BICGSTAB.cu:95-112).
        const ST rho_old = (ST)sc.rho;
        const ST rho = (ST)t[0];
        sc.rho_old = rho_old;
        sc.rho = rho;
        const ST mag = rho < ST(0) ? -rho : rho;
        if (mag < (ST)sc.eps2 * (ST)sc.r0_sq) {
            sc.restart = 1;
        } else {
            sc.beta = (double)((rho / rho_old) * ((ST)sc.alpha / (ST)sc.omega));
        }
    }
};

// ===========================================================================
// MIXED BiCGSTAB in two sweeps per iteration (FP32 vectors, FP64 scalars).
// The reference's three steps (BICGSTAB.cu:112-212) regroup so that every
// global dot product still precedes the vectors that need it:
//   step 1 (iteration k): r_k = s - w t and e += a y + w z of iteration k-1
//     (pointwise, from r, v, t, p of k-1), then p_k = r_k + b (p - w v),
//     v_k = A (p_k / diag); dots r0.v_k, |r_k|^2, r0.r_k;
//   step 2: s = r_k - a v_k, t = A (s / diag) (stored); dots t.s, t.t, r0.t,
//     r0.s, from which w = t.s / t.t and rho_{k+1} = r0.r_{k+1} =
//     r0.s - w r0.t follow without a third sweep.
// The FP64 residual replacement runs at the head of an iteration: it forms
// the iterate of the pending updates on the fly, folds it into x64 and hands
// fp32(b - A x64) to step 1 through t (k1_mode = 1: r_k = t, e = 0).
// ===========================================================================
__device__ __forceinline__ void bicg2_k1_finish(Scalars &sc, double r0v, double rr)
{
    sc.k1_mode = 0;
    sc.rsq = rr;
    sc.iter += 1;
    if (!(rr <= sc.div_thresh)) {  // non-finite or exploding: restart from the true residual
        sc.restarts += 1;
        sc.replace = 2;
        return;
    }
    sc.alpha = sc.rho / r0v;
    if (!(fabs(sc.alpha) < 1e300)) {
        sc.restarts += 1;
        sc.replace = 2;
        return;
    }
    mixed_request(sc, rr, 2);
}

__device__ __forceinline__ void bicg2_k2_finish(Scalars &sc, double ts, double tt, double r0t, double r0s)
{
    const double omega = tt > 0.0 ? ts / tt : 0.0;
    sc.omega = omega;
    const double rho_new = r0s - omega * r0t;
    const double rho_old = sc.rho;
    sc.rho_old = rho_old;
    sc.rho = rho_new;
    // w = 0 (t vanished) or a shadow residual numerically orthogonal to r
    // (in FP32, r0.r is noise well before |rho| reaches eps^2 |r0|^2): restart
    // from the true residual.
    if (omega == 0.0 || fabs(rho_new) < sc.eps2 * sc.r0_sq || rho_new * rho_new < sc.cos2_min * sc.r0_sq * sc.rsq) {
        sc.restarts += 1;
        sc.replace = 2;
        return;
    }
    sc.beta = (rho_new / rho_old) * (sc.alpha / omega);
}

#ifndef FAST_TAU_HINT_K1
#define FAST_TAU_HINT_K1 20000
#endif
#ifndef FAST_TAU_HINT_K2
#define FAST_TAU_HINT_K2 0
#endif

struct OpBiK1 {
    using T = float;
    static constexpr bool FB = true;
    static constexpr bool clears_gate = true;
    static constexpr uint32_t wait_hint_ns = FAST_TAU_HINT_K1;
    using SL = Streams<4, 4, 4, 4, own_only(4), own_only(4), 1>;  // r, v, t, p (halo), e, r0 (own points only), code
    static constexpr int NV = 2;
    using Shared = FaceShared;
    struct Vals { float r, v, t, p, e, r0; uint32_t code; };
    struct Own { uint32_t code; float rk, pk, e, r0; };
    struct Out { float r, p, v, e; };
    const CUtensorMap *tmap[SL::N];
    Faces<T> F;
    float *rnew, *pnew, *vnew, *e;
    float cr, cv, ct, ce, beta, nomega, alpha, omega;
    Acc<float> r0v, rr;

    __device__ static bool active(const Scalars &sc) { return sc.state == RUNNING; }
    __device__ static void load_shared(Shared &S, const Job &J, int tid) { load_faces(S, J, tid); }
    __device__ static void load2(const unsigned char *st, const Pt &p, Vals &a, Vals &b)
    {
        sv2<float, SL, 0>(st, p, a.r, b.r);
        sv2<float, SL, 1>(st, p, a.v, b.v);
        sv2<float, SL, 2>(st, p, a.t, b.t);
        sv2<float, SL, 3>(st, p, a.p, b.p);
        sv2<float, SL, 4>(st, p, a.e, b.e);
        sv2<float, SL, 5>(st, p, a.r0, b.r0);
        load_code2<SL, 6>(st, p, a.code, b.code);
    }
    __device__ static void load1(const unsigned char *st, const Pt &p, Vals &a)
    {
        a.r = sv<float, SL, 0>(st, p);
        a.v = sv<float, SL, 1>(st, p);
        a.t = sv<float, SL, 2>(st, p);
        a.p = sv<float, SL, 3>(st, p);
        a.code = sv<uint8_t, SL, 6>(st, p);
    }
    __device__ static void load2h(const unsigned char *st, const Pt &p, Vals &a, Vals &b)
    {
        sv2<float, SL, 0>(st, p, a.r, b.r);
        sv2<float, SL, 1>(st, p, a.v, b.v);
        sv2<float, SL, 2>(st, p, a.t, b.t);
        sv2<float, SL, 3>(st, p, a.p, b.p);
        load_code2<SL, 6>(st, p, a.code, b.code);
    }
    __device__ void init(const Job &J, Shared &)
    {
        F = faces_of<T>(J);
        const Scalars &sc = *J.sc;
        const int par = (int)(sc.iter & 1);
        tmap[0] = &J.tm[TM_R + par];
        tmap[1] = &J.tm[TM_V + par];
        tmap[2] = &J.tm[TM_T];
        tmap[3] = &J.tm[TM_P + par];
        tmap[4] = &J.tm[FAST_TAU_INTERIOR ? TM_XI : TM_X];
        tmap[5] = &J.tm[FAST_TAU_INTERIOR ? TM_R0I : TM_R0];
        tmap[6] = &J.tm[TM_CODE];
        rnew = (float *)J.r[par ^ 1];
        pnew = (float *)J.p[par ^ 1];
        vnew = (float *)J.v[par ^ 1];
        e = (float *)J.x;
        alpha = (float)sc.alpha;
        omega = (float)sc.omega;
        if (sc.k1_mode) {  // r_k = t (the true residual), e folded into x64
            cr = 0.f; cv = 0.f; ct = 1.f; ce = 0.f;
        } else {           // r_k = r - a v - w t
            cr = 1.f; cv = -alpha; ct = -omega; ce = 1.f;
        }
        beta = (float)sc.beta;
        nomega = -omega;
    }
    __device__ __forceinline__ float rk(const Vals &v) const { return cr * v.r + cv * v.v + ct * v.t; }
    __device__ __forceinline__ float pk(const Vals &v, float r) const { return r + beta * (v.p + nomega * v.v); }
    __device__ T field(const Geo &g, const Coef<T> &C, Shared &, const Vals &v, const Pos &ps) const
    {
        return pk(v, rk(v)) * inv_of<T, FB>(C, g, v.code, ps);
    }
    __device__ Own own(const Geo &g, const Coef<T> &C, Shared &, const Vals &v, const Pos &ps, T &f) const
    {
        const float inv = inv_of<T, FB>(C, g, v.code, ps);
        const float r = rk(v), p = pk(v, r);
        f = p * inv;
        // e_k = e + a y + w z, y = p_{k-1}/diag, z = s_{k-1}/diag
        const float en = ce * (v.e + alpha * (v.p * inv) + omega * ((v.r - alpha * v.v) * inv));
        return Own{v.code, r, p, en, v.r0};
    }
    __device__ Out apply(const Geo &g, const Coef<T> &C, Shared &S, const Own &o, const Pos &ps, T fc, T fxp, T fxm,
                         T fyp, T fym, T fzp, T fzm)
    {
        const T d = diag_of<T, FB>(C, g, o.code, ps);
        const T vn = stencil7s(F, S, o.code, fc, fxp, fxm, fyp, fym, fzp, fzm, d);
        r0v.add_prod(o.r0, vn);
        rr.add_prod(o.rk, o.rk);
        return Out{o.rk, o.pk, vn, o.e};
    }
    __device__ void store(int64_t i, const Out &a, const Out &b, bool v0, bool v1)
    {
        store2<float>(rnew, i, a.r, b.r, v0, v1);
        store2<float>(pnew, i, a.p, b.p, v0, v1);
        store2<float>(vnew, i, a.v, b.v, v0, v1);
        store2<float>(e, i, a.e, b.e, v0, v1);
    }
    __device__ void partials(T (&v_)[NV]) const { v_[0] = r0v.hi(); v_[1] = rr.hi(); }
    __device__ static void finish(Scalars &sc, const double (&t)[NV]) { bicg2_k1_finish(sc, t[0], t[1]); }
};

struct OpBiK2 {
    using T = float;
    static constexpr bool FB = true;
    static constexpr int RPT = FAST_TAU_RPT_K2;
    static constexpr uint32_t wait_hint_ns = FAST_TAU_HINT_K2;
    using SL = Streams<4, 4, own_only(4), 1>;  // r, v (halo), r0 (own points only), code
    static constexpr int NV = 4;
    using Shared = FaceShared;
    struct Vals { float r, v, r0; uint32_t code; };
    struct Own { uint32_t code; float s, r0; };
    struct Out { float t; };
    const CUtensorMap *tmap[SL::N];
    Faces<T> F;
    float *tout;
    float nalpha;
    Acc<float> ts, tt, r0t, r0s;

    __device__ static bool active(const Scalars &sc) { return sc.state == RUNNING; }
    __device__ static void load_shared(Shared &S, const Job &J, int tid) { load_faces(S, J, tid); }
    __device__ static void load2(const unsigned char *st, const Pt &p, Vals &a, Vals &b)
    {
        sv2<float, SL, 0>(st, p, a.r, b.r);
        sv2<float, SL, 1>(st, p, a.v, b.v);
        sv2<float, SL, 2>(st, p, a.r0, b.r0);
        load_code2<SL, 3>(st, p, a.code, b.code);
    }
    __device__ static void load1(const unsigned char *st, const Pt &p, Vals &a)
    {
        a.r = sv<float, SL, 0>(st, p);
        a.v = sv<float, SL, 1>(st, p);
        a.code = sv<uint8_t, SL, 3>(st, p);
    }
    __device__ static void load2h(const unsigned char *st, const Pt &p, Vals &a, Vals &b)
    {
        sv2<float, SL, 0>(st, p, a.r, b.r);
        sv2<float, SL, 1>(st, p, a.v, b.v);
        load_code2<SL, 3>(st, p, a.code, b.code);
    }
    __device__ void init(const Job &J, Shared &)
    {
        F = faces_of<T>(J);
        const int par = (int)(J.sc->iter & 1);  // step 1 has counted the iteration
        tmap[0] = &J.tm[TM_R + par];
        tmap[1] = &J.tm[TM_V + par];
        tmap[2] = &J.tm[FAST_TAU_INTERIOR ? TM_R0I : TM_R0];
        tmap[3] = &J.tm[TM_CODE];
        tout = (float *)J.t;
        nalpha = (float)(-J.sc->alpha);
    }
    __device__ T field(const Geo &g, const Coef<T> &C, Shared &, const Vals &v, const Pos &ps) const
    {
        return (v.r + nalpha * v.v) * inv_of<T, FB>(C, g, v.code, ps);
    }
    __device__ Own own(const Geo &g, const Coef<T> &C, Shared &, const Vals &v, const Pos &ps, T &f) const
    {
        const float s = v.r + nalpha * v.v;
        f = s * inv_of<T, FB>(C, g, v.code, ps);
        return Own{v.code, s, v.r0};
    }
    __device__ Out apply(const Geo &g, const Coef<T> &C, Shared &S, const Own &o, const Pos &ps, T fc, T fxp, T fxm,
                         T fyp, T fym, T fzp, T fzm)
    {
        const T d = diag_of<T, FB>(C, g, o.code, ps);
        const T t = stencil7s(F, S, o.code, fc, fxp, fxm, fyp, fym, fzp, fzm, d);
        ts.add_prod(t, o.s);
        tt.add_prod(t, t);
        r0t.add_prod(o.r0, t);
        r0s.add_prod(o.r0, o.s);
        return Out{t};
    }
    __device__ void store(int64_t i, const Out &a, const Out &b, bool v0, bool v1)
    {
        store2<float>(tout, i, a.t, b.t, v0, v1);
    }
    __device__ void partials(T (&v_)[NV]) const { v_[0] = ts.hi(); v_[1] = tt.hi(); v_[2] = r0t.hi(); v_[3] = r0s.hi(); }
    __device__ static void finish(Scalars &sc, const double (&t)[NV]) { bicg2_k2_finish(sc, t[0], t[1], t[2], t[3]); }
};

// ===========================================================================
// MIXED CG in one sweep per iteration: Chronopoulos & Gear's CG (one
// reduction phase per iteration), with w = A u (u = r/diag) and s = A p kept
// as vectors so that the sweep's only stencil is the one on u.  Sweep k
// applies the pending updates of iteration k-1 pointwise,
//   p = u + beta p,  s = w + beta s,  e += alpha p,  r -= alpha s
// (u from the incoming r, w as stored), then forms u_k = r_k/diag (at the
// halo too, from the same pointwise update of its r, s, w), w_k = A u_k and
// the dots gamma = r_k.u_k, delta = w_k.u_k and |r_k|^2.  The finisher turns
// them into beta = gamma/gamma_old and alpha = gamma/(delta - beta
// gamma/alpha_old) for the next sweep.  After a residual replacement
// (k1_mode = 1) the sweep restarts from the replaced residual: no pending
// update, e = 0, and beta = 0 for the next sweep (p and s are written as 0).
// Streams: r, s, w (ping-pong, read with a halo), p, e (in place), code.
// ===========================================================================
__device__ __forceinline__ void cgf_finish(Scalars &sc, double gamma, double delta, double rr)
{
    const bool restart = sc.k1_mode != 0;
    sc.k1_mode = 0;
    sc.e_reset = 0;
    sc.rsq = rr;
    sc.iter += 1;
    if (!(rr <= sc.div_thresh)) {  // non-finite or exploding: restart from the true residual
        sc.restarts += 1;
        sc.replace = 2;
        return;
    }
    double beta = 0.0, den = delta;
    if (!restart) {
        beta = gamma / sc.zr;
        den = delta - beta * gamma / sc.alpha;
    }
    const double alpha = gamma / den;
    if (!(fabs(alpha) < 1e300) || !(fabs(beta) < 1e300) || alpha == 0.0) {
        sc.restarts += 1;
        sc.replace = 2;
        return;
    }
    sc.beta = beta;
    sc.alpha = alpha;
    sc.zr = gamma;
    mixed_request(sc, rr, 2);
}

#ifndef FAST_TAU_HINT_CGF
#define FAST_TAU_HINT_CGF 0
#endif
struct OpCGF {
    using T = float;
    static constexpr bool FB = true;
    static constexpr bool clears_gate = true;
    static constexpr uint32_t wait_hint_ns = FAST_TAU_HINT_CGF;
    using SL = Streams<4, 4, 4, 4, 4, 1>;  // r, s, w, p, e, code
    static constexpr int NV = 3;
    using Shared = NoShared;
    struct Vals { float r, s, w, p, e; uint32_t code; };
    struct Own { uint32_t code; float rk, pk, sk, ek; };
    struct Out { float r, p, s, w, e; };
    const CUtensorMap *tmap[SL::N];
    Faces<T> F;
    float *rout, *sout, *wout, *pio, *eio;
    float a, bt;
    bool restart, ezero;
    Acc<float> g_, d_, rr_;

    __device__ static bool active(const Scalars &sc) { return sc.state == RUNNING; }
    __device__ static void load_shared(Shared &, const Job &, int) {}
    __device__ static void load2(const unsigned char *st, const Pt &p, Vals &a, Vals &b)
    {
        sv2<float, SL, 0>(st, p, a.r, b.r);
        sv2<float, SL, 1>(st, p, a.s, b.s);
        sv2<float, SL, 2>(st, p, a.w, b.w);
        sv2<float, SL, 3>(st, p, a.p, b.p);
        sv2<float, SL, 4>(st, p, a.e, b.e);
        load_code2<SL, 5>(st, p, a.code, b.code);
    }
    __device__ static void load1(const unsigned char *st, const Pt &p, Vals &a)
    {
        a.r = sv<float, SL, 0>(st, p);
        a.s = sv<float, SL, 1>(st, p);
        a.w = sv<float, SL, 2>(st, p);
        a.code = sv<uint8_t, SL, 5>(st, p);
    }
    __device__ void init(const Job &J, Shared &)
    {
        F = faces_of<T>(J);
        const Scalars &sc = *J.sc;
        const int par = (int)(sc.iter & 1);
        tmap[0] = &J.tm[TM_R + par];
        tmap[1] = &J.tm[TM_V + par];
        tmap[2] = &J.tm[par ? TM_R0 : TM_T];
        tmap[3] = &J.tm[TM_P];
        tmap[4] = &J.tm[TM_X];
        tmap[5] = &J.tm[TM_CODE];
        rout = (float *)J.r[par ^ 1];
        sout = (float *)J.v[par ^ 1];
        wout = (float *)(par ? J.t : J.r0);
        pio = (float *)J.p[0];
        eio = (float *)J.x;
        restart = sc.k1_mode != 0;
        ezero = sc.e_reset != 0;
        a = restart ? 0.f : (float)sc.alpha;
        bt = restart ? 0.f : (float)sc.beta;
    }
    __device__ float rk(const Vals &v) const { return restart ? v.r : v.r - a * (v.w + bt * v.s); }
    __device__ T field(const Geo &g, const Coef<T> &C, Shared &, const Vals &v, const Pos &ps) const
    {
        return rk(v) * inv_of<T, FB>(C, g, v.code, ps);
    }
    __device__ Own own(const Geo &g, const Coef<T> &C, Shared &, const Vals &v, const Pos &ps, T &f) const
    {
        const float inv = inv_of<T, FB>(C, g, v.code, ps);
        const float r = rk(v);
        f = r * inv;
        const float e0 = ezero ? 0.f : v.e;
        if (restart) return Own{v.code, r, 0.f, 0.f, e0};
        const float pk = v.r * inv + bt * v.p;  // p_{k-1} = u_{k-1} + beta p
        return Own{v.code, r, pk, v.w + bt * v.s, e0 + a * pk};
    }
    __device__ Out apply(const Geo &g, const Coef<T> &C, Shared &, const Own &o, const Pos &ps, T fc, T fxp, T fxm,
                         T fyp, T fym, T fzp, T fzm)
    {
        const T d = diag_of<T, FB>(C, g, o.code, ps);
        const T w = stencil7<T>(F, o.code, fc, fxp, fxm, fyp, fym, fzp, fzm, d);
        g_.add_prod(o.rk, fc);
        d_.add_prod(w, fc);
        rr_.add_prod(o.rk, o.rk);
        return Out{o.rk, o.pk, o.sk, w, o.ek};
    }
    __device__ void store(int64_t i, const Out &a_, const Out &b_, bool v0, bool v1)
    {
        store2<float>(rout, i, a_.r, b_.r, v0, v1);
        store2<float>(sout, i, a_.s, b_.s, v0, v1);
        store2<float>(wout, i, a_.w, b_.w, v0, v1);
        store2<float>(pio, i, a_.p, b_.p, v0, v1);
        store2<float>(eio, i, a_.e, b_.e, v0, v1);
    }
    __device__ void partials(T (&v_)[NV]) const { v_[0] = g_.hi(); v_[1] = d_.hi(); v_[2] = rr_.hi(); }
    __device__ static void finish(Scalars &sc, const double (&t)[NV]) { cgf_finish(sc, t[0], t[1], t[2]); }
};

}  // namespace ft
