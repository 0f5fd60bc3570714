// Serving context: continuous batching of tortuosity requests on one GPU.
//
// Requests (a volume, a direction, a solver) are queued on submit.  Each poll
// runs one scheduling step on the context's stream:
//   1. wait for the chunk launched by the previous step and read every
//      in-flight solve's scalars (one copy of the slot array);
//   2. retire the solves that left RUNNING: one tau launch over all of them,
//      results to the caller, their device memory back to the pool;
//   3. admit queued requests, oldest first, while a slot is free and their
//      device footprint fits the HBM budget: upload the mask, build the
//      stencil codes and the initial iterate (one launch each for all new
//      solves);
//   4. if the set of solves changed, rebuild each solver group's job table
//      and re-capture its chunk graph (`chunk` iterations of the group's
//      kernels over all of its solves);
//   5. launch one chunk per group and copy the slot array back behind it.
// Two chunks are kept in flight: a poll first queues the next chunk of the
// current solves, then reads the snapshot of the older one, so the GPU keeps
// iterating while the host retires and admits.  Chunks carry sequence
// numbers; a snapshot speaks only for solves admitted before its chunk.  All
// work is on one stream, so a slot or job table reused for a new solve is
// rewritten only after every queued chunk that names its previous owner; the
// host-side staging of those copies is rewritten only after the previous
// step's copies out of it have run.
// A request's arithmetic is exactly that of a solve of it alone: its kernels
// see only its own scalars and partial sums, whatever else shares the
// launches.  There is no counterpart in the reference (fast tau solves one
// volume per process run, fast/src/TauModule.h:64-114).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <vector>

#include "tau_engine.h"

namespace ft {
namespace {

using Clock = std::chrono::steady_clock;

#define SV(call)                                                                                 \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess)                                                                   \
            return ft_fail(e_ == cudaErrorMemoryAllocation ? FAST_NOMEM : FAST_CUDA_ERROR,       \
                           "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

struct Request {
    uint64_t ticket;
    std::vector<uint8_t> mask;
    int64_t nx, ny, nz;
    int dir, solver;
    double t_submit;
};

struct Active {
    Request req;
    int slot;
    char *arena;
    size_t bytes;
    Job job;          // descriptor (tile_base set per launch)
    double t_admit;
    uint64_t first_seq;  // the first chunk that advances this solve
};

struct Group {
    std::vector<int> members;       // indices into Ctx::active
    Job *d_jobs = nullptr;          // device job table (capacity kMax)
    cudaGraphExec_t exec = nullptr;
    int64_t nblocks = 0;
    uint32_t *d_gate = nullptr;     // the group's replacement gate word (MIXED)
};

struct Ctx {
    fast_ctx_config cfg;
    fast_tau_params P[2];  // by solver
    cudaStream_t st = nullptr;
    Clock::time_point t0;
    int kMax = 0;
    Scalars *d_slots = nullptr;
    uint32_t *d_cnt = nullptr;
    Scalars *h_snap[2] = {};        // pinned copies of the slot array, one per chunk in flight
    Scalars *h_init = nullptr;      // pinned staging of new solves' scalars
    Job *h_stage = nullptr;         // pinned staging of job tables (5 regions of kMax)
    Job *d_tmp[3] = {};             // device job tables for retire / code / init launches
    std::vector<int> free_slots;
    std::deque<Request> pending;
    std::vector<Active> active;
    Group groups[2];
    bool dirty = true;
    // Up to two chunks in flight: the GPU runs the next one while the host
    // retires and admits from the snapshot of the previous one.
    int inflight = 0, head = 0;
    cudaEvent_t ev[2] = {};
    uint64_t snap_seq[2] = {};
    // Recorded behind a step's copies out of the pinned staging (new solves'
    // scalars, job tables); the next step waits for it before rewriting the
    // staging, since the chunk it consumes may precede those copies.
    cudaEvent_t ev_copy = nullptr;
    bool copy_pending = false;
    uint64_t next_seq = 0;
    uint64_t next_ticket = 1;
    size_t bytes_inflight = 0;
    uint64_t completed = 0, admitted = 0, steps = 0;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

int steps_of(const Ctx &C, int solver, std::vector<Step> &steps)
{
    const bool mixed = C.cfg.precision == FAST_PREC_MIXED;
    if (solver == FAST_SOLVER_CG) {
        steps = mixed ? mixed_steps(FAST_SOLVER_CG, false) : std::vector<Step>{Step::CG1, Step::CG2};
    } else {
        steps = mixed ? mixed_steps(FAST_SOLVER_BICGSTAB, false)
                      : std::vector<Step>{Step::BI_RESTART, Step::BI1, Step::BI2, Step::BI3};
    }
    return FAST_OK;
}

void dispatch(const Ctx &C, Step s, const Launch &L, cudaStream_t st)
{
    if (C.cfg.precision == FAST_PREC_MIXED) dispatch_mixed(s, L, st);
    else if (C.cfg.precision == FAST_PREC_F64) launch_pure_f64(s, L, st);
    else launch_pure_f32(s, L, st);
}

// Copies `n` descriptors to a device job table with consecutive tile numbering.
int upload_jobs(Ctx &C, Job *stage, const std::vector<const Job *> &src, Job *d_dst, int64_t &nblocks)
{
    nblocks = 0;
    for (size_t k = 0; k < src.size(); k++) {
        stage[k] = *src[k];
        stage[k].tile_base = nblocks;
        nblocks += stage[k].ntiles;
    }
    if (nblocks > (int64_t)INT32_MAX) return ft_fail(FAST_BAD_ARG, "too many tiles in flight");
    if (!src.empty()) SV(cudaMemcpyAsync(d_dst, stage, sizeof(Job) * src.size(), cudaMemcpyHostToDevice, C.st));
    return FAST_OK;
}

// Retires the solves that the snapshot of chunk `seq` (buffer `snap`) shows
// finished; solves admitted after that chunk was launched are not in it.
int retire(Ctx &C, Scalars *snap, uint64_t seq, fast_ctx_completion *out, int32_t cap, int32_t &n_out)
{
    std::vector<int> done;
    for (int a = 0; a < (int)C.active.size(); a++)
        if (C.active[a].first_seq <= seq && snap[C.active[a].slot].state != RUNNING) done.push_back(a);
    if (done.empty()) return FAST_OK;
    // Results go out in the poll that retires them: only as many as fit.
    if ((int32_t)done.size() > cap - n_out) done.resize((size_t)std::max(0, cap - n_out));
    if (done.empty()) return FAST_OK;
    std::vector<const Job *> jobs;
    for (int a : done)
        if (snap[C.active[a].slot].state == CONVERGED) jobs.push_back(&C.active[a].job);
    if (!jobs.empty()) {
        int64_t nb = 0;
        int s = upload_jobs(C, C.h_stage, jobs, C.d_tmp[0], nb);
        if (s != FAST_OK) return s;
        const Launch L{C.d_tmp[0], (int32_t)jobs.size(), 0, nb, nullptr};
        const int prec = C.cfg.precision;
        launch_tau(prec == FAST_PREC_MIXED ? 3 : (prec == FAST_PREC_F32 ? 1 : 0), L, C.st);
        SV(cudaGetLastError());
    }
    // Every retiring solve's final scalars (flux sums included).
    for (int a : done)
        SV(cudaMemcpyAsync(snap + C.active[a].slot, C.d_slots + C.active[a].slot, sizeof(Scalars),
                           cudaMemcpyDeviceToHost, C.st));
    SV(cudaStreamSynchronize(C.st));
    const double t = C.now();
    for (int a : done) {
        Active &A = C.active[a];
        const Scalars &S = snap[A.slot];
        fast_ctx_completion &R = out[n_out++];
        memset(&R, 0, sizeof(R));
        R.ticket = A.req.ticket;
        R.dir = A.req.dir;
        R.solver = A.req.solver;
        R.t_submit = A.req.t_submit;
        R.t_admit = A.t_admit;
        R.t_done = t;
        fast_tau_result &X = R.result;
        X.status = status_of(S.state);
        X.iterations = S.iter;
        const bool mixed = C.cfg.precision == FAST_PREC_MIXED;
        X.outer_steps = mixed ? (uint32_t)S.outer_steps : 0;
        if (mixed) X.rel_residual = S.b64_sq > 0 ? std::sqrt(S.r64_sq / S.b64_sq) : 0.0;
        else X.rel_residual = S.rhs_sq > 0 ? std::sqrt(S.rsq / S.rhs_sq) : 0.0;
        const int64_t N = A.req.nx * A.req.ny * A.req.nz;
        const int k = A.req.dir >> 1;
        const int64_t dimk = k == 0 ? A.req.nx : (k == 1 ? A.req.ny : A.req.nz);
        const int64_t nplane = N / dimk;
        if (C.cfg.precision == FAST_PREC_F32) {
            const float phi = (float)S.pores / (float)N;
            X.porosity = phi;
            const float dc = ((float)S.flux_sum / (float)nplane) / (float)dimk;
            X.tau = X.status == FAST_OK ? (double)(phi / (dc * (float)dimk)) : 0.0;
        } else {
            const double phi = (double)S.pores / (double)N;
            X.porosity = phi;
            const double dc = (S.flux_sum / (double)nplane) / (double)dimk;
            X.tau = X.status == FAST_OK ? phi / (dc * (double)dimk) : 0.0;
        }
        cudaFreeAsync(A.arena, C.st);
        C.bytes_inflight -= A.bytes;
        C.free_slots.push_back(A.slot);
        C.completed++;
    }
    // Drop the retired entries (descending index order keeps the rest valid).
    std::sort(done.begin(), done.end());
    for (int i = (int)done.size() - 1; i >= 0; i--) C.active.erase(C.active.begin() + done[i]);
    C.dirty = true;
    return FAST_OK;
}

int admit(Ctx &C)
{
    std::vector<int> fresh;
    while (!C.pending.empty() && !C.free_slots.empty()) {
        Request &R = C.pending.front();
        const fast_tau_params &P = C.P[R.solver];
        const size_t bytes = align_up((size_t)(R.nx * R.ny * R.nz), 256) + code_bytes(R.nx, R.ny, R.nz) +
                             job_bytes(R.nx, R.ny, R.nz, P.precision, P.solver) + 4096;
        // Admit by footprint; a request larger than the whole budget still
        // runs, alone.
        if (C.bytes_inflight + bytes > C.cfg.hbm_budget && !C.active.empty()) break;
        Active A;
        A.req = std::move(R);
        C.pending.pop_front();
        A.slot = C.free_slots.back();
        A.bytes = bytes;
        A.arena = nullptr;
        cudaError_t e = cudaMallocAsync((void **)&A.arena, bytes, C.st);
        if (e != cudaSuccess) return ft_fail(FAST_NOMEM, "admission: %s", cudaGetErrorString(e));
        C.free_slots.pop_back();
        Arena M;
        M.base = A.arena;
        M.cap = bytes;
        const size_t n = (size_t)(A.req.nx * A.req.ny * A.req.nz);
        uint8_t *d_mask = (uint8_t *)M.take(n);
        uint8_t *d_code = (uint8_t *)M.take(code_bytes(A.req.nx, A.req.ny, A.req.nz));
        SV(cudaMemcpyAsync(d_mask, A.req.mask.data(), n, cudaMemcpyHostToDevice, C.st));
        Scalars &S0 = C.h_init[fresh.size()];
        int s = build_job(A.job, S0, d_mask, A.req.nx, A.req.ny, A.req.nz, A.req.dir, d_code, C.d_slots + A.slot,
                          C.d_cnt + A.slot, M, P);
        if (s != FAST_OK) {
            cudaFreeAsync(A.arena, C.st);
            C.free_slots.push_back(A.slot);
            return s;
        }
        SV(cudaMemcpyAsync(C.d_slots + A.slot, &S0, sizeof(Scalars), cudaMemcpyHostToDevice, C.st));
        A.req.mask.clear();
        A.req.mask.shrink_to_fit();
        A.t_admit = C.now();
        A.first_seq = C.next_seq;
        C.bytes_inflight += bytes;
        C.admitted++;
        C.active.push_back(std::move(A));
        fresh.push_back((int)C.active.size() - 1);
    }
    if (fresh.empty()) return FAST_OK;
    // Stencil codes + pore counts, then the initial iterate, of the new solves.
    std::vector<const Job *> jobs;
    for (int a : fresh) jobs.push_back(&C.active[a].job);
    int64_t nb = 0;
    int s = upload_jobs(C, C.h_stage + C.kMax, jobs, C.d_tmp[1], nb);
    if (s != FAST_OK) return s;
    launch_code(Launch{C.d_tmp[1], (int32_t)jobs.size(), 0, nb, nullptr}, C.st);
    if (C.cfg.precision == FAST_PREC_MIXED) {
        launch_init64(Launch{C.d_tmp[1], (int32_t)jobs.size(), 0, nb, nullptr}, C.st);
    } else {
        for (int g = 0; g < 2; g++) {
            std::vector<const Job *> gj;
            for (int a : fresh)
                if (C.active[a].req.solver == g) gj.push_back(&C.active[a].job);
            if (gj.empty()) continue;
            int64_t gb = 0;
            s = upload_jobs(C, C.h_stage + (2 + g) * C.kMax, gj, C.d_tmp[2 - g], gb);
            if (s != FAST_OK) return s;
            dispatch(C, g == FAST_SOLVER_CG ? Step::INIT_CG : Step::INIT_BI, Launch{C.d_tmp[2 - g], (int32_t)gj.size(), 0, gb, nullptr},
                     C.st);
        }
    }
    SV(cudaGetLastError());
    C.dirty = true;
    return FAST_OK;
}

int rebuild(Ctx &C)
{
    // The pinned staging regions of this step may still feed copies queued
    // above; the group tables use their own regions (4 and 5 of the stage).
    for (int g = 0; g < 2; g++) {
        Group &G = C.groups[g];
        G.members.clear();
        std::vector<const Job *> jobs;
        for (int a = 0; a < (int)C.active.size(); a++)
            if (C.active[a].req.solver == g) {
                G.members.push_back(a);
                jobs.push_back(&C.active[a].job);
            }
        if (G.exec) {
            cudaGraphExecDestroy(G.exec);
            G.exec = nullptr;
        }
        if (jobs.empty()) continue;
        int s = upload_jobs(C, C.h_stage + (4 + g) * C.kMax, jobs, G.d_jobs, G.nblocks);
        if (s != FAST_OK) return s;
        std::vector<Step> steps;
        steps_of(C, g, steps);
        const bool mixed = C.cfg.precision == FAST_PREC_MIXED;
        // the replacement gate opens for the group's new solves (they start
        // with a pending replacement); an extra scan for the others is cheap
        if (mixed) SV(cudaMemsetAsync(G.d_gate, 1, 1, C.st));
        const Launch L{G.d_jobs, (int32_t)jobs.size(), 0, G.nblocks, mixed ? G.d_gate : nullptr};
        s = capture_chunk(C.st, L, steps, C.cfg.chunk,
                          C.cfg.precision == FAST_PREC_MIXED ? dispatch_mixed
                          : C.cfg.precision == FAST_PREC_F64 ? launch_pure_f64 : launch_pure_f32,
                          &G.exec);
        if (s != FAST_OK) return s;
    }
    C.dirty = false;
    return FAST_OK;
}

int launch_chunk(Ctx &C)
{
    const int b = (C.head + C.inflight) & 1;
    for (int g = 0; g < 2; g++)
        if (C.groups[g].exec) SV(cudaGraphLaunch(C.groups[g].exec, C.st));
    int hi = 0;
    for (const Active &A : C.active) hi = std::max(hi, A.slot + 1);
    SV(cudaMemcpyAsync(C.h_snap[b], C.d_slots, sizeof(Scalars) * hi, cudaMemcpyDeviceToHost, C.st));
    SV(cudaEventRecord(C.ev[b], C.st));
    C.snap_seq[b] = C.next_seq++;
    C.inflight++;
    C.steps++;
    return FAST_OK;
}

int step(Ctx &C, fast_ctx_completion *out, int32_t cap, int32_t *n_out)
{
    *n_out = 0;
    // Keep the GPU busy: queue the next chunk of the current set of solves
    // before waiting for the previous one.
    if (C.inflight == 1 && !C.dirty && !C.active.empty()) {
        int s = launch_chunk(C);
        if (s != FAST_OK) return s;
    }
    if (C.copy_pending) {
        SV(cudaEventSynchronize(C.ev_copy));
        C.copy_pending = false;
    }
    if (C.inflight > 0) {
        const int b = C.head;
        SV(cudaEventSynchronize(C.ev[b]));
        C.head ^= 1;
        C.inflight--;
        int s = retire(C, C.h_snap[b], C.snap_seq[b], out, cap, *n_out);
        if (s != FAST_OK) return s;
    }
    int s = admit(C);
    if (s != FAST_OK) return s;
    if (C.active.empty()) return FAST_OK;
    if (C.dirty) {
        s = rebuild(C);
        if (s != FAST_OK) return s;
    }
    SV(cudaEventRecord(C.ev_copy, C.st));
    C.copy_pending = true;
    while (C.inflight < 2) {
        s = launch_chunk(C);
        if (s != FAST_OK) return s;
    }
    return FAST_OK;
}

void destroy(Ctx *C)
{
    if (!C) return;
    if (C->st) cudaStreamSynchronize(C->st);
    for (Active &A : C->active) cudaFreeAsync(A.arena, C->st);
    for (Group &G : C->groups) {
        if (G.exec) cudaGraphExecDestroy(G.exec);
        if (G.d_jobs) cudaFreeAsync(G.d_jobs, C->st);
        if (G.d_gate) cudaFreeAsync(G.d_gate, C->st);
    }
    for (Job *d : C->d_tmp)
        if (d) cudaFreeAsync(d, C->st);
    if (C->d_slots) cudaFreeAsync(C->d_slots, C->st);
    if (C->d_cnt) cudaFreeAsync(C->d_cnt, C->st);
    if (C->st) cudaStreamSynchronize(C->st);
    for (Scalars *h : C->h_snap)
        if (h) cudaFreeHost(h);
    if (C->h_init) cudaFreeHost(C->h_init);
    if (C->h_stage) cudaFreeHost(C->h_stage);
    for (cudaEvent_t e : C->ev)
        if (e) cudaEventDestroy(e);
    if (C->ev_copy) cudaEventDestroy(C->ev_copy);
    if (C->st) cudaStreamDestroy(C->st);
    delete C;
}

int create(const fast_ctx_config &cfg, Ctx **out)
{
    Engine *E = nullptr;
    int s = get_engine(&E);  // kernel attributes of this device
    if (s != FAST_OK) return s;
    Ctx *C = new Ctx();
    C->cfg = cfg;
    C->t0 = Clock::now();
    C->kMax = cfg.max_inflight;
    for (int g = 0; g < 2; g++) {
        fast_tau_params_init(&C->P[g]);
        C->P[g].solver = g;
        C->P[g].precision = cfg.precision;
        C->P[g].tolerance = cfg.tolerance;
        C->P[g].max_iter = cfg.max_iter;
        C->P[g].d0 = cfg.d0;
        C->P[g].d1 = cfg.d1;
        C->P[g].face_mean = cfg.face_mean;
        s = check_params(&C->P[g]);
        if (s != FAST_OK) {
            delete C;
            return s;
        }
    }
    const int K = C->kMax;
    auto fin = [&](int st) {
        destroy(C);
        return st;
    };
    if (cudaStreamCreateWithFlags(&C->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&C->ev[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&C->ev[1], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&C->ev_copy, cudaEventDisableTiming) != cudaSuccess)
        return fin(ft_fail(FAST_CUDA_ERROR, "stream/event creation failed"));
    if (cudaMallocAsync((void **)&C->d_slots, sizeof(Scalars) * K, C->st) != cudaSuccess ||
        cudaMallocAsync((void **)&C->d_cnt, sizeof(uint32_t) * K, C->st) != cudaSuccess ||
        cudaMallocAsync((void **)&C->groups[0].d_jobs, sizeof(Job) * K, C->st) != cudaSuccess ||
        cudaMallocAsync((void **)&C->groups[1].d_jobs, sizeof(Job) * K, C->st) != cudaSuccess ||
        cudaMallocAsync((void **)&C->d_tmp[0], sizeof(Job) * K, C->st) != cudaSuccess ||
        cudaMallocAsync((void **)&C->d_tmp[1], sizeof(Job) * K, C->st) != cudaSuccess ||
        cudaMallocAsync((void **)&C->d_tmp[2], sizeof(Job) * K, C->st) != cudaSuccess ||
        cudaMallocAsync((void **)&C->groups[0].d_gate, sizeof(uint32_t), C->st) != cudaSuccess ||
        cudaMallocAsync((void **)&C->groups[1].d_gate, sizeof(uint32_t), C->st) != cudaSuccess)
        return fin(ft_fail(FAST_NOMEM, "context tables"));
    if (cudaMemsetAsync(C->d_cnt, 0, sizeof(uint32_t) * K, C->st) != cudaSuccess ||
        cudaMemsetAsync(C->groups[0].d_gate, 0, sizeof(uint32_t), C->st) != cudaSuccess ||
        cudaMemsetAsync(C->groups[1].d_gate, 0, sizeof(uint32_t), C->st) != cudaSuccess ||
        cudaMallocHost(&C->h_snap[0], sizeof(Scalars) * K) != cudaSuccess ||
        cudaMallocHost(&C->h_snap[1], sizeof(Scalars) * K) != cudaSuccess ||
        cudaMallocHost(&C->h_init, sizeof(Scalars) * K) != cudaSuccess ||
        cudaMallocHost(&C->h_stage, sizeof(Job) * 6 * K) != cudaSuccess)
        return fin(ft_fail(FAST_NOMEM, "context staging"));
    if (cudaStreamSynchronize(C->st) != cudaSuccess) return fin(ft_fail(FAST_CUDA_ERROR, "context setup"));
    for (int k = K - 1; k >= 0; k--) C->free_slots.push_back(k);
    *out = C;
    return FAST_OK;
}

}  // namespace
}  // namespace ft

using namespace ft;

extern "C" {

FAST_API void fast_ctx_config_init(fast_ctx_config *cfg)
{
    if (!cfg) return;
    memset(cfg, 0, sizeof(*cfg));
    cfg->precision = FAST_PREC_MIXED;
    cfg->face_mean = FAST_FACE_ARITHMETIC;
    cfg->tolerance = 1e-6;
    cfg->max_iter = 10000;
    cfg->d0 = (double)1.0f;
    cfg->d1 = (double)0.001f;
    cfg->chunk = 16;
    cfg->max_inflight = 256;
    cfg->hbm_budget = 0;
}

FAST_API int fast_ctx_create(const fast_ctx_config *cfg, void **ctx)
{
    ft_clear_error();
    if (!cfg || !ctx) return ft_fail(FAST_BAD_ARG, "null argument");
    fast_ctx_config c = *cfg;
    if (c.chunk < 1 || c.chunk > 1024) return ft_fail(FAST_BAD_ARG, "chunk must be 1..1024");
    if (c.max_inflight < 1 || c.max_inflight > 1024) return ft_fail(FAST_BAD_ARG, "max_inflight must be 1..1024");
    if (c.hbm_budget == 0) {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return ft_fail(FAST_CUDA_ERROR, "cudaMemGetInfo failed");
        c.hbm_budget = (uint64_t)(fr * 0.8);
    }
    Ctx *C = nullptr;
    const int s = create(c, &C);
    if (s != FAST_OK) return s;
    *ctx = C;
    return FAST_OK;
}

FAST_API int fast_ctx_submit(void *ctx, const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, int32_t dir,
                             int32_t solver, uint64_t *ticket)
{
    ft_clear_error();
    Ctx *C = (Ctx *)ctx;
    if (!C) return ft_fail(FAST_BAD_ARG, "context is NULL");
    int s = check_volume(mask, nx, ny, nz);
    if (s != FAST_OK) return s;
    if (dir < 0 || dir > 5) return ft_fail(FAST_BAD_ARG, "bad direction %d", dir);
    if (solver != FAST_SOLVER_BICGSTAB && solver != FAST_SOLVER_CG) return ft_fail(FAST_BAD_ARG, "Unknown solver %d", solver);
    const Geometry G = make_geometry(nx, ny, nz);
    if (G.ntiles > (int64_t)INT32_MAX / 2) return ft_fail(FAST_BAD_ARG, "volume too large");
    Request R;
    R.ticket = C->next_ticket++;
    R.mask.assign(mask, mask + (size_t)(nx * ny * nz));
    R.nx = nx; R.ny = ny; R.nz = nz;
    R.dir = dir;
    R.solver = solver;
    R.t_submit = C->now();
    C->pending.push_back(std::move(R));
    if (ticket) *ticket = C->pending.back().ticket;
    return FAST_OK;
}

FAST_API int fast_ctx_poll(void *ctx, fast_ctx_completion *out, int32_t cap, int32_t *n_done)
{
    ft_clear_error();
    Ctx *C = (Ctx *)ctx;
    if (!C || !out || !n_done || cap < 1) return ft_fail(FAST_BAD_ARG, "bad poll arguments");
    return step(*C, out, cap, n_done);
}

FAST_API int fast_ctx_query(void *ctx, fast_ctx_stats *out)
{
    Ctx *C = (Ctx *)ctx;
    if (!C || !out) return ft_fail(FAST_BAD_ARG, "null argument");
    memset(out, 0, sizeof(*out));
    out->pending = C->pending.size();
    out->inflight = C->active.size();
    out->completed = C->completed;
    out->admitted = C->admitted;
    out->steps = C->steps;
    out->bytes_inflight = C->bytes_inflight;
    out->hbm_budget = C->cfg.hbm_budget;
    out->now = C->now();
    return FAST_OK;
}

FAST_API int fast_ctx_destroy(void *ctx)
{
    destroy((Ctx *)ctx);
    return FAST_OK;
}

}  // extern "C"
