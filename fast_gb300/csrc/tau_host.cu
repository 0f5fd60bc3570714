// Host orchestration and the C ABI of libfasttau.so.
//
// Replaces the reference's getTortuosity<T> driver
// (fastlib/src/volume/VolumeMeasures.cpp:42-285): system assembly
// (GenerateDiffusionLinearSystemDevice, fastlib/src/solver/Diffusion.cpp:
// 177-231) becomes the one-byte stencil-code build; the solver dispatch
// (CG.cpp:40-109, BICGSTAB.cpp:41-103) becomes fused kernels replayed from a
// captured CUDA graph; the host tau loop (VolumeMeasures.cpp:188-275) becomes
// a device FP64 reduction.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <mutex>
#include <string>
#include <vector>

#include "fasttau.h"
#include "tau_engine.h"

using namespace ft;

// ---------------------------------------------------------------------------
// Errors
// ---------------------------------------------------------------------------
static thread_local std::string g_last_error;

static int fail(int status, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

int ft_fail(int status, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

void ft_clear_error() { g_last_error.clear(); }

void ft_retain_pool_memory(int device)
{
    static std::once_flag once[64];
    if (device < 0 || device >= 64) return;
    std::call_once(once[device], [device] {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t thr = std::numeric_limits<uint64_t>::max();
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
    });
}

#define CU(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) {                                                                   \
            return fail(e_ == cudaErrorMemoryAllocation ? FAST_NOMEM : FAST_CUDA_ERROR,            \
                        "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
        }                                                                                          \
    } while (0)

// ---------------------------------------------------------------------------
// Per-thread engine: one non-blocking stream per device, pinned staging.
// ---------------------------------------------------------------------------
namespace ft {

int Engine::init(int dev)
{
    device = dev;
    CU(cudaSetDevice(dev));
    CU(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    CU(cudaMallocHost(&h_sc, sizeof(Scalars) * 2 * kMaxJobs));
    CU(cudaMallocHost(&h_jobs, sizeof(Job) * 2 * kMaxJobs));  // jobs + one code job per volume
    cudaError_t ce = configure_f64();
    if (ce == cudaSuccess) ce = configure_f32();
    if (ce == cudaSuccess) ce = configure_misc();
    if (ce != cudaSuccess) return fail(FAST_CUDA_ERROR, "kernel configuration: %s", cudaGetErrorString(ce));
    ft_retain_pool_memory(dev);
    return FAST_OK;
}

thread_local Engine *t_engines[64] = {};

int get_engine(Engine **out)
{
    int dev = 0;
    CU(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(FAST_CUDA_ERROR, "device ordinal %d out of range", dev);
    if (!t_engines[dev]) {
        Engine *e = new Engine();
        int st = e->init(dev);
        if (st != FAST_OK) {
            delete e;
            return st;
        }
        t_engines[dev] = e;
    }
    *out = t_engines[dev];
    return FAST_OK;
}

int env_int(const char *name, int dflt)
{
    const char *v = getenv(name);
    return v ? atoi(v) : dflt;
}

double env_double(const char *name, double dflt)
{
    const char *v = getenv(name);
    return v ? atof(v) : dflt;
}

// Launch bookkeeping and the optional per-launch CUDA-event profile.
struct Prof {
    fast_tau_stats st;
    bool on = false;
    cudaEvent_t a = nullptr, b = nullptr;
    void reset(bool enable)
    {
        memset(&st, 0, sizeof(st));
        on = enable;
        st.profiled = enable ? 1 : 0;
        if (on && !a) {
            cudaEventCreate(&a);
            cudaEventCreate(&b);
        }
    }
};
thread_local Prof t_prof;

int kind_of(Step s)
{
    switch (s) {
    case Step::INIT_CG:
    case Step::INIT_BI: return FAST_K_INIT;
    case Step::CG1: return FAST_K_CG1;
    case Step::CG2: return FAST_K_CG2;
    case Step::BI_RESTART: return FAST_K_BI_RESTART;
    case Step::BI1: return FAST_K_BI1;
    case Step::BI2: return FAST_K_BI2;
    case Step::BI3: return FAST_K_BI3;
    case Step::REPLACE_CG:
    case Step::REPLACE_BI:
    case Step::REPLACE_CG_FF:
    case Step::REPLACE_BI_FF: return FAST_K_REPLACE;
    case Step::BI_K1: return FAST_K_BI1;
    case Step::BI_K2: return FAST_K_BI2;
    case Step::CG_F: return FAST_K_CGF;
    }
    return FAST_K_COUNT - 1;
}

// Runs one kernel launch, counting it and, when profiling, timing it with a
// CUDA event pair on the launching stream.
template <class F>
void launch_counted(int kind, cudaStream_t st, F &&f)
{
    Prof &P = t_prof;
    if (!P.on) {
        f();
    } else {
        cudaEventRecord(P.a, st);
        f();
        cudaEventRecord(P.b, st);
        cudaEventSynchronize(P.b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, P.a, P.b);
        P.st.kernel_ms[kind] += ms;
    }
    P.st.kernel_launches[kind] += 1;
    P.st.launches += 1;
}

// Coefficient tables of one job, in h = 1 units (see tau_device.cuh).
void fill_tables(Job &J, double d0, double d1, int face_mean)
{
    // Domain values as T(params.d0/d1) (LinearSystemDevice.cu:8-20).
    const double Dd[2] = {d0, d1};
    const float Df[2] = {(float)d0, (float)d1};
    for (int s = 0; s < 2; s++) {
        J.dcell[s] = Dd[s];
        for (int n = 0; n < 2; n++) {
            if (face_mean == FAST_FACE_HARMONIC) {
                J.dface[s][n] = 2.0 * Dd[n] * Dd[s] / (Dd[n] + Dd[s]);
                J.fface[s][n] = 2.0f * Df[n] * Df[s] / (Df[n] + Df[s]);
            } else {
                // (D(neighbour) + D(here)) * 0.5 (Diffusion.cu:47-53)
                J.dface[s][n] = (Dd[n] + Dd[s]) * 0.5;
                J.fface[s][n] = (Df[n] + Df[s]) * 0.5f;
            }
        }
    }
    for (int code = 0; code < 128; code++) {
        const int self = (code >> SELF_BIT) & 1;
        double dd = 0.0;
        float df = 0.f;
        for (int f = 0; f < 6; f++) {  // subtraction order of Diffusion.cuh:85-105
            const int nb = (code >> f) & 1;
            dd -= J.dface[self][nb];
            df -= J.fface[self][nb];
        }
        J.ddiag_int[code] = dd;
        J.dinv_int[code] = 1.0 / dd;
        // FP32 rows by boundary count bc = (missing secondary-axis
        // neighbours) - (missing primary-axis neighbours): a missing
        // neighbour's clamped code bit contributed -D_self above; a zero-flux
        // face contributes 0 and a Dirichlet face -2 D_self.
        for (int bc = -2; bc <= 4; bc++) {
            const float d = df + Df[self] * (float)bc;
            J.fdiag_b[bc + 2][code] = d;
            J.finv_b[bc + 2][code] = 1.0f / d;
        }
    }
    // Float-float splits (hi = nearest float, lo = nearest float of the rest).
    auto split = [](double v, float &hi, float &lo) {
        hi = (float)v;
        lo = (float)(v - (double)hi);
    };
    for (int s = 0; s < 2; s++) {
        split(2.0 * Dd[s], J.xcell2[s][0], J.xcell2[s][1]);
        for (int n = 0; n < 2; n++) split(J.dface[s][n], J.xface[s][n][0], J.xface[s][n][1]);
    }
    for (int code = 0; code < 128; code++) {
        const int self = (code >> SELF_BIT) & 1;
        for (int bc = -2; bc <= 4; bc++)
            split(J.ddiag_int[code] + Dd[self] * (double)bc, J.xdiag_hi[bc + 2][code], J.xdiag_lo[bc + 2][code]);
    }
    J.c_tau[0] = (float)d0;
    J.c_tau[1] = (float)d1;
}

Geometry make_geometry(int64_t nx, int64_t ny, int64_t nz, int zc_req)
{
    Geometry g;
    g.nx = nx; g.ny = ny; g.nz = nz;
    g.N = nx * ny * nz;
    g.tx = (int)((nx + TX - 1) / TX);
    g.ty = (int)((ny + TY - 1) / TY);
    int zc = zc_req > 0 ? zc_req : env_int("FAST_TAU_ZC", kSlabDepth);
    if (zc < 1) zc = 1;
    if (zc > nz) zc = (int)nz;
    g.zc = zc;
    g.tz = (int)((nz + zc - 1) / zc);
    g.ntiles = (int64_t)g.tx * g.ty * g.tz;
    return g;
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

int64_t row_pitch(int64_t nx) { return (nx + 15) / 16 * 16; }

// cuTensorMapEncodeTiled through the runtime's driver entry point (no -lcuda).
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::mutex g_encode_mu;

int tensor_map(CUtensorMap *tm, const void *base, int es, int64_t nx, int64_t ny, int64_t nz, int64_t pitch,
               bool interior = false)
{
    {
        std::lock_guard<std::mutex> lk(g_encode_mu);
        if (!g_encode) {
            cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
            void *fn = nullptr;
            cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
            if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
                return fail(FAST_CUDA_ERROR, "cuTensorMapEncodeTiled unavailable");
            g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
        }
    }
    const CUtensorMapDataType dt = es == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8
                                 : (es == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64);
    const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
    const cuuint64_t strides[2] = {(cuuint64_t)(pitch * es), (cuuint64_t)(pitch * ny * es)};
    // Box: the TX x TY tile plus a one-voxel halo, widened in x so that its
    // start (x0 - 16/es) and width are multiples of 16 bytes; or (interior)
    // the tile alone, for streams read only at a block's own points.
    const cuuint32_t box[3] = {(cuuint32_t)(interior ? TX : TX + 2 * (16 / es)), (cuuint32_t)(interior ? TY : HY), 1u};
    const cuuint32_t estr[3] = {1u, 1u, 1u};
    CUresult r = g_encode(tm, dt, 3, const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(FAST_CUDA_ERROR, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return FAST_OK;
}

// Captures `chunk` iterations of `steps` on `st` into an executable graph.
int capture_chunk(cudaStream_t st, const Launch &L, const std::vector<Step> &steps, int chunk,
                  void (*launch)(Step, const Launch &, cudaStream_t), cudaGraphExec_t *exec)
{
    cudaGraph_t graph = nullptr;
    CU(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int c = 0; c < chunk; c++)
        for (Step s : steps) launch(s, L, st);
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (e != cudaSuccess) return fail(FAST_CUDA_ERROR, "graph capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(FAST_CUDA_ERROR, "graph instantiate failed: %s", cudaGetErrorString(e));
    return FAST_OK;
}

// Replays `chunk` iterations from a captured graph until every job has left
// RUNNING; polls the device scalars one chunk behind so the queue never
// drains while the host waits.
int iterate(Engine &E, const Launch &L, int njobs, Scalars *d_sc, const std::vector<Step> &steps,
            void (*launch)(Step, const Launch &, cudaStream_t), uint64_t max_iter)
{
    cudaStream_t st = E.stream;
    const int chunk = std::max(1, env_int("FAST_TAU_CHUNK", 16));
    const int trace = env_int("FAST_TAU_TRACE", 0);
    if (trace >= 2) {
        // Trace: direct launches, scalars of job 0 printed after each kernel
        // (level 2) or after each iteration (level 3).
        for (uint64_t it = 0; it < max_iter + 2; it++) {
            bool running = false;
            for (size_t k = 0; k < steps.size(); k++) {
                const Step s = steps[k];
                launch(s, L, st);
                if (trace >= 3 && k + 1 < steps.size()) continue;
                CU(cudaMemcpyAsync(E.h_sc, d_sc, sizeof(Scalars) * njobs, cudaMemcpyDeviceToHost, st));
                CU(cudaStreamSynchronize(st));
                const Scalars &S = E.h_sc[0];
                fprintf(stderr,
                        "trace step %d iter %llu state %d rsq %.6e zr %.6e alpha %.6e beta %.6e rho %.6e omega %.6e "
                        "dots %.6e %.6e %.6e r0sq %.6e rsqmax %.6e r64sq %.6e b64sq %.6e repl %d nrepl %d restarts %llu\n",
                        (int)s, (unsigned long long)S.iter, S.state, S.rsq, S.zr, S.alpha, S.beta, S.rho, S.omega,
                        S.dbg[0], S.dbg[1], S.dbg[2], S.r0_sq, S.rsq_max, S.r64_sq, S.b64_sq, S.replace,
                        S.outer_steps, (unsigned long long)S.restarts);
            }
            for (int j = 0; j < njobs; j++) running |= (E.h_sc[j].state == RUNNING);
            if (!running) break;
        }
        return FAST_OK;
    }
    if (t_prof.on) {
        // Profiling: direct launches, each timed; the scalars are read after
        // every chunk.
        const uint64_t max_chunks = max_iter / (uint64_t)chunk + 4;
        for (uint64_t k = 0; k < max_chunks; k++) {
            for (int c = 0; c < chunk; c++)
                for (Step s : steps) launch_counted(kind_of(s), st, [&] { launch(s, L, st); });
            CU(cudaMemcpyAsync(E.h_sc, d_sc, sizeof(Scalars) * njobs, cudaMemcpyDeviceToHost, st));
            CU(cudaStreamSynchronize(st));
            bool running = false;
            for (int j = 0; j < njobs; j++) running |= (E.h_sc[j].state == RUNNING);
            if (!running) break;
        }
        return FAST_OK;
    }
    cudaGraphExec_t exec = nullptr;
    int cs = capture_chunk(st, L, steps, chunk, launch, &exec);
    if (cs != FAST_OK) return cs;
    cudaError_t cerr = cudaSuccess;

    cudaEvent_t ev[2];
    cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
    const uint64_t max_chunks = max_iter / (uint64_t)chunk + 4;
    int status = FAST_OK;
    uint64_t k = 0;
    for (; k < max_chunks; k++) {
        cerr = cudaGraphLaunch(exec, st);
        if (cerr != cudaSuccess) { status = fail(FAST_CUDA_ERROR, "graph launch: %s", cudaGetErrorString(cerr)); break; }
        t_prof.st.graph_replays += 1;
        t_prof.st.launches += (uint64_t)chunk * steps.size();
        for (Step s : steps) t_prof.st.kernel_launches[kind_of(s)] += (uint64_t)chunk;
        Scalars *hb = E.h_sc + (k & 1) * Engine::kMaxJobs;
        cudaMemcpyAsync(hb, d_sc, sizeof(Scalars) * njobs, cudaMemcpyDeviceToHost, st);
        cudaEventRecord(ev[k & 1], st);
        if (k == 0) continue;
        cerr = cudaEventSynchronize(ev[(k - 1) & 1]);
        if (cerr != cudaSuccess) { status = fail(FAST_CUDA_ERROR, "solver step: %s", cudaGetErrorString(cerr)); break; }
        const Scalars *prev = E.h_sc + ((k - 1) & 1) * Engine::kMaxJobs;
        bool running = false;
        for (int j = 0; j < njobs; j++) running |= (prev[j].state == RUNNING);
        if (!running) break;
    }
    cerr = cudaStreamSynchronize(st);
    if (cerr != cudaSuccess && status == FAST_OK) status = fail(FAST_CUDA_ERROR, "solver: %s", cudaGetErrorString(cerr));
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    cudaGraphExecDestroy(exec);
    return status;
}

void dispatch_f64(Step s, const Launch &L, cudaStream_t st) { launch_pure_f64(s, L, st); }
void dispatch_f32(Step s, const Launch &L, cudaStream_t st) { launch_pure_f32(s, L, st); }
std::vector<Step> mixed_steps(int solver, bool ff)
{
    if (solver == FAST_SOLVER_CG) {
        const Step rep = ff ? Step::REPLACE_CG_FF : Step::REPLACE_CG;
        return cg_fused_enabled() ? std::vector<Step>{rep, Step::CG_F} : std::vector<Step>{rep, Step::CG1, Step::CG2};
    }
    return {ff ? Step::REPLACE_BI_FF : Step::REPLACE_BI, Step::BI_K1, Step::BI_K2};
}

void dispatch_mixed(Step s, const Launch &L, cudaStream_t st)
{
    switch (s) {
    case Step::REPLACE_CG: launch_replace(false, false, L, st); break;
    case Step::REPLACE_BI: launch_replace(true, false, L, st); break;
    case Step::REPLACE_CG_FF: launch_replace(false, true, L, st); break;
    case Step::REPLACE_BI_FF: launch_replace(true, true, L, st); break;
    default: launch_mixed_inner(s, L, st);
    }
}

int status_of(int state)
{
    switch (state) {
    case CONVERGED: return FAST_OK;
    case DIVERGED: return FAST_DIVERGED;
    case FAULT: return FAST_TIMEOUT;
    case RUNNING: return FAST_TIMEOUT;
    default: return FAST_NO_CONVERGENCE;  // MAXITER, ZERO_RHS (CG.cu:41-44 returns false)
    }
}

// A volume of a solve (device-resident mask) and a right-hand side of it.
struct VolSpec {
    const uint8_t *d_mask;
    int64_t nx, ny, nz;
};
struct JobSpec {
    int vol;
    int dir;
};

size_t code_bytes(int64_t nx, int64_t ny, int64_t nz) { return align_up((size_t)(row_pitch(nx) * ny * nz), 256); }

// Slab depth by size class.  A launch's size class is floor(log2(W)), W its
// tile-planes: the sum over its right-hand sides of x tiles * y tiles * nz,
// i.e. its block count at one plane per block.  Each (precision, solver,
// class) has a depth: from the built-in table (slab_table.inc, written by
// the autotuner, fast_gb300/autotune.py, from timings of a fixed number of
// iterations at every candidate depth on a GB300), or from a table installed
// at run time with fast_tau_set_slab_table.  A class without an entry uses
// the full depth, halved (down to 2 planes) while the launch would give the
// GPU fewer than kMinBlocks blocks.  FAST_TAU_ZC overrides all of it.
// slab_depth sizes a volume solved alone (one right-hand side, the serving
// context's unit, so a served result equals the same request solved alone);
// launch_slab_depth a whole launch.
#include "slab_table.inc"

namespace {
std::atomic<int> g_slab[3][2][kSlabClasses];
std::once_flag g_slab_once;

void slab_init()
{
    std::call_once(g_slab_once, [] {
        for (int p = 0; p < 3; p++)
            for (int v = 0; v < 2; v++)
                for (int c = 0; c < kSlabClasses; c++) g_slab[p][v][c].store(kSlabTable[p][v][c]);
    });
}

int slab_class(int64_t W)
{
    int c = 0;
    while (c + 1 < kSlabClasses && (W >> (c + 1)) > 0) c++;
    return c;
}

// The depth of a launch of right-hand sides with dimensions dims.
int tuned_depth(int prec, int solver, const std::vector<const int64_t *> &dims)
{
    const int env = env_int("FAST_TAU_ZC", 0);
    if (env > 0) return env;
    int64_t W = 0;
    for (const int64_t *d : dims) {
        const Geometry G = make_geometry(d[0], d[1], d[2], 1);
        W += (int64_t)G.tx * G.ty * d[2];
    }
    if (prec >= 0 && prec < 3 && solver >= 0 && solver < 2) {
        slab_init();
        const int t = g_slab[prec][solver][slab_class(W)].load(std::memory_order_relaxed);
        if (t > 0) return t;
    }
    int zc = kSlabDepth;
    for (; zc > 2; zc /= 2) {
        int64_t blocks = 0;
        for (const int64_t *d : dims) blocks += make_geometry(d[0], d[1], d[2], zc).ntiles;
        if (blocks >= kMinBlocks) break;
    }
    return zc;
}
}  // namespace

int slab_depth(int64_t nx, int64_t ny, int64_t nz, int prec, int solver)
{
    const int64_t d[3] = {nx, ny, nz};
    return tuned_depth(prec, solver, {d});
}

int launch_slab_depth(const std::vector<VolSpec> &vols, const std::vector<JobSpec> &jobs, int prec, int solver)
{
    std::vector<const int64_t *> dims;
    std::vector<int64_t> flat(3 * vols.size());
    for (size_t v = 0; v < vols.size(); v++) {
        flat[3 * v] = vols[v].nx;
        flat[3 * v + 1] = vols[v].ny;
        flat[3 * v + 2] = vols[v].nz;
    }
    for (const JobSpec &j : jobs) dims.push_back(&flat[3 * j.vol]);
    return tuned_depth(prec, solver, dims);
}

// The one-sweep MIXED CG (OpCGF) is opt-in (FAST_TAU_CG_FUSED=1): its
// sweep is 7 % faster than the two classic ones (415 against 447 us on the
// 256^3 three-direction benchmark), but restarting at every residual
// replacement costs it about 4 % more iterations and four more vectors per
// right-hand side; the batched and served workloads ran slower with it
// (58.0 against 60.7 and 20.2 against 21.1 solves/s).
bool cg_fused_enabled()
{
    static const int on = env_int("FAST_TAU_CG_FUSED", 0);
    return on != 0;
}

size_t job_bytes(int64_t nx, int64_t ny, int64_t nz, int prec, int solver, int zc)
{
    const bool mixed = prec == FAST_PREC_MIXED;
    const size_t vec_t = (prec == FAST_PREC_F64) ? 8 : 4;
    // CG: x, r, p x2; BiCGSTAB: x, r x2, r0, p x2, v x2 (+ t for MIXED);
    // the one-sweep MIXED CG uses the MIXED BiCGSTAB set (r, s = v, w = t/r0
    // ping-pong, p and x in place)
    const bool fused = mixed && solver == FAST_SOLVER_CG && cg_fused_enabled();
    const size_t nvec = (solver == FAST_SOLVER_CG && !fused) ? 4 : (mixed ? 9 : 8);
    const size_t NP = (size_t)(row_pitch(nx) * ny * nz);
    const Geometry G = make_geometry(nx, ny, nz, zc > 0 ? zc : slab_depth(nx, ny, nz, prec, solver));
    return nvec * align_up(NP * vec_t, 256) + (mixed ? 2 * align_up(NP * 8, 256) : 0) +
           align_up((size_t)G.ntiles * NPART * sizeof(double), 256);
}

// Device bytes of a solve: one stencil-code array per volume, the state
// vectors, partial sums and scalars of every right-hand side.
size_t solve_bytes(const std::vector<VolSpec> &vols, const std::vector<JobSpec> &jobs, int prec, int solver, int zc)
{
    size_t need = 4096;
    for (const VolSpec &v : vols) need += code_bytes(v.nx, v.ny, v.nz);
    for (const JobSpec &j : jobs) need += job_bytes(vols[j.vol].nx, vols[j.vol].ny, vols[j.vol].nz, prec, solver, zc);
    const size_t nj = jobs.size(), nv = vols.size();
    need += align_up(sizeof(Scalars) * nj, 256) + align_up(sizeof(uint32_t) * nj, 256) +
            align_up(sizeof(Job) * (nj + nv), 256) + 256;  // + the replacement gate word
    return need;
}

int build_job(Job &J, Scalars &S, const uint8_t *d_mask, int64_t nx, int64_t ny, int64_t nz, int dir,
              const uint8_t *d_code, Scalars *d_sc, uint32_t *d_counter, Arena &A, const fast_tau_params &P, int zc)
{
    const int prec = P.precision, solver = P.solver;
    const bool mixed = prec == FAST_PREC_MIXED;
    const size_t vec_t = (prec == FAST_PREC_F64) ? 8 : 4;
    const Geometry G = make_geometry(nx, ny, nz, zc > 0 ? zc : slab_depth(nx, ny, nz, prec, solver));
    const int64_t pitch = row_pitch(nx);
    const int64_t NP = pitch * ny * nz;
    const size_t vbytes = align_up((size_t)NP * vec_t, 256);
    const size_t v64 = align_up((size_t)NP * 8, 256);
    memset(&J, 0, sizeof(Job));
    memset(&S, 0, sizeof(Scalars));
    J.nx = (int32_t)nx; J.ny = (int32_t)ny; J.nz = (int32_t)nz;
    J.pitch = (int32_t)pitch;
    J.dir = dir;
    J.tiles_x = G.tx; J.tiles_y = G.ty; J.tiles_z = G.tz;
    J.zc = G.zc;
    J.ntiles = G.ntiles;
    J.code = d_code;
    J.mask = d_mask;
    J.x = A.take(vbytes);
    J.r[0] = A.take(vbytes);
    J.p[0] = A.take(vbytes);
    J.p[1] = A.take(vbytes);
    const bool fused = mixed && solver == FAST_SOLVER_CG && cg_fused_enabled();
    if (solver == FAST_SOLVER_BICGSTAB || fused) {
        J.r[1] = A.take(vbytes);
        J.r0 = A.take(vbytes);
        J.v[0] = A.take(vbytes);
        J.v[1] = A.take(vbytes);
    }
    if (mixed) {
        J.x64[0] = A.take(v64);
        J.x64[1] = A.take(v64);
        if (solver == FAST_SOLVER_BICGSTAB || fused) J.t = A.take(vbytes);
    }
    J.part = (double *)A.take((size_t)G.ntiles * NPART * sizeof(double));
    if (A.off > A.cap) return fail(FAST_CUDA_ERROR, "internal: device plan overflow");
    const int es = (int)vec_t;
    int ts = tensor_map(&J.tm[TM_CODE], J.code, 1, nx, ny, nz, pitch);
    if (ts == FAST_OK) ts = tensor_map(&J.tm[TM_X], J.x, es, nx, ny, nz, pitch);
    if (ts == FAST_OK) ts = tensor_map(&J.tm[TM_R], J.r[0], es, nx, ny, nz, pitch);
    if (ts == FAST_OK) ts = tensor_map(&J.tm[TM_P], J.p[0], es, nx, ny, nz, pitch);
    if (ts == FAST_OK) ts = tensor_map(&J.tm[TM_P + 1], J.p[1], es, nx, ny, nz, pitch);
    if (ts == FAST_OK) ts = tensor_map(&J.tm[TM_XI], J.x, es, nx, ny, nz, pitch, true);
    if (ts == FAST_OK) ts = tensor_map(&J.tm[TM_RI], J.r[0], es, nx, ny, nz, pitch, true);
    if (ts == FAST_OK && (solver == FAST_SOLVER_BICGSTAB || fused)) {
        ts = tensor_map(&J.tm[TM_R + 1], J.r[1], es, nx, ny, nz, pitch);
        if (ts == FAST_OK) ts = tensor_map(&J.tm[TM_R0], J.r0, es, nx, ny, nz, pitch);
        if (ts == FAST_OK) ts = tensor_map(&J.tm[TM_R0I], J.r0, es, nx, ny, nz, pitch, true);
        if (ts == FAST_OK) ts = tensor_map(&J.tm[TM_V], J.v[0], es, nx, ny, nz, pitch);
        if (ts == FAST_OK) ts = tensor_map(&J.tm[TM_V + 1], J.v[1], es, nx, ny, nz, pitch);
    }
    if (ts == FAST_OK && mixed) {
        ts = tensor_map(&J.tm[TM_X64], J.x64[0], 8, nx, ny, nz, pitch);
        if (ts == FAST_OK) ts = tensor_map(&J.tm[TM_X64 + 1], J.x64[1], 8, nx, ny, nz, pitch);
        if (ts == FAST_OK && J.t) ts = tensor_map(&J.tm[TM_T], J.t, 4, nx, ny, nz, pitch);
    }
    if (ts != FAST_OK) return ts;
    J.sc = d_sc;
    J.counter = d_counter;
    fill_tables(J, P.d0, P.d1, P.face_mean);

    const int64_t maxdim = std::max(nx, std::max(ny, nz));
    const float h = 1.0f / (float)maxdim;  // cellDim = vec3(1.0f / maxDim) (VolumeMeasures.cpp:68)
    const double h2 = (double)h * (double)h;
    // Solver tolerance is T-typed (Solver.h:155-158).
    S.tol = (prec == FAST_PREC_F32) ? (double)(float)P.tolerance : P.tolerance;
    S.max_iter = P.max_iter;
    S.div_thresh = 10e+10 / h2;  // |r|^2 > 1e11 in the reference's h-scaled units
    S.eps2 = (prec == FAST_PREC_F64) ? (double)DBL_EPSILON * DBL_EPSILON : (double)FLT_EPSILON * (double)FLT_EPSILON;
    S.state = RUNNING;
    S.tol_outer = P.tolerance;
    // MIXED: the first step is a replacement with restart (x64 = x0, e = 0).
    S.replace = mixed ? 2 : 0;
    const double delta = env_double("FAST_TAU_REPLACE_DELTA", 0.03);
    S.delta2 = delta * delta;
    const double cmin = env_double("FAST_TAU_SHADOW_COS", 1e-6);
    S.cos2_min = cmin * cmin;
    S.inner_mode = mixed ? 1 : 0;
    S.cg_fused = fused ? 1 : 0;
    J.x64_ff = (mixed && (P.flags & FAST_FLAG_REPLACE_FLOAT_FLOAT)) ? 1 : 0;
#if defined(FAST_TAU_TEST_HOOKS) && FAST_TAU_TEST_HOOKS
    // test builds: FAST_TAU_TEST_WITHHOLD = 1 + direction arms the withheld
    // tile load of that direction's first sweep
    S.test_withhold = env_int("FAST_TAU_TEST_WITHHOLD", 0) == dir + 1 ? 1 : 0;
#endif
    // MIXED BiCGSTAB: no update is pending before the first replacement.
    S.alpha = 0.0;
    S.omega = 0.0;
    return FAST_OK;
}

// Solves every right-hand side of `jobs` (directions of the volumes in
// `vols`) together: one launch per solver step covers all of them, each
// block working for one (job, tile); converged right-hand sides drop out of
// the launches at block entry.  conc_out: only with a single job.
int solve_jobs(Engine &E, const std::vector<VolSpec> &vols, const std::vector<JobSpec> &jobs,
               const fast_tau_params &P, fast_tau_result *res, void *conc_out)
{
    cudaStream_t st = E.stream;
    t_prof.reset((P.flags & FAST_FLAG_PROFILE) != 0);
    const int prec = P.precision, solver = P.solver;
    const bool mixed = prec == FAST_PREC_MIXED;
    const bool ff = mixed && (P.flags & FAST_FLAG_REPLACE_FLOAT_FLOAT) != 0;
    const int nj = (int)jobs.size(), nv = (int)vols.size();
    if (nj < 1 || nj > Engine::kMaxJobs || nv < 1 || nv > nj)
        return fail(FAST_BAD_ARG, "1..%d right-hand sides per call", Engine::kMaxJobs);
    const size_t vec_t = (prec == FAST_PREC_F64) ? 8 : 4;

    // --- memory plan (the reference's fit check, VolumeMeasures.cpp:104-125)
    const int zc = launch_slab_depth(vols, jobs, prec, solver);
    const size_t need = solve_bytes(vols, jobs, prec, solver, zc);
    size_t free_b = 0, total_b = 0;
    CU(cudaMemGetInfo(&free_b, &total_b));
#if defined(FAST_TAU_TEST_HOOKS) && FAST_TAU_TEST_HOOKS
    // test builds: FAST_TAU_TEST_FREE_BYTES pretends the device has that much
    // free memory and nothing cached, so the fit check can be made to fail
    const char *fake_free = getenv("FAST_TAU_TEST_FREE_BYTES");
    if (fake_free) {
        free_b = (size_t)strtoull(fake_free, nullptr, 10);
        if (need > free_b)
            return fail(FAST_NOMEM, "Solver will not fit in GPU memory: needs %.3f GB, %.3f GB free", need / 1e9,
                        free_b / 1e9);
    }
#endif
    if (need > free_b) {
        // Memory already cached by the stream-ordered pool counts as available.
        size_t reserved = 0;
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, E.device) == cudaSuccess) {
            uint64_t r = 0, u = 0;
            cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &r);
            cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &u);
            reserved = (size_t)(r - u);
        }
        if (need > free_b + reserved)
            return fail(FAST_NOMEM, "Solver will not fit in GPU memory: needs %.3f GB, %.3f GB free", need / 1e9,
                        (free_b + reserved) / 1e9);
    }
    (void)total_b;

    Arena A;
    CU(cudaMallocAsync((void **)&A.base, need, st));
    A.cap = need;
    Scalars *d_sc = (Scalars *)A.take(sizeof(Scalars) * nj);
    uint32_t *d_cnt = (uint32_t *)A.take(sizeof(uint32_t) * nj);
    Job *d_jobs = (Job *)A.take(sizeof(Job) * (nj + nv));  // jobs, then one code job per volume
    uint32_t *d_gate = (uint32_t *)A.take(sizeof(uint32_t));  // MIXED replacement gate
    std::vector<uint8_t *> d_code(nv);
    std::vector<int> first_job(nv, -1);
    for (int v = 0; v < nv; v++) {
        const VolSpec &V = vols[v];
        d_code[v] = (uint8_t *)A.take((size_t)(row_pitch(V.nx) * V.ny * V.nz));
    }
    for (int j = 0; j < nj; j++)
        if (first_job[jobs[j].vol] < 0) first_job[jobs[j].vol] = j;

    // --- job descriptors
    Job *hj = E.h_jobs;
    Scalars *hs = E.h_sc;  // staging (the poll buffers are not in use yet)
    int64_t tile_base = 0;
    for (int j = 0; j < nj; j++) {
        const VolSpec &V = vols[jobs[j].vol];
        const int bs = build_job(hj[j], hs[j], V.d_mask, V.nx, V.ny, V.nz, jobs[j].dir, d_code[jobs[j].vol], d_sc + j,
                                 d_cnt + j, A, P, zc);
        if (bs != FAST_OK) {
            cudaFreeAsync(A.base, st);
            cudaStreamSynchronize(st);
            return bs;
        }
        hj[j].tile_base = tile_base;
        tile_base += hj[j].ntiles;
    }
    // One stencil-code job per volume (a copy of its first right-hand side
    // with its own tile numbering); the pore count lands in that job's scalars.
    int64_t code_base = 0;
    for (int v = 0; v < nv; v++) {
        Job &C = hj[nj + v];
        C = hj[first_job[v]];
        C.tile_base = code_base;
        code_base += C.ntiles;
    }
    if (tile_base > (int64_t)INT32_MAX || code_base > (int64_t)INT32_MAX) {
        cudaFreeAsync(A.base, st);
        cudaStreamSynchronize(st);
        return fail(FAST_BAD_ARG, "too many tiles in one launch (%lld)", (long long)tile_base);
    }
    CU(cudaMemcpyAsync(d_jobs, hj, sizeof(Job) * (nj + nv), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(d_sc, hs, sizeof(Scalars) * nj, cudaMemcpyHostToDevice, st));
    CU(cudaMemsetAsync(d_cnt, 0, sizeof(uint32_t) * nj, st));
    // every MIXED right-hand side starts with a pending replacement (x = x0):
    // the gate word reads 1
    CU(cudaMemsetAsync(d_gate, 0, sizeof(uint32_t), st));
    if (mixed) CU(cudaMemsetAsync(d_gate, 1, 1, st));
    // The staging buffers are reused below: wait for the copies to land.
    CU(cudaStreamSynchronize(st));

    Launch L{d_jobs, nj, 0, tile_base, mixed ? d_gate : nullptr};
    Launch LC{d_jobs + nj, nv, 0, code_base, nullptr};

    int status = FAST_OK;
    launch_counted(FAST_K_CODE, st, [&] { launch_code(LC, st); });
    if (!mixed) {
        void (*fn)(Step, const Launch &, cudaStream_t) = (prec == FAST_PREC_F64) ? dispatch_f64 : dispatch_f32;
        launch_counted(FAST_K_INIT, st, [&] { fn(solver == FAST_SOLVER_CG ? Step::INIT_CG : Step::INIT_BI, L, st); });
        std::vector<Step> steps;
        if (solver == FAST_SOLVER_CG) steps = {Step::CG1, Step::CG2};
        else steps = {Step::BI_RESTART, Step::BI1, Step::BI2, Step::BI3};
        status = iterate(E, L, nj, d_sc, steps, fn, P.max_iter);
    } else {
        // FP32 iterations with in-graph FP64 residual replacement: the
        // replacement slot leads every iteration and is a no-op launch unless
        // the recursion asked for it.
        launch_counted(FAST_K_INIT64, st, [&] { launch_init64(L, st); });
        std::vector<Step> steps;
        steps = mixed_steps(solver, ff);
        status = iterate(E, L, nj, d_sc, steps, dispatch_mixed, P.max_iter);
    }
    if (status == FAST_OK)
        launch_counted(FAST_K_TAU, st, [&] { launch_tau(mixed ? (ff ? 2 : 3) : (prec == FAST_PREC_F32 ? 1 : 0), L, st); });
    CU(cudaMemcpyAsync(hs, d_sc, sizeof(Scalars) * nj, cudaMemcpyDeviceToHost, st));
    if (conc_out && nj == 1) {
        const void *src = hj[0].x;
        size_t es = vec_t;
        CU(cudaStreamSynchronize(st));
        if (mixed && ff) {
            // The iterate is float-float: widen it to FP64 in the other
            // ping-pong buffer (free now), then copy that.
            const int cur = hs[0].x64_cur;
            const int64_t n = (int64_t)hj[0].pitch * vols[0].ny * vols[0].nz;
            launch_ff_to_double(hj[0].x64[cur], (double *)hj[0].x64[cur ^ 1], n, st);
            CU(cudaGetLastError());
            src = hj[0].x64[cur ^ 1];
            es = 8;
        } else if (mixed) {
            src = hj[0].x64[hs[0].x64_cur];
            es = 8;
        }
        // de-pad the rows: host layout is x-fastest with pitch nx
        const int64_t nx = vols[0].nx;
        CU(cudaMemcpy2DAsync(conc_out, (size_t)nx * es, src, (size_t)hj[0].pitch * es, (size_t)nx * es,
                             (size_t)(vols[0].ny * vols[0].nz), cudaMemcpyDeviceToHost, st));
    }
    cudaError_t ferr = cudaFreeAsync(A.base, st);
    CU(cudaStreamSynchronize(st));
    if (ferr != cudaSuccess) return fail(FAST_CUDA_ERROR, "cudaFreeAsync: %s", cudaGetErrorString(ferr));
    if (status != FAST_OK) return status;

    // --- results (the stencil-code pass counted each volume's pores into its
    // first right-hand side)
    int first_bad = FAST_OK;
    for (int j = 0; j < nj; j++) {
        Scalars &S = hs[j];
        const VolSpec &V = vols[jobs[j].vol];
        const uint64_t pores = hs[first_job[jobs[j].vol]].pores;
        const int64_t N = V.nx * V.ny * V.nz;
        fast_tau_result &R = res[j];
        memset(&R, 0, sizeof(R));
        R.status = status_of(S.state);
        R.iterations = S.iter;
        R.outer_steps = mixed ? (uint32_t)S.outer_steps : 0;
        if (mixed) R.rel_residual = S.b64_sq > 0 ? std::sqrt(S.r64_sq / S.b64_sq) : 0.0;
        else R.rel_residual = S.rhs_sq > 0 ? std::sqrt(S.rsq / S.rhs_sq) : 0.0;
        // Porosity: precomputed by the caller, or getPorosity<T> (VolumeMeasures.cpp:179-181).
        const int k = jobs[j].dir >> 1;
        const int64_t dimk = k == 0 ? V.nx : (k == 1 ? V.ny : V.nz);
        const int64_t nplane = N / dimk;
        if (prec == FAST_PREC_F32) {
            const float phi = P.porosity >= 0 ? (float)P.porosity : (float)pores / (float)N;
            R.porosity = phi;
            // tau = porosity / (dc * n_k), dc = sum over planes of (plane sum / n) / n_k
            const float S32 = (float)S.flux_sum;
            const float dc = (S32 / (float)nplane) / (float)dimk;
            R.tau = (R.status == FAST_OK) ? (double)(phi / (dc * (float)dimk)) : 0.0;
        } else {
            const double phi = P.porosity >= 0 ? P.porosity : (double)pores / (double)N;
            R.porosity = phi;
            const double dc = (S.flux_sum / (double)nplane) / (double)dimk;
            R.tau = (R.status == FAST_OK) ? phi / (dc * (double)dimk) : 0.0;
        }
        if (S.oob) {  // bounds-check builds only
            R.status = FAST_CUDA_ERROR;
            R.tau = 0.0;
            if (first_bad == FAST_OK)
                first_bad = fail(FAST_CUDA_ERROR, "bounds check: right-hand side %d, access site %d out of range", j,
                                 S.oob);
        }
        if (R.status != FAST_OK && first_bad == FAST_OK) {
            first_bad = R.status;
            fail(R.status, "right-hand side %d (direction %d): %s after %llu iterations (|r|/|b| = %.3e)", j,
                 jobs[j].dir,
                 R.status == FAST_DIVERGED  ? "solver diverged"
                 : R.status == FAST_TIMEOUT ? "a bounded device-side wait for tile loads ran out"
                                            : "solver did not converge",
                 (unsigned long long)R.iterations, R.rel_residual);
        }
        if (P.verbose)
            fprintf(stderr, "fasttau: rhs %d dir %d tau %.10g iters %llu outer %u relres %.3e status %d\n", j,
                    jobs[j].dir, R.tau, (unsigned long long)R.iterations, R.outer_steps, R.rel_residual, R.status);
    }
    return first_bad;
}

// The multi-direction solve of one device-resident volume.
int solve_device(Engine &E, const uint8_t *d_mask, int64_t nx, int64_t ny, int64_t nz, const fast_tau_params &P,
                 int ndirs, const int32_t *dirs, fast_tau_result *res, void *conc_out)
{
    std::vector<VolSpec> vols{{d_mask, nx, ny, nz}};
    std::vector<JobSpec> jobs;
    for (int j = 0; j < ndirs; j++) jobs.push_back({0, dirs[j]});
    return solve_jobs(E, vols, jobs, P, res, conc_out);
}

int check_params(const fast_tau_params *p);

int check_volume(const void *mask, int64_t nx, int64_t ny, int64_t nz)
{
    if (!mask) return fail(FAST_NO_HOST_DATA, "mask must be allocated (VolumeMeasures.cpp:55)");
    if (nx <= 0 || ny <= 0 || nz <= 0) return fail(FAST_BAD_ARG, "dimensions must be positive");
    if (nx > INT32_MAX / 2 || ny > INT32_MAX / 2 || nz > INT32_MAX / 2)
        return fail(FAST_BAD_ARG, "dimension too large");
    return FAST_OK;
}

int check_args(const void *mask, int64_t nx, int64_t ny, int64_t nz, const fast_tau_params *p, int ndirs,
               const int32_t *dirs)
{
    int s = check_volume(mask, nx, ny, nz);
    if (s != FAST_OK) return s;
    if (!p) return fail(FAST_BAD_ARG, "params is NULL");
    const Geometry G = make_geometry(nx, ny, nz);
    if (G.ntiles * (int64_t)std::max(ndirs, 1) > (int64_t)INT32_MAX) return fail(FAST_BAD_ARG, "volume too large");
    s = check_params(p);
    if (s != FAST_OK) return s;
    if (ndirs < 1 || ndirs > 6 || !dirs) return fail(FAST_BAD_ARG, "need 1..6 directions");
    for (int j = 0; j < ndirs; j++)
        if (dirs[j] < 0 || dirs[j] > 5) return fail(FAST_BAD_ARG, "bad direction %d", dirs[j]);
    return FAST_OK;
}

int check_params(const fast_tau_params *p)
{
    if (p->solver != FAST_SOLVER_BICGSTAB && p->solver != FAST_SOLVER_CG)
        return fail(FAST_BAD_ARG, "Unknown solver %d", p->solver);
    if (p->precision < FAST_PREC_F64 || p->precision > FAST_PREC_MIXED)
        return fail(FAST_BAD_ARG, "unknown precision %d", p->precision);
    if (p->face_mean != FAST_FACE_ARITHMETIC && p->face_mean != FAST_FACE_HARMONIC)
        return fail(FAST_BAD_ARG, "unknown face mean %d", p->face_mean);
    if (!(p->tolerance >= 0.0)) return fail(FAST_BAD_ARG, "tolerance must be >= 0");
    if (!(p->d0 > 0.0) || !(p->d1 > 0.0)) return fail(FAST_BAD_ARG, "diffusivities must be positive");
    return FAST_OK;
}

int check_batch(const fast_tau_volume *vols, int32_t nvols, const fast_tau_params *p, const fast_tau_result *res)
{
    if (!vols || !res) return fail(FAST_BAD_ARG, "volumes or results is NULL");
    if (!p) return fail(FAST_BAD_ARG, "params is NULL");
    if (nvols < 1 || nvols > 1024) return fail(FAST_BAD_ARG, "need 1..1024 volumes, got %d", nvols);
    for (int32_t v = 0; v < nvols; v++) {
        const int s = check_volume(vols[v].mask, vols[v].nx, vols[v].ny, vols[v].nz);
        if (s != FAST_OK) return fail(s, "volume %d: %s", v, g_last_error.c_str());
        if (vols[v].dir < 0 || vols[v].dir > 5) return fail(FAST_BAD_ARG, "volume %d: bad direction %d", v, vols[v].dir);
    }
    return check_params(p);
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

FAST_API const char *fast_last_error(void) { return g_last_error.c_str(); }

FAST_API const char *fast_version(void) { return "fasttau 0.1 (sm_103a)"; }

FAST_API int fast_tau_slab_depth(int64_t nx, int64_t ny, int64_t nz, int32_t nrhs, int32_t precision,
                                 int32_t solver, int32_t *depth, int32_t *size_class)
{
    ft_clear_error();
    if (!depth) return fail(FAST_BAD_ARG, "depth is NULL");
    if (nx < 1 || ny < 1 || nz < 1 || nrhs < 1 || nrhs > 6) return fail(FAST_BAD_ARG, "bad dimensions or nrhs");
    if (precision < FAST_PREC_F64 || precision > FAST_PREC_MIXED) return fail(FAST_BAD_ARG, "bad precision");
    if (solver != FAST_SOLVER_BICGSTAB && solver != FAST_SOLVER_CG) return fail(FAST_BAD_ARG, "bad solver");
    const int64_t d[3] = {nx, ny, nz};
    const std::vector<const int64_t *> dims((size_t)nrhs, d);
    *depth = std::min<int64_t>(tuned_depth(precision, solver, dims), nz);
    if (size_class) {
        const Geometry G = make_geometry(nx, ny, nz, 1);
        *size_class = slab_class((int64_t)G.tx * G.ty * nz * nrhs);
    }
    return FAST_OK;
}

FAST_API int fast_tau_set_slab_table(int32_t precision, int32_t solver, const int32_t *depth_by_class, int32_t nclass)
{
    ft_clear_error();
    if (precision < FAST_PREC_F64 || precision > FAST_PREC_MIXED) return fail(FAST_BAD_ARG, "bad precision");
    if (solver != FAST_SOLVER_BICGSTAB && solver != FAST_SOLVER_CG) return fail(FAST_BAD_ARG, "bad solver");
    if (nclass < 0 || nclass > kSlabClasses) return fail(FAST_BAD_ARG, "0..%d classes", kSlabClasses);
    if (nclass > 0 && !depth_by_class) return fail(FAST_BAD_ARG, "depth_by_class is NULL");
    for (int c = 0; c < nclass; c++)
        if (depth_by_class[c] < 0 || depth_by_class[c] > 1024) return fail(FAST_BAD_ARG, "depth out of range");
    slab_init();
    for (int c = 0; c < kSlabClasses; c++)
        g_slab[precision][solver][c].store(!depth_by_class ? kSlabTable[precision][solver][c]
                                                           : (c < nclass ? depth_by_class[c] : 0));
    return FAST_OK;
}

FAST_API int fast_tau_last_stats(fast_tau_stats *out)
{
    if (!out) return fail(FAST_BAD_ARG, "stats is NULL");
    *out = t_prof.st;
    return FAST_OK;
}

FAST_API void fast_tau_params_init(fast_tau_params *p)
{
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->dir = FAST_X_NEG;
    p->solver = FAST_SOLVER_BICGSTAB;
    p->precision = FAST_PREC_F64;
    p->face_mean = FAST_FACE_ARITHMETIC;
    p->tolerance = 1e-6;
    p->max_iter = 10000;
    p->d0 = (double)1.0f;
    p->d1 = (double)0.001f;
    p->porosity = -1.0;
}

FAST_API int fast_tau_solve_dirs_device(const uint8_t *d_mask, int64_t nx, int64_t ny, int64_t nz,
                                        const fast_tau_params *p, int32_t ndirs, const int32_t *dirs,
                                        fast_tau_result *results, void *stream)
{
    g_last_error.clear();
    int st = check_args(d_mask, nx, ny, nz, p, ndirs, dirs);
    if (st != FAST_OK) return st;
    if (!results) return fail(FAST_BAD_ARG, "results is NULL");
    Engine *E = nullptr;
    st = get_engine(&E);
    if (st != FAST_OK) return st;
    cudaStream_t saved = E->stream;
    if (stream) E->stream = (cudaStream_t)stream;
    st = solve_device(*E, d_mask, nx, ny, nz, *p, ndirs, dirs, results, nullptr);
    E->stream = saved;
    return st;
}

FAST_API int fast_tau_solve_batch_device(const fast_tau_volume *vols, int32_t nvols, const fast_tau_params *p,
                                         fast_tau_result *results, void *stream)
{
    g_last_error.clear();
    int st = check_batch(vols, nvols, p, results);
    if (st != FAST_OK) return st;
    Engine *E = nullptr;
    st = get_engine(&E);
    if (st != FAST_OK) return st;
    std::vector<VolSpec> vs;
    std::vector<JobSpec> js;
    for (int32_t v = 0; v < nvols; v++) {
        vs.push_back({vols[v].mask, vols[v].nx, vols[v].ny, vols[v].nz});
        js.push_back({(int)v, vols[v].dir});
    }
    cudaStream_t saved = E->stream;
    if (stream) E->stream = (cudaStream_t)stream;
    st = solve_jobs(*E, vs, js, *p, results, nullptr);
    E->stream = saved;
    return st;
}

FAST_API int fast_tau_solve_batch(const fast_tau_volume *vols, int32_t nvols, const fast_tau_params *p,
                                  fast_tau_result *results)
{
    g_last_error.clear();
    int st = check_batch(vols, nvols, p, results);
    if (st != FAST_OK) return st;
    Engine *E = nullptr;
    st = get_engine(&E);
    if (st != FAST_OK) return st;
    size_t total = 0;
    for (int32_t v = 0; v < nvols; v++) total += align_up((size_t)(vols[v].nx * vols[v].ny * vols[v].nz), 256);
    uint8_t *d_all = nullptr;
    CU(cudaMallocAsync((void **)&d_all, total, E->stream));
    std::vector<VolSpec> vs;
    std::vector<JobSpec> js;
    size_t off = 0;
    cudaError_t e = cudaSuccess;
    for (int32_t v = 0; v < nvols && e == cudaSuccess; v++) {
        const size_t n = (size_t)(vols[v].nx * vols[v].ny * vols[v].nz);
        e = cudaMemcpyAsync(d_all + off, vols[v].mask, n, cudaMemcpyHostToDevice, E->stream);
        vs.push_back({d_all + off, vols[v].nx, vols[v].ny, vols[v].nz});
        js.push_back({(int)v, vols[v].dir});
        off += align_up(n, 256);
    }
    if (e != cudaSuccess) st = fail(FAST_CUDA_ERROR, "mask upload: %s", cudaGetErrorString(e));
    else st = solve_jobs(*E, vs, js, *p, results, nullptr);
    cudaFreeAsync(d_all, E->stream);
    cudaStreamSynchronize(E->stream);
    return st;
}

static int solve_host(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, const fast_tau_params *p,
                      int32_t ndirs, const int32_t *dirs, fast_tau_result *results, void *conc_out)
{
    g_last_error.clear();
    int st = check_args(mask, nx, ny, nz, p, ndirs, dirs);
    if (st != FAST_OK) return st;
    Engine *E = nullptr;
    st = get_engine(&E);
    if (st != FAST_OK) return st;
    const size_t N = (size_t)(nx * ny * nz);
    uint8_t *d_mask = nullptr;
    CU(cudaMallocAsync((void **)&d_mask, N, E->stream));
    cudaError_t e = cudaMemcpyAsync(d_mask, mask, N, cudaMemcpyHostToDevice, E->stream);
    if (e != cudaSuccess) {
        cudaFreeAsync(d_mask, E->stream);
        return fail(FAST_CUDA_ERROR, "mask upload: %s", cudaGetErrorString(e));
    }
    st = solve_device(*E, d_mask, nx, ny, nz, *p, ndirs, dirs, results, conc_out);
    cudaFreeAsync(d_mask, E->stream);
    cudaStreamSynchronize(E->stream);
    return st;
}

FAST_API int fast_tau_solve_dirs(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz,
                                 const fast_tau_params *p, int32_t ndirs, const int32_t *dirs,
                                 fast_tau_result *results)
{
    if (!results) return fail(FAST_BAD_ARG, "results is NULL");
    return solve_host(mask, nx, ny, nz, p, ndirs, dirs, results, nullptr);
}

FAST_API int fast_tau_solve(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, const fast_tau_params *p,
                            double *tau, uint64_t *iters, double *rel_err, void *conc_out)
{
    if (tau) *tau = 0.0;
    if (!p) return fail(FAST_BAD_ARG, "params is NULL");
    fast_tau_result r;
    memset(&r, 0, sizeof(r));
    const int32_t dir = p->dir;
    int st = solve_host(mask, nx, ny, nz, p, 1, &dir, &r, conc_out);
    if (tau) *tau = r.tau;
    if (iters) *iters = r.iterations;
    if (rel_err) *rel_err = r.rel_residual;
    return st;
}

FAST_API int fast_porosity(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, double *porosity,
                           uint64_t *pore_count)
{
    g_last_error.clear();
    if (!mask) return fail(FAST_NO_HOST_DATA, "mask must be allocated");
    if (nx <= 0 || ny <= 0 || nz <= 0) return fail(FAST_BAD_ARG, "dimensions must be positive");
    Engine *E = nullptr;
    int st = get_engine(&E);
    if (st != FAST_OK) return st;
    const Geometry G = make_geometry(nx, ny, nz);
    const size_t N = (size_t)G.N;
    const int64_t P = row_pitch(nx);
    const size_t NP = (size_t)(P * ny * nz);
    cudaStream_t s = E->stream;
    Arena A;
    const size_t need = align_up(N, 256) + align_up(NP, 256) + align_up((size_t)G.ntiles * NPART * 8, 256) +
                        align_up(sizeof(Scalars), 256) + align_up(sizeof(uint32_t), 256) + align_up(sizeof(Job), 256);
    CU(cudaMallocAsync((void **)&A.base, need, s));
    uint8_t *d_mask = (uint8_t *)A.take(N);
    uint8_t *d_code = (uint8_t *)A.take(NP);
    double *d_part = (double *)A.take((size_t)G.ntiles * NPART * 8);
    Scalars *d_sc = (Scalars *)A.take(sizeof(Scalars));
    uint32_t *d_cnt = (uint32_t *)A.take(sizeof(uint32_t));
    Job *d_job = (Job *)A.take(sizeof(Job));
    Job &J = E->h_jobs[0];
    memset(&J, 0, sizeof(Job));
    J.nx = (int32_t)nx; J.ny = (int32_t)ny; J.nz = (int32_t)nz;
    J.pitch = (int32_t)P;
    J.tiles_x = G.tx; J.tiles_y = G.ty; J.tiles_z = G.tz; J.zc = G.zc;
    J.ntiles = G.ntiles;
    J.code = d_code; J.mask = d_mask; J.part = d_part; J.sc = d_sc; J.counter = d_cnt;
    CU(cudaMemcpyAsync(d_mask, mask, N, cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(d_job, &J, sizeof(Job), cudaMemcpyHostToDevice, s));
    CU(cudaMemsetAsync(d_sc, 0, sizeof(Scalars), s));
    CU(cudaMemsetAsync(d_cnt, 0, sizeof(uint32_t), s));
    Launch L{d_job, 1, 0, G.ntiles, nullptr};
    launch_code(L, s);
    CU(cudaMemcpyAsync(E->h_sc, d_sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
    cudaFreeAsync(A.base, s);
    CU(cudaStreamSynchronize(s));
    const uint64_t pores = E->h_sc[0].pores;
    if (pore_count) *pore_count = pores;
    if (porosity) *porosity = (double)pores / (double)N;
    return FAST_OK;
}

}  // extern "C"
