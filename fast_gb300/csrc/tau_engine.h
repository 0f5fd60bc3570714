// Host-side engine internals shared by the solver entry points
// (tau_host.cu) and the serving context (serve.cu).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <vector>

#include "fasttau.h"
#include "tau_errors.h"
#include "tau_launch.h"
#include "tau_types.h"

namespace ft {

// Per-thread, per-device engine: one non-blocking stream, pinned staging.
struct Engine {
    int device = -1;
    cudaStream_t stream = nullptr;
    Scalars *h_sc = nullptr;   // pinned, 2 * kMaxJobs (double-buffered poll)
    Job *h_jobs = nullptr;     // pinned staging for job descriptors (2 * kMaxJobs)
    static constexpr int kMaxJobs = 1024;
    int init(int dev);
};

int get_engine(Engine **out);
int env_int(const char *name, int dflt);
double env_double(const char *name, double dflt);

struct Geometry {
    int64_t nx, ny, nz, N;
    int zc, tx, ty, tz;
    int64_t ntiles;
};
constexpr int kSlabDepth = 32;   // planes per block (full size)
constexpr int kMinBlocks = 608;  // 4 blocks per SM on 152 SMs
// zc_req > 0: that slab depth; 0: FAST_TAU_ZC or kSlabDepth.
Geometry make_geometry(int64_t nx, int64_t ny, int64_t nz, int zc_req = 0);
// The slab depth of a volume solved alone with (precision, solver): the
// tuned table of its size class; FAST_TAU_ZC overrides.
int slab_depth(int64_t nx, int64_t ny, int64_t nz, int prec, int solver);
size_t align_up(size_t v, size_t a);
// Row pitch (elements) of every array of a volume: nx rounded up to 16, so a
// row of any element size starts on a 16-byte boundary (TMA stride rule).
int64_t row_pitch(int64_t nx);

// Device bytes of one right-hand side (state vectors + partial sums; zc = 0:
// the volume's slab depth) and of a volume's stencil codes.
size_t job_bytes(int64_t nx, int64_t ny, int64_t nz, int prec, int solver, int zc = 0);
size_t code_bytes(int64_t nx, int64_t ny, int64_t nz);

// Bump allocator over one device allocation.
struct Arena {
    char *base = nullptr;
    size_t off = 0, cap = 0;
    void *take(size_t bytes)
    {
        void *p = base + off;
        off += align_up(bytes, 256);
        return p;
    }
};

// Fills the descriptor and initial scalars of one right-hand side: state
// vectors carved from `A`, tensor maps, coefficient tables; `d_sc` and
// `d_counter` are its device scalars and finisher counter; tile_base is left
// to the caller.  zc = 0: the volume's slab depth.
int build_job(Job &J, Scalars &S, const uint8_t *d_mask, int64_t nx, int64_t ny, int64_t nz, int dir,
              const uint8_t *d_code, Scalars *d_sc, uint32_t *d_counter, Arena &A, const fast_tau_params &P,
              int zc = 0);

int status_of(int state);
int check_params(const fast_tau_params *p);
int check_volume(const void *mask, int64_t nx, int64_t ny, int64_t nz);
void dispatch_mixed(Step s, const Launch &L, cudaStream_t st);
// The per-iteration steps of a MIXED solve (CG: one fused sweep, or the
// classic two with FAST_TAU_CG_FUSED=0).
bool cg_fused_enabled();
// Captures `chunk` iterations of `steps` on `st` into an executable graph.
int capture_chunk(cudaStream_t st, const Launch &L, const std::vector<Step> &steps, int chunk,
                  void (*launch)(Step, const Launch &, cudaStream_t), cudaGraphExec_t *exec);
// MIXED steps of one iteration: the replacement slot (FP64 iterate, or
// float-float with `ff`) and the FP32 sweeps.
std::vector<Step> mixed_steps(int solver, bool ff);

}  // namespace ft
