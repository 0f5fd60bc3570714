/*
 * fasttau.h -- C ABI of the GB300 tortuosity engine (libfasttau.so).
 *
 * The drop-in boundary for fastlib's tortuosity path (krsvojte/fast):
 *   template<T> T fast::getTortuosity(const Volume&, const TortuosityParams&,
 *       DiffusionSolverType, Volume* concetrationOutput, size_t* iterationsOut)
 *   (fastlib/include/fastlib/volume/VolumeMeasures.h:51-58, implemented at
 *    fastlib/src/volume/VolumeMeasures.cpp:42-285)
 * and its helpers getPorosity<T> (VolumeMeasures.h:60-61), getVolumeCCL
 * (fastlib/src/volume/VolumeSegmentation.cpp:26-64).
 *
 * All entry points are plain C: pointers, sizes and POD structs.  Volumes are
 * uint8 arrays with x fastest, index i = x + nx*(y + ny*z)
 * (fastlib/include/fastlib/utility/Types.h:30-32); 0 = pore (D0), nonzero =
 * solid (D1).  Every function returns a fast_status; on failure
 * fast_last_error() gives a message for the calling thread.
 */
#ifndef FASTTAU_H
#define FASTTAU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define FAST_API __attribute__((visibility("default")))
#else
#define FAST_API
#endif

/* Status codes.  The reference reports every failure as tau = 0 plus a
 * message on stderr (VolumeMeasures.cpp:50-58,100,104-125,157-159); the C
 * ABI names the cause instead and the language shims map non-OK to 0. */
typedef enum fast_status {
    FAST_OK = 0,
    FAST_BAD_TYPE = 1,      /* mask is not uint8 / bad argument (VolumeMeasures.cpp:50) */
    FAST_NO_HOST_DATA = 2,  /* mask pointer is NULL (VolumeMeasures.cpp:55) */
    FAST_NOMEM = 3,         /* device memory does not fit (VolumeMeasures.cpp:104-125) */
    FAST_NO_CONVERGENCE = 4,/* iteration limit reached (CG.cpp:70, VolumeMeasures.cpp:157) */
    FAST_DIVERGED = 5,      /* |r|^2 > 1e11 in reference units (CG.cu:152, BICGSTAB.cu:207) */
    FAST_CUDA_ERROR = 6,    /* a CUDA call failed; the context stays usable */
    FAST_TIMEOUT = 7,       /* a bounded device-side wait ran out */
    FAST_BAD_ARG = 8,       /* invalid dimension / direction / solver / precision */
    FAST_IO_ERROR = 9       /* a volume file or folder cannot be read (VolumeIO.cpp:197-254) */
} fast_status;

/* enum Dir (fastlib/include/fastlib/utility/PrimitiveTypes.h:142-150). */
typedef enum fast_dir {
    FAST_X_POS = 0, FAST_X_NEG = 1, FAST_Y_POS = 2,
    FAST_Y_NEG = 3, FAST_Z_POS = 4, FAST_Z_NEG = 5
} fast_dir;

/* enum DiffusionSolverType (VolumeMeasures.h:15-18). */
typedef enum fast_solver { FAST_SOLVER_BICGSTAB = 0, FAST_SOLVER_CG = 1 } fast_solver;

/* Arithmetic of the solve.  F64 / F32 are the reference's `-p double` /
 * `-p float` (TauModule.h:19,125-129): the whole solve in that type.  MIXED is
 * the engine's fast path: FP32 Krylov iterations (FP32-accumulated,
 * block-compensated dot products) on a correction e of an FP64 iterate x;
 * whenever the FP32 recursive residual has fallen well below its recent
 * largest value, claims convergence or breaks down, an FP64 step folds e into
 * x, recomputes the true residual b - A x in FP64 and hands it back to the
 * recursion (residual replacement, with a Krylov restart on breakdown).  Convergence is decided
 * on the FP64 true residual; the tau flux integral is FP64. */
typedef enum fast_precision { FAST_PREC_F64 = 0, FAST_PREC_F32 = 1, FAST_PREC_MIXED = 2 } fast_precision;

/* Face diffusivity between two voxels.  The reference uses the arithmetic
 * mean (fastlib/src/cuda/Diffusion.cu:47-53, fastlib/src/solver/Diffusion.cpp:
 * 119-125); HARMONIC is an opt-in extension and never the parity mode. */
typedef enum fast_face_mean { FAST_FACE_ARITHMETIC = 0, FAST_FACE_HARMONIC = 1 } fast_face_mean;

/* TortuosityParams (VolumeMeasures.h:20-34) + the CLI's precision/solver. */
typedef struct fast_tau_params {
    int32_t dir;            /* fast_dir; reference default X_NEG */
    int32_t solver;         /* fast_solver; reference API default BICGSTAB, CLI default CG */
    int32_t precision;      /* fast_precision */
    int32_t face_mean;      /* fast_face_mean; 0 = arithmetic */
    double tolerance;       /* relative residual, reference default 1e-6 */
    uint64_t max_iter;      /* reference default 10000; MIXED: cap on the FP32 iterations */
    double d0;              /* pore diffusivity; the reference passes float 1.0 */
    double d1;              /* solid diffusivity; the reference passes (double)0.001f */
    double porosity;        /* < 0: computed on the GPU (getPorosity<T>); else used as given */
    int32_t verbose;        /* print per-solve summary to stderr */
    int32_t flags;          /* FAST_FLAG_* */
} fast_tau_params;

/* fast_tau_params.flags: time every kernel launch of the solve with CUDA
 * events (launches are serialised and not graph-replayed while profiling). */
#define FAST_FLAG_PROFILE 1
/* MIXED only: keep the iterate as a float-float pair per voxel and evaluate
 * the replacement's b - A x with error-free FP32 transformations (about 48
 * significant bits) instead of FP64.  Off by default: FP64 is the contract. */
#define FAST_FLAG_REPLACE_FLOAT_FLOAT 2

/* Per-direction result. */
typedef struct fast_tau_result {
    double tau;             /* 0 on failure, as the reference */
    double porosity;        /* the porosity used */
    double rel_residual;    /* |r|/|b| at exit (recursive residual; MIXED: true FP64 residual) */
    uint64_t iterations;    /* reference counting: CG excludes the converging iteration,
                               BiCGSTAB counts it (CG.cu:109-144, BICGSTAB.cu:211);
                               MIXED: FP32 iterations */
    uint32_t outer_steps;   /* MIXED: FP64 residual replacements, the first (x = x0) included;
                               0 otherwise */
    int32_t status;         /* fast_status */
} fast_tau_result;

/* Fill *p with the reference defaults (TortuosityParams with the CLI's
 * float coeffs {1.0, 0.001}): dir X_NEG, BICGSTAB, F64, tol 1e-6, 10000 iters. */
FAST_API void fast_tau_params_init(fast_tau_params *p);

/* getTortuosity<T> (VolumeMeasures.h:51-58).  `mask` is a HOST uint8 array of
 * nx*ny*nz voxels, borrowed.  Solves one direction on the calling thread's
 * device and stream, synchronously.  conc_out (nullable) receives the HOST
 * concentration field: double for F64/MIXED, float for F32 (the reference's
 * concetrationOutput, VolumeMeasures.cpp:146-149).  tau/iters/rel_err are
 * nullable.  Returns FAST_OK or the failure cause; *tau is 0 on failure. */
FAST_API int fast_tau_solve(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz,
                            const fast_tau_params *p, double *tau, uint64_t *iters,
                            double *rel_err, void *conc_out);

/* Several directions of one volume in one call: the directions share the
 * device-resident phase field and are advanced together as multiple
 * right-hand sides (one launch per kernel step for all of them).  `dirs` has
 * ndirs entries (each a fast_dir, ndirs <= 6); p->dir is ignored.  results has
 * ndirs entries.  Returns the first non-OK status, FAST_OK if all succeeded. */
FAST_API int fast_tau_solve_dirs(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz,
                                 const fast_tau_params *p, int32_t ndirs, const int32_t *dirs,
                                 fast_tau_result *results);

/* The same on a DEVICE-resident mask (a cudaMalloc'ed pointer on the current
 * device) on a caller stream (cudaStream_t passed as void*, NULL = the
 * library's stream).  Synchronises that stream before returning. */
FAST_API int fast_tau_solve_dirs_device(const uint8_t *d_mask, int64_t nx, int64_t ny, int64_t nz,
                                        const fast_tau_params *p, int32_t ndirs,
                                        const int32_t *dirs, fast_tau_result *results,
                                        void *stream);

/* One volume of a batch: a uint8 mask (HOST for fast_tau_solve_batch,
 * DEVICE for fast_tau_solve_batch_device), its dimensions and the direction
 * to solve. */
typedef struct fast_tau_volume {
    const uint8_t *mask;
    int64_t nx, ny, nz;
    int32_t dir;            /* fast_dir */
    int32_t reserved;
} fast_tau_volume;

/* Many volumes of different sizes in one call (no counterpart in the
 * reference, which solves one volume per getTortuosity call): all right-hand
 * sides advance together, one launch per solver step covering every
 * (volume, tile) pair, and each is retired as soon as it converges.  The
 * reductions of a right-hand side never mix with another's; a result equals
 * solving the volume alone up to the summation order of its dot products,
 * which follows the slab depth (chosen for the whole launch by its size; a
 * volume alone may get a shallower one).  1..1024 volumes; p->dir is ignored.
 * Returns the first non-OK status. */
FAST_API int fast_tau_solve_batch(const fast_tau_volume *vols, int32_t nvols, const fast_tau_params *p,
                                  fast_tau_result *results);
FAST_API int fast_tau_solve_batch_device(const fast_tau_volume *vols, int32_t nvols, const fast_tau_params *p,
                                         fast_tau_result *results, void *stream);

/* ------------------------------------------------------------------------ */
/* Serving context: continuous batching of requests on one GPU (no          */
/* counterpart in the reference, which solves one volume per run).  A       */
/* context queues submitted requests; every fast_ctx_poll runs one          */
/* scheduling step: it retires the solves that finished, admits queued      */
/* requests (oldest first) while a slot is free and their device footprint  */
/* fits hbm_budget, and advances every in-flight solve by `chunk`           */
/* iterations in shared launches (one CUDA graph per solver).  A request's  */
/* result is identical to solving it alone.  A context is used by one host  */
/* thread at a time.                                                        */
/* ------------------------------------------------------------------------ */
typedef struct fast_ctx_config {
    int32_t precision;      /* fast_precision; default MIXED */
    int32_t face_mean;      /* fast_face_mean */
    double tolerance;       /* default 1e-6 */
    uint64_t max_iter;      /* default 10000 */
    double d0, d1;          /* default (double)1.0f, (double)0.001f */
    int32_t chunk;          /* iterations per scheduling step, default 16 */
    int32_t max_inflight;   /* solves on the GPU at once, 1..1024, default 256 */
    uint64_t hbm_budget;    /* device bytes for in-flight solves; 0 = 80 % of free memory */
} fast_ctx_config;

typedef struct fast_ctx_completion {
    uint64_t ticket;        /* from fast_ctx_submit */
    fast_tau_result result;
    int32_t dir, solver;
    double t_submit, t_admit, t_done;  /* seconds on the context's clock */
} fast_ctx_completion;

typedef struct fast_ctx_stats {
    uint64_t pending, inflight, completed, admitted, steps;
    uint64_t bytes_inflight, hbm_budget;
    double now;             /* the context's clock, seconds since creation */
} fast_ctx_stats;

FAST_API void fast_ctx_config_init(fast_ctx_config *cfg);
FAST_API int fast_ctx_create(const fast_ctx_config *cfg, void **ctx);
/* Queues a request; the HOST mask is copied, so the caller may free it. */
FAST_API int fast_ctx_submit(void *ctx, const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, int32_t dir,
                             int32_t solver, uint64_t *ticket);
/* One scheduling step; up to `cap` finished requests are written to out and
 * counted in *n_done (the others are returned by later polls). */
FAST_API int fast_ctx_poll(void *ctx, fast_ctx_completion *out, int32_t cap, int32_t *n_done);
FAST_API int fast_ctx_query(void *ctx, fast_ctx_stats *out);
FAST_API int fast_ctx_destroy(void *ctx);

/* getPorosity<T> (VolumeMeasures.h:60-61 via Volume::sumZeroElems,
 * fastlib/src/volume/Volume.cpp:261-272): fraction of zero voxels, counted on
 * the GPU.  pore_count is nullable. */
FAST_API int fast_porosity(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz,
                           double *porosity, uint64_t *pore_count);

/* Kernel kinds of fast_tau_stats. */
enum {
    FAST_K_CODE = 0, FAST_K_INIT = 1, FAST_K_CG1 = 2, FAST_K_CG2 = 3, FAST_K_BI_RESTART = 4,
    FAST_K_BI1 = 5, FAST_K_BI2 = 6, FAST_K_BI3 = 7, FAST_K_REPLACE = 8, FAST_K_INIT64 = 9,
    FAST_K_TAU = 10, FAST_K_CGF = 11, FAST_K_COUNT = 16
};

/* Launch statistics of the calling thread's last solve. */
typedef struct fast_tau_stats {
    uint64_t launches;                 /* kernel launches of the engine (graph-replayed ones included) */
    uint64_t graph_replays;
    uint64_t kernel_launches[FAST_K_COUNT];
    double kernel_ms[FAST_K_COUNT];    /* summed CUDA-event durations (FAST_FLAG_PROFILE only) */
    int32_t profiled;
    int32_t pad;
} fast_tau_stats;

FAST_API int fast_tau_last_stats(fast_tau_stats *out);

/* Slab depth (z planes per block of the solver sweeps) by size class.  No
 * reference counterpart: the reference launches one thread per voxel.  A
 * launch's class is floor(log2(W)), W = the sum over its right-hand sides of
 * ceil(nx/64) * ceil(ny/8) * nz.  fast_tau_slab_depth gives the depth a solve
 * of nrhs right-hand sides of an nx x ny x nz volume would use (the
 * FAST_TAU_ZC environment variable overrides the table).
 * fast_tau_set_slab_table installs the depths of one (precision, solver) for
 * classes 0..nclass-1 (0 = no entry: the full depth, halved while the launch
 * has fewer than 608 blocks); depth_by_class NULL restores the built-in
 * table, which fast_gb300/autotune.py writes from GB300 timings. */
FAST_API int fast_tau_slab_depth(int64_t nx, int64_t ny, int64_t nz, int32_t nrhs, int32_t precision,
                                 int32_t solver, int32_t *depth, int32_t *size_class /* nullable */);
FAST_API int fast_tau_set_slab_table(int32_t precision, int32_t solver, const int32_t *depth_by_class,
                                     int32_t nclass);

/* Pore count of a DEVICE-resident mask that allocates nothing, for callers
 * that cannot allocate device memory: an application whose own allocator has
 * reserved all of the GPU's memory, or a plug-in host that forbids its
 * plug-ins to allocate device memory.  No counterpart in the reference.  The
 * reduction's scratch is a 256 KiB static device array inside the library,
 * held by every GPU that loads the library until exit; volumes above
 * 2,145,386,496 voxels (32736 blocks x 65536 voxels) are rejected with
 * FAST_BAD_ARG.  The first call on a device looks up the array's device
 * address and loads the kernel: make one complete call on each device before
 * any stream capture.  The address is kept for the life of the process and
 * is not valid after a cudaDeviceReset.  All calls share the array, so calls
 * that overlap on the GPU race.  stream: a cudaStream_t as void*, NULL = the
 * legacy default stream; the call copies the count into host memory and
 * synchronises that stream before it returns.  porosity is nullable. */
FAST_API int fast_porosity_device_noalloc(const uint8_t *d_mask, int64_t nx, int64_t ny, int64_t nz,
                                          uint64_t *pore_count, double *porosity, void *stream);

/* ------------------------------------------------------------------------ */
/* Connected components (the reachability pre-pass)                         */
/* ------------------------------------------------------------------------ */

/* getVolumeCCL(mask, background) (fastlib/src/volume/VolumeSegmentation.cpp:
 * 33-64) = VolumeCCL_Label + VolumeCCL_BoundaryLabels (fastlib/src/cuda/
 * VolumeCCL.cu:381-620, 753-818), on the GPU, with the reference's numbering:
 * foreground = voxels != background, 6-connected; labels[i] = 0 for
 * background, else 1..K with components ordered by their smallest linear
 * index (x fastest); *num_labels = K + 1.  boundary (nullable, host,
 * boundary_cap bytes, needs 7 * num_labels): row d (Dir order; X_POS is the
 * x = nx-1 face) marks labels touching face d, row 6 is the AND of rows 0-5
 * (VolumeCCL::getDirMask).  A too small boundary buffer gives FAST_BAD_ARG
 * with *num_labels set.  labels (host, nx*ny*nz uint32) is nullable.  Volumes
 * of 4294967295 voxels or more are rejected. */
FAST_API int fast_ccl_label(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, uint8_t background,
                            uint32_t *labels, uint32_t *num_labels, uint8_t *boundary, uint64_t boundary_cap);

/* The same on a DEVICE mask, labels written to DEVICE memory d_labels
 * (nx*ny*nz uint32); boundary stays a host buffer.  stream: a cudaStream_t
 * as void*, NULL = the legacy default stream; the call synchronises it. */
FAST_API int fast_ccl_label_device(const uint8_t *d_mask, int64_t nx, int64_t ny, int64_t nz, uint8_t background,
                                   uint32_t *d_labels, uint32_t *num_labels, uint8_t *boundary,
                                   uint64_t boundary_cap, void *stream);

/* VolumeCCL_BoundaryLabels (fastlib/src/cuda/VolumeCCL.cu:753-818) alone, on
 * DEVICE labels from fast_ccl_label_device: boundary (host, 7 * num_labels
 * bytes) as fast_ccl_label fills it. */
FAST_API int fast_ccl_boundary_device(const uint32_t *d_labels, int64_t nx, int64_t ny, int64_t nz,
                                      uint32_t num_labels, uint8_t *boundary, void *stream);

/* ------------------------------------------------------------------------ */
/* Volume input: TIFF folders and binarize                                   */
/* ------------------------------------------------------------------------ */

/* The scan of loadTiffFolder (fastlib/src/volume/VolumeIO.cpp:197-235): the
 * dimensions of the volume a folder of 2D slices makes.  nx, ny = the first
 * slice's width and height in byte-wise name order, nz = the number of files
 * named *.tif or *.tiff (case-sensitive, as checkExtension).  Slices are
 * baseline TIFF: uncompressed strips, 8-bit unsigned samples, either byte
 * order; sample 0 of multi-sample pixels is read.  Other forms give
 * FAST_BAD_TYPE (not 8-bit unsigned) or FAST_IO_ERROR.  Host-only work. */
FAST_API int fast_tiff_folder_info(const char *folder, int64_t *nx, int64_t *ny, int64_t *nz);

/* loadTiffFolder's reads (VolumeIO.cpp:237-248): slice z of the folder (name
 * order) into out + z*nx*ny, rows y-major, x fastest; capacity = bytes of
 * out.  Slices whose size differs from the first give FAST_IO_ERROR.  The
 * voxels are the slices' raw values: the reference's TIFF input binarizes
 * them next (fast_binarize). */
FAST_API int fast_tiff_folder_read(const char *folder, uint8_t *out, uint64_t capacity);

/* Volume::binarize(threshold) on a uint8 volume (fastlib/src/volume/
 * Volume.cpp:478-486, kernelBinarizeUnsigned in fastlib/src/cuda/Volume.cu:
 * 157-183): v = v < t ? 0 : 255 with t = uchar(threshold * 255) (threshold
 * clamped to [0, 1] first; the reference's `fast tau` passes 1.0, so only 255
 * stays 255).  Runs on the GPU.  fast_binarize takes a HOST volume of n bytes
 * (copied in and back); fast_binarize_device a DEVICE one on `stream` (a
 * cudaStream_t as void*, NULL = legacy default stream; not synchronised). */
FAST_API int fast_binarize(uint8_t *volume, uint64_t n, float threshold);
FAST_API int fast_binarize_device(uint8_t *d_volume, uint64_t n, float threshold, void *stream);

/* ------------------------------------------------------------------------ */
/* Reactive area density (`fast alpha`)                                       */
/* ------------------------------------------------------------------------ */

/* getReactiveAreaDensity<T>(mask, mask.dim(), isovalue) (fastlib/src/volume/
 * VolumeMeasures.cpp:294-301 over getVolumeArea, VolumeSurface.cpp:10-36, and
 * the marching-cubes cell kernel, fastlib/src/cuda/VolumeSurface.cu:198-262):
 * the area of the isovalue surface of the volume read as v/255 at the cell
 * corners (each corner = mean of the 2x2x2 voxels around it, clamped at the
 * faces), in normalized units (axis a scaled by 1/n_a), summed in double.
 * The mask must hold 0 and 255 only (FAST_BAD_TYPE otherwise); `fast alpha`
 * uses isovalue 0.5.  The triangulation table is the engine's own (see
 * alpha.cu): areas of cells whose loop is not planar differ slightly from the
 * reference's table.  Host mask; synchronous. */
FAST_API int fast_reactive_area(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, float isovalue,
                                double *area);

/* The same on a DEVICE mask; stream: a cudaStream_t as void*, NULL = the
 * legacy default stream; the call synchronises it. */
FAST_API int fast_reactive_area_device(const uint8_t *d_mask, int64_t nx, int64_t ny, int64_t nz, float isovalue,
                                       double *area, void *stream);

/* getVolumeCCL(mask, 255) + getReactiveAreaDensityTensor<T>(ccl, dims,
 * isovalue) (VolumeMeasures.cpp:303-335, generateBoundaryConnectedVolume in
 * VolumeSegmentation.cpp:66-90): tensor[d] (6 doubles, Dir order) = the area
 * of the pore space (voxels != 255) whose component touches face d.  The
 * solid/pore area of fast_reactive_area comes from the same pass into
 * *area_solid (nullable).  One labelling and one area pass for all seven.
 * Volumes of 4294967295 voxels or more are rejected (labels are 32-bit). */
FAST_API int fast_reactive_area_tensor(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, float isovalue,
                                       double *tensor, double *area_solid);

/* getVolumeAreaMesh(mask, false, mask.dim(), isovalue) (fastlib/src/volume/
 * VolumeSurface.cpp:38-68): the triangles of the same surface, 12 floats each
 * (vertices v0, v1, v2, then the unit face normal), in the reference's mesh
 * frame (voxel size 1/max(nx, ny, nz) on every axis, grid centred on the
 * origin), in cell order.  *ntri gets the count; triangles (host, capacity
 * triangles) may be NULL to ask for the count only.  `fast alpha --mesh`
 * writes them (of the volume zero-padded by one voxel) as an OBJ file. */
FAST_API int fast_reactive_area_mesh(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, float isovalue,
                                     float *triangles, uint64_t capacity, uint64_t *ntri);

/* The same on a DEVICE mask (stream as above; synchronised). */
FAST_API int fast_reactive_area_tensor_device(const uint8_t *d_mask, int64_t nx, int64_t ny, int64_t nz,
                                              float isovalue, double *tensor, double *area_solid, void *stream);

/* Message of the calling thread's last failure ("" if none). */
FAST_API const char *fast_last_error(void);

/* Library version string. */
FAST_API const char *fast_version(void);

/* ------------------------------------------------------------------------ */
/* Synthetic microstructures (the reference's VolumeGenerator uses an        */
/* unseedable process-global RNG, VolumeGenerator.cpp:14; these generators   */
/* are seeded and bit-identical across hosts).  255 = solid, 0 = pore        */
/* (VolumeGenerator.cpp:218).  Output is a host array of nx*ny*nz bytes.      */
/* ------------------------------------------------------------------------ */

/* Overlapping solid spheres of radius uniform in [r_min, r_max] voxels added
 * until the solid fraction reaches `solid_fraction`. */
FAST_API int fast_gen_spheres(uint8_t *out, int64_t nx, int64_t ny, int64_t nz, uint64_t seed,
                              double r_min, double r_max, double solid_fraction);

/* Randomly oriented solid ellipsoids (uniform random rotations) with
 * semi-axes (a, a*aspect, a*aspect), overlapping allowed, added until the
 * solid fraction is reached (stand-in for the reference's SA packer). */
FAST_API int fast_gen_ellipsoids(uint8_t *out, int64_t nx, int64_t ny, int64_t nz, uint64_t seed,
                                 double semi_major, double aspect, double solid_fraction);

#ifdef __cplusplus
}
#endif
#endif /* FASTTAU_H */
