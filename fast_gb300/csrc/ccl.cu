// 6-connected component labelling of a uint8 volume on the GPU, numbered as
// the reference numbers them (fastlib/src/cuda/VolumeCCL.cu:381-620
// VolumeCCL_Label, :753-818 VolumeCCL_BoundaryLabels;
// fastlib/src/volume/VolumeSegmentation.cpp:14-64):
//
//   * foreground = voxels whose value differs from `background`;
//   * label 0 = background; components are numbered 1..K in increasing order
//     of their smallest linear index (x fastest); num_labels = K + 1;
//   * boundary[d * num_labels + l] = 1 when label l > 0 has a voxel on face d
//     (Dir order: X_POS is x = nx-1, X_NEG is x = 0, ...); row 6 is the AND of
//     rows 0..5.
//
// The reference gets that numbering from span labels merged by atomicMin and a
// scan over root spans.  Here it comes from a union-find whose links always
// point from a larger to a smaller linear index, so the root of every tree is
// its component's minimum index; roots are then ranked by a two-level scan in
// linear-index order.  Passes:
//   1. rows: one warp per (y, z) row seeds parent[i] = first index of the
//      voxel's x-run (ballot + count-leading-zeros over 32-voxel chunks);
//   2. union: each foreground voxel joins its y-1 and z-1 neighbours, skipping
//      a join already implied through the x-1 voxel (both x-1 voxels
//      foreground); Rem's union with splicing, lock-free (compare-and-swap).
//      Every stored parent is a run start, so afterwards a voxel points at
//      a run start (its own or one joined to it);
//   3. starts: one warp per row; every run start that is a root counts
//      itself in its 8192-voxel chunk and sets its bit of a root bitmap,
//      every other run start is pointed straight at its root;
//   4. scan the chunk counts;
//   5. rank: one block per chunk numbers the chunk's roots from the bitmap;
//   6. relabel: labels[i] = label of parent[parent[i]] (the root: the run
//      start's parent), 0 on the background;
//   7. face bitmaps, 8. the all-faces AND.
// Every loop terminates: a find follows strictly decreasing indices, and a
// failed link continues from a strictly smaller index.
#include <cuda_runtime.h>
#include <stdint.h>

#include "fasttau.h"
#include "tau_errors.h"

namespace ft {
namespace {

constexpr uint32_t kNone = 0xFFFFFFFFu;  // parent of a background voxel
constexpr int kChunk = 8192;             // voxels per block in the ranking passes
constexpr int kRankThreads = 256;        // one root-bitmap word (32 voxels) per thread
static_assert(kChunk == kRankThreads * 32, "a rank block covers one chunk");

// Parent reads during the union and starts passes go through L1
// (ld.global.ca): a read may return a stale parent written earlier in the
// same pass by another SM, which is harmless.  Every value ever stored is a
// pointer to a smaller index of the same component, so a walk that follows
// stale pointers still ends at a root.  A stale "root" is caught by the
// linking compare-and-swap, whose old value the union continues from.  The next
// pass, after the kernel boundary, sees the final values.  The root of a
// large component is read by most finds; through L2 alone that one line
// would serialise them.
__device__ __forceinline__ uint32_t ld_par(const uint32_t *p, uint32_t i) { return __ldca(p + i); }

// Root of a's tree (no writes).
__device__ __forceinline__ uint32_t find_root(const uint32_t *par, uint32_t a)
{
    uint32_t p = ld_par(par, a);
    while (p != a) {
        a = p;
        p = ld_par(par, a);
    }
    return a;
}

// Joins the trees of x and y: Rem's union with splicing, concurrent form
// (links by compare-and-swap).  The node whose parent is larger moves up;
// before it does, its parent is swung to the other node's (smaller) parent,
// so paths shorten as unions proceed; the walk stops as soon as both nodes
// have the same parent, which for two voxels already in one component
// usually happens well below the root.  Invariants: a parent never exceeds
// its node (so a root is its tree's smallest index) and every stored parent
// is a run start (a voxel inside a run is never anyone's parent), which the
// starts and relabel passes rely on.  A link or splice that loses a race
// only fails its compare-and-swap; a failed link hands back the node's
// current parent, so a stale read cannot make the loop spin, and every
// step moves a node to a strictly smaller index.
__device__ void unite(uint32_t *par, uint32_t x, uint32_t y)
{
    uint32_t px = ld_par(par, x), py = ld_par(par, y);
    for (;;) {
        if (px == py) return;
        if (px < py) {
            uint32_t t = x;
            x = y;
            y = t;
            t = px;
            px = py;
            py = t;
        }
        // px > py
        if (x == px) {  // x is a root: hang it under y's parent
            const uint32_t old = atomicCAS(par + x, x, py);
            if (old == x) return;
            px = old;  // x got a parent meanwhile
            continue;
        }
        atomicCAS(par + x, px, py);  // splice; losing the race is harmless
        x = px;
        px = ld_par(par, x);
    }
}

// Pass 1: one warp per row.
__global__ void ccl_rows(const uint8_t *__restrict__ m, uint32_t *__restrict__ par, int nx, int64_t rows,
                         uint8_t bg)
{
    const int64_t row = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    if (row >= rows) return;
    const int lane = threadIdx.x & 31;
    const uint32_t base = (uint32_t)(row * nx);
    uint32_t carry_start = 0;
    uint32_t carry_fg = 0;
    for (int x0 = 0; x0 < nx; x0 += 32) {
        const int x = x0 + lane;
        const bool fg = x < nx && m[(int64_t)base + x] != bg;
        const uint32_t bfg = __ballot_sync(0xFFFFFFFFu, fg);
        const uint32_t prev = (bfg << 1) | carry_fg;  // bit l: voxel x0+l-1 is foreground
        const uint32_t bstart = bfg & ~prev;          // bit l: an x-run starts at x0+l
        const uint32_t upto = lane == 31 ? 0xFFFFFFFFu : ((2u << lane) - 1u);
        const uint32_t below = bstart & upto;
        const uint32_t start = below ? (uint32_t)(x0 + 31 - __clz(below)) : carry_start;
        if (x < nx) par[base + (uint32_t)x] = fg ? base + start : kNone;
        carry_fg = bfg >> 31;
        if (carry_fg) carry_start = bstart ? (uint32_t)(x0 + 31 - __clz(bstart)) : carry_start;
    }
}

// Pass 2: joins across y and z.
__global__ void ccl_union(const uint8_t *__restrict__ m, uint32_t *par, int nx, int ny, int nz, uint8_t bg)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= nx || y >= ny) return;
    const uint32_t sy = (uint32_t)nx, sz = (uint32_t)nx * (uint32_t)ny;
    for (int z = blockIdx.z; z < nz; z += gridDim.z) {
        const uint32_t i = (uint32_t)x + sy * (uint32_t)y + sz * (uint32_t)z;
        // The six mask bytes are loaded together (one round trip), not one
        // behind the other's branch.
        const uint8_t c = m[i];
        const uint8_t l = x > 0 ? m[i - 1] : bg;
        const uint8_t u = y > 0 ? m[i - sy] : bg;
        const uint8_t ul = (x > 0 && y > 0) ? m[i - 1 - sy] : bg;
        const uint8_t b = z > 0 ? m[i - sz] : bg;
        const uint8_t bl = (x > 0 && z > 0) ? m[i - 1 - sz] : bg;
        if (c == bg) continue;
        const bool left = l != bg;
        if (u != bg && !(left && ul != bg)) unite(par, i, i - sy);
        if (b != bg && !(left && bl != bg)) unite(par, i, i - sz);
    }
}

// Pass 3: run starts.  A root (a start whose parent is itself) counts
// itself in its chunk and sets its bit in the root bitmap; another start
// gets its root as parent.  The other voxels of a run keep the start.
__global__ void ccl_starts(const uint8_t *__restrict__ m, uint32_t *par, int nx, int64_t rows, uint8_t bg,
                           uint32_t *chunk_cnt, uint32_t *root_bits)
{
    const int64_t row = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    if (row >= rows) return;
    const int lane = threadIdx.x & 31;
    const uint32_t base = (uint32_t)(row * nx);
    bool carry = false;  // voxel x0 - 1 is foreground
    for (int x0 = 0; x0 < nx; x0 += 32) {
        const int x = x0 + lane;
        const bool fg = x < nx && m[base + x] != bg;
        const unsigned fgm = __ballot_sync(0xFFFFFFFFu, fg);
        const bool prev = lane == 0 ? carry : ((fgm >> (lane - 1)) & 1u) != 0;
        carry = (fgm >> 31) & 1u;
        if (fg && !prev) {
            const uint32_t i = base + (uint32_t)x;
            const uint32_t p = ld_par(par, i);
            if (p == i) {
                atomicAdd(chunk_cnt + i / (uint32_t)kChunk, 1u);
                atomicOr(root_bits + (i >> 5), 1u << (i & 31u));
            } else {
                const uint32_t r = find_root(par, p);
                if (r != p) par[i] = r;
            }
        }
    }
}

// Exclusive block scan of one value per thread (kRankThreads threads).
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *s_warp, uint32_t &total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) s_warp[w] = inc;
    __syncthreads();
    if (w == 0) {
        uint32_t s = lane < kRankThreads / 32 ? s_warp[lane] : 0u;
        uint32_t si = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, si, o);
            if (lane >= o) si += t;
        }
        if (lane < kRankThreads / 32) s_warp[lane] = si - s;  // exclusive warp offsets
        if (lane == kRankThreads / 32 - 1) s_warp[kRankThreads / 32] = si;
    }
    __syncthreads();
    total = s_warp[kRankThreads / 32];
    return s_warp[w] + inc - v;
}

// Pass 4: exclusive scan of the chunk counts in place (one block of 1024
// threads, each summing a contiguous slice); cnt[nchunks] = number of roots.
__global__ void __launch_bounds__(1024) ccl_scan_chunks(uint32_t *cnt, uint32_t nchunks)
{
    __shared__ uint32_t s[1024];
    const uint32_t per = (nchunks + 1023u) / 1024u;
    const uint32_t a = threadIdx.x * per, b = min(a + per, nchunks);
    uint32_t sum = 0;
    for (uint32_t k = a; k < b; k++) sum += cnt[k];
    s[threadIdx.x] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {  // Hillis-Steele inclusive scan
        const uint32_t t = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0u;
        __syncthreads();
        s[threadIdx.x] += t;
        __syncthreads();
    }
    uint32_t run = s[threadIdx.x] - sum;
    for (uint32_t k = a; k < b; k++) {
        const uint32_t c = cnt[k];
        cnt[k] = run;
        run += c;
    }
    if (threadIdx.x == 1023) cnt[nchunks] = s[1023];
}

// Pass 5: label of every root = 1 + its rank.  One block per chunk, one
// bitmap word (32 voxels) per thread.
__global__ void __launch_bounds__(kRankThreads) ccl_rank(const uint32_t *__restrict__ root_bits, uint32_t nwords,
                                                         const uint32_t *__restrict__ chunk_off, uint32_t *labels)
{
    __shared__ uint32_t s_warp[kRankThreads / 32 + 1];
    const uint32_t w = blockIdx.x * (uint32_t)kRankThreads + threadIdx.x;
    uint32_t bits = w < nwords ? root_bits[w] : 0u;
    uint32_t total;
    uint32_t r = chunk_off[blockIdx.x] + block_exclusive_scan((uint32_t)__popc(bits), s_warp, total) + 1u;
    while (bits) {
        const uint32_t k = (uint32_t)(__ffs(bits) - 1);
        labels[w * 32u + k] = r++;
        bits &= bits - 1u;
    }
}

// Pass 6: every other voxel: 0 on the background, else the label of its
// root, which is its parent's parent (a run start points at its root, a
// root at itself).  Roots were labelled by pass 5 and are not written here.
// Four voxels a thread per step, their loads issued together.  A root's
// label is read through the non-coherent L1 path: one component can own
// most of the volume, and its root's label, read by every one of its
// voxels, would otherwise be one L2 line hit by every SM.  Root entries
// were written by the rank pass and are not written here (only non-root
// entries are), so the cached values are current.
__global__ void ccl_relabel(const uint32_t *__restrict__ par, uint32_t n, uint32_t *labels)
{
    constexpr int U = 4;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += U * stride) {
        uint32_t p[U], r[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const uint64_t i = i0 + u * stride;
            p[u] = i < n ? __ldg(par + i) : kNone;
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const uint64_t i = i0 + u * stride;
            r[u] = (p[u] != kNone && p[u] != i) ? __ldg(par + p[u]) : kNone;
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const uint64_t i = i0 + u * stride;
            if (i >= n) break;
            if (p[u] == kNone) labels[i] = 0u;
            else if (r[u] != kNone) labels[i] = __ldg(labels + r[u]);
        }
    }
}

// Pass 7: the six face bitmaps.  Face d (Dir order) of the volume, flattened
// over the two secondary axes; faces are concatenated in d order.
__global__ void ccl_faces(const uint32_t *labels, int nx, int ny, int nz, uint32_t num_labels, uint8_t *bnd)
{
    const int64_t fxy = (int64_t)nx * ny, fxz = (int64_t)nx * nz, fyz = (int64_t)ny * nz;
    const int64_t sizes[3] = {fyz, fxz, fxy};  // face area by primary axis
    const int64_t total = 2 * (fyz + fxz + fxy);
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        int d = 0;
        int64_t u = t;
        while (u >= sizes[d >> 1]) {
            u -= sizes[d >> 1];
            d++;
        }
        const int k = d >> 1;
        const bool pos = (d & 1) == 0;  // X_POS, Y_POS, Z_POS: the last plane
        int x, y, z;
        if (k == 0) { x = pos ? nx - 1 : 0; y = (int)(u % ny); z = (int)(u / ny); }
        else if (k == 1) { y = pos ? ny - 1 : 0; x = (int)(u % nx); z = (int)(u / nx); }
        else { z = pos ? nz - 1 : 0; x = (int)(u % nx); y = (int)(u / nx); }
        const uint32_t l = labels[(uint32_t)x + (uint32_t)nx * ((uint32_t)y + (uint32_t)ny * (uint32_t)z)];
        if (l > 0) bnd[(size_t)d * num_labels + l] = 1;
    }
}

// Pass 8: row 6 = AND of rows 0..5.
__global__ void ccl_all_faces(uint32_t num_labels, uint8_t *bnd)
{
    for (uint32_t l = blockIdx.x * blockDim.x + threadIdx.x; l < num_labels; l += gridDim.x * blockDim.x) {
        uint8_t all = 1;
        for (int d = 0; d < 6; d++) all &= bnd[(size_t)d * num_labels + l];
        bnd[(size_t)6 * num_labels + l] = all;
    }
}

#define CK(expr)                                                                                        \
    do {                                                                                                \
        cudaError_t e_ = (expr);                                                                        \
        if (e_ != cudaSuccess) return ft_fail(FAST_CUDA_ERROR, "%s: %s", #expr, cudaGetErrorString(e_)); \
    } while (0)

int check_dims(int64_t nx, int64_t ny, int64_t nz)
{
    if (nx <= 0 || ny <= 0 || nz <= 0) return ft_fail(FAST_BAD_ARG, "dimensions must be positive");
    if (nx > INT32_MAX || ny > INT32_MAX || nz > INT32_MAX) return ft_fail(FAST_BAD_ARG, "dimension too large");
    const double n = (double)nx * (double)ny * (double)nz;
    if (n >= 4294967295.0) return ft_fail(FAST_BAD_ARG, "labelling is limited to 4294967294 voxels");
    return FAST_OK;
}

// Scratch words of a labelling beside the parent array: the chunk counts
// (nchunks + 1) and the root bitmap (one bit per voxel).
size_t scratch_words(uint32_t n)
{
    const size_t nchunks = (n + kChunk - 1) / kChunk;
    return nchunks + 1 + nchunks * (kChunk / 32);
}

// Labels of d_mask into d_labels (device, N uint32) on `st`, using d_par
// (device, N uint32) and d_scr (device, scratch_words(N) uint32) as scratch.
int label_device(const uint8_t *d_mask, int64_t nx, int64_t ny, int64_t nz, uint8_t bg, uint32_t *d_labels,
                 uint32_t *d_par, uint32_t *d_scr, uint32_t *num_labels, cudaStream_t st)
{
    const uint32_t n = (uint32_t)(nx * ny * nz);
    const int64_t rows = ny * nz;
    const uint32_t nchunks = (n + kChunk - 1) / kChunk;
    uint32_t *d_cnt = d_scr, *d_bits = d_scr + nchunks + 1;
    CK(cudaMemsetAsync(d_scr, 0, scratch_words(n) * 4, st));
    ccl_rows<<<(unsigned)((rows + 7) / 8), 256, 0, st>>>(d_mask, d_par, (int)nx, rows, bg);
    const dim3 ub(32, 8, 1);
    // At most 128 grid layers in z, each thread striding over nz/128 planes:
    // 1024^3 labelling 18.2 ms against 19.0 with one layer per plane (24.5
    // with 32 layers, 35.5 with 8: fewer threads, fewer joins in flight).
    const dim3 ug((unsigned)((nx + 31) / 32), (unsigned)((ny + 7) / 8), (unsigned)(nz < 128 ? nz : 128));
    ccl_union<<<ug, ub, 0, st>>>(d_mask, d_par, (int)nx, (int)ny, (int)nz, bg);
    ccl_starts<<<(unsigned)((rows + 7) / 8), 256, 0, st>>>(d_mask, d_par, (int)nx, rows, bg, d_cnt, d_bits);
    ccl_scan_chunks<<<1, 1024, 0, st>>>(d_cnt, nchunks);
    ccl_rank<<<nchunks, kRankThreads, 0, st>>>(d_bits, (n + 31) / 32, d_cnt, d_labels);
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    ccl_relabel<<<(unsigned)sms * 8u, 256, 0, st>>>(d_par, n, d_labels);
    CK(cudaGetLastError());
    uint32_t roots = 0;
    CK(cudaMemcpyAsync(&roots, d_cnt + nchunks, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    *num_labels = roots + 1u;
    return FAST_OK;
}

// Face bitmaps of device labels into the host buffer `boundary`.
int boundary_device(const uint32_t *d_labels, int64_t nx, int64_t ny, int64_t nz, uint32_t num_labels,
                    uint8_t *boundary, cudaStream_t st)
{
    const size_t bytes = (size_t)7 * num_labels;
    uint8_t *d_bnd = nullptr;
    CK(cudaMallocAsync((void **)&d_bnd, bytes, st));
    cudaError_t e = cudaMemsetAsync(d_bnd, 0, bytes, st);
    if (e == cudaSuccess) {
        ccl_faces<<<1024, 256, 0, st>>>(d_labels, (int)nx, (int)ny, (int)nz, num_labels, d_bnd);
        ccl_all_faces<<<(num_labels + 255) / 256 < 4096 ? (num_labels + 255) / 256 : 4096, 256, 0, st>>>(
            num_labels, d_bnd);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(boundary, d_bnd, bytes, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d_bnd, st);
    const cudaError_t e2 = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return ft_fail(FAST_CUDA_ERROR, "boundary labels: %s", cudaGetErrorString(e));
    return FAST_OK;
}

int label_common(const uint8_t *d_mask, int64_t nx, int64_t ny, int64_t nz, uint8_t bg, uint32_t *d_labels,
                 uint32_t *num_labels, uint8_t *boundary, uint64_t boundary_cap, cudaStream_t st)
{
    const uint32_t n = (uint32_t)(nx * ny * nz);
    int dev = 0;
    CK(cudaGetDevice(&dev));
    ft_retain_pool_memory(dev);
    uint32_t *d_par = nullptr, *d_cnt = nullptr;
    CK(cudaMallocAsync((void **)&d_par, (size_t)n * 4, st));
    cudaError_t e = cudaMallocAsync((void **)&d_cnt, scratch_words(n) * 4, st);
    if (e != cudaSuccess) {
        cudaFreeAsync(d_par, st);
        return ft_fail(FAST_NOMEM, "labelling scratch: %s", cudaGetErrorString(e));
    }
    int s = label_device(d_mask, nx, ny, nz, bg, d_labels, d_par, d_cnt, num_labels, st);
    cudaFreeAsync(d_par, st);
    cudaFreeAsync(d_cnt, st);
    if (s == FAST_OK && boundary) {
        if (boundary_cap < (uint64_t)7 * *num_labels)
            s = ft_fail(FAST_BAD_ARG, "boundary buffer holds %llu bytes, 7 x %u needed",
                        (unsigned long long)boundary_cap, *num_labels);
        else
            s = boundary_device(d_labels, nx, ny, nz, *num_labels, boundary, st);
    }
    return s;
}

}  // namespace
}  // namespace ft

using namespace ft;

extern "C" {

FAST_API int fast_ccl_label_device(const uint8_t *d_mask, int64_t nx, int64_t ny, int64_t nz, uint8_t background,
                                   uint32_t *d_labels, uint32_t *num_labels, uint8_t *boundary,
                                   uint64_t boundary_cap, void *stream)
{
    ft_clear_error();
    if (!d_mask || !d_labels || !num_labels) return ft_fail(FAST_BAD_ARG, "null argument");
    int s = check_dims(nx, ny, nz);
    if (s != FAST_OK) return s;
    cudaStream_t st = (cudaStream_t)stream;
    s = label_common(d_mask, nx, ny, nz, background, d_labels, num_labels, boundary, boundary_cap, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    if (s == FAST_OK && e != cudaSuccess) s = ft_fail(FAST_CUDA_ERROR, "labelling: %s", cudaGetErrorString(e));
    return s;
}

FAST_API int fast_ccl_boundary_device(const uint32_t *d_labels, int64_t nx, int64_t ny, int64_t nz,
                                      uint32_t num_labels, uint8_t *boundary, void *stream)
{
    ft_clear_error();
    if (!d_labels || !boundary || num_labels == 0) return ft_fail(FAST_BAD_ARG, "null argument or no labels");
    const int s = check_dims(nx, ny, nz);
    if (s != FAST_OK) return s;
    return boundary_device(d_labels, nx, ny, nz, num_labels, boundary, (cudaStream_t)stream);
}

FAST_API int fast_ccl_label(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, uint8_t background,
                            uint32_t *labels, uint32_t *num_labels, uint8_t *boundary, uint64_t boundary_cap)
{
    ft_clear_error();
    if (!mask) return ft_fail(FAST_NO_HOST_DATA, "mask must be allocated");
    if (!num_labels) return ft_fail(FAST_BAD_ARG, "num_labels is NULL");
    int s = check_dims(nx, ny, nz);
    if (s != FAST_OK) return s;
    const size_t n = (size_t)(nx * ny * nz);
    cudaStream_t st = nullptr;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    uint8_t *d_mask = nullptr;
    uint32_t *d_labels = nullptr;
    cudaError_t e = cudaMallocAsync((void **)&d_mask, n, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&d_labels, n * 4, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_mask, mask, n, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
        s = ft_fail(FAST_NOMEM, "labelling buffers: %s", cudaGetErrorString(e));
    } else {
        s = label_common(d_mask, nx, ny, nz, background, d_labels, num_labels, boundary, boundary_cap, st);
        if (s == FAST_OK && labels) {
            e = cudaMemcpyAsync(labels, d_labels, n * 4, cudaMemcpyDeviceToHost, st);
            if (e != cudaSuccess) s = ft_fail(FAST_CUDA_ERROR, "labels download: %s", cudaGetErrorString(e));
        }
    }
    if (d_mask) cudaFreeAsync(d_mask, st);
    if (d_labels) cudaFreeAsync(d_labels, st);
    e = cudaStreamSynchronize(st);
    if (s == FAST_OK && e != cudaSuccess) s = ft_fail(FAST_CUDA_ERROR, "labelling: %s", cudaGetErrorString(e));
    cudaStreamDestroy(st);
    return s;
}

}  // extern "C"
