// Reactive area density ("alpha"): the marching-cubes area of a binary
// volume's 0.5 iso-surface (getReactiveAreaDensity, fastlib/src/volume/
// VolumeMeasures.cpp:294-301; getVolumeArea, fastlib/src/volume/
// VolumeSurface.cpp:10-36; the per-cell kernel ___generateTrianglesSurfaceArea,
// fastlib/src/cuda/VolumeSurface.cu:198-262) and its per-direction form over
// the pore space connected to each face (getReactiveAreaDensityTensor,
// VolumeMeasures.cpp:303-335, on generateBoundaryConnectedVolume,
// fastlib/src/volume/VolumeSegmentation.cpp:66-90).
//
// What the reference computes, restated:
//   * one cell per voxel position (i, j, k) in [0, n)^3; its corners are the
//     grid points (i..i+1, j..j+1, k..k+1);
//   * a grid point's value is the volume's texture read there: normalized
//     coordinates, linear filtering, clamp addressing, uint8 read as v/255
//     (fastlib/src/utility/DataPtr.cpp:565-595).  At the grid point g/n the
//     filter weights are 1/2, so the value is the mean of the 2x2x2 voxels
//     (g-1..g per axis, clamped to the volume): a multiple of 1/8 for a
//     0/255 volume;
//   * a corner is "below" when its value < isovalue (getCubeIndex); vertices
//     are interpolated on the cut edges, vertex = p0 + t (p1 - p0),
//     t = (iso - f0) / (f1 - f0); positions are in normalized units,
//     p = (i/nx, j/ny, k/nz) + corner offsets of 1/n per axis;
//   * triangle area = |(v1 - v0) x (v2 - v0)| / 2 in float, summed per cell
//     in double, then over all cells.
//
// The engine evaluates all of it in one pass over the volume and, for the
// per-direction form, over the CCL labels at the same time: each voxel gets
// a 7-bit code (bit d: its pore component touches face d; bit 6: the voxel
// is solid), expanded to one 4-bit lane per bit, so adding the eight voxels
// around a grid point counts all seven fields at once.  A block owns a 32x8
// column of cells and walks a z-slab, keeping a ring of three expanded voxel
// planes in shared memory; a cell whose eight corner words are equal has no
// surface in any field and costs nothing more.  Reductions are per block
// then in a fixed order, so results are run-to-run identical.
//
// The triangulation table is generated here, not copied: for each of the 256
// corner patterns the cut edges of every cube face are joined in pairs (on a
// face with four cut edges, the two "below" corners are kept apart), the
// pairs close into loops, and each loop is fanned from its first edge.  Two
// cells sharing a face join that face's cut edges the same way, so the
// surface is closed.  The reference uses a fixed published table; on cells
// where the loop is not planar, or a face is ambiguous, its triangles and so
// its area differ slightly from these.
//
// The reference's texture unit quantises filter weights to 1/256; at the
// grid points the weights are 1/2 (exact) whenever 1/n is exact (n a power of
// two) and within 1/512 of 1/2 otherwise.  The engine uses exactly 1/2.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include "fasttau.h"
#include "tau_errors.h"

namespace {

// A block is 32 x 8 threads; each thread owns two cells in y (rows ty and
// ty + 8), so a block covers 32 x 16 cells.
constexpr int TX = 32, TYT = 8, NT = TX * TYT, CY = 2, TY = TYT * CY;
constexpr int PW = TX + 2, PH = TY + 2;  // expanded plane tile with a one-voxel rim
constexpr int NLOAD = (PW * PH + NT - 1) / NT;
constexpr int kMaxSlab = 32;             // z-slab depth limit (5 bits in a queue item)
constexpr int kMaxTri = 5;
constexpr int kFields = 7;               // six face-connected pore fields + the solid field

struct McTable {
    uint8_t ntri[256];
    uint8_t edge[256][3 * kMaxTri];
};
static_assert(sizeof(McTable) == 4096, "table is copied as 256 x 16 bytes");

// Corner c of a cell sits at offset (c&1 ^ c>>1&1, c>>1&1, c>>2) in the
// reference's order: 0 (0,0,0) 1 (1,0,0) 2 (1,1,0) 3 (0,1,0), 4..7 the same at
// z + 1.  Edge e joins corners kEdgeA[e] and kEdgeB[e] (the vertexInterp
// order of the per-cell kernel).
constexpr int kEdgeA[12] = {0, 1, 2, 3, 4, 5, 6, 7, 0, 1, 2, 3};
constexpr int kEdgeB[12] = {1, 2, 3, 0, 5, 6, 7, 4, 4, 5, 6, 7};
constexpr int kFaces[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4}, {3, 2, 6, 7}, {0, 3, 7, 4}, {1, 2, 6, 5}};

int edge_between(int a, int b)
{
    for (int e = 0; e < 12; e++)
        if ((kEdgeA[e] == a && kEdgeB[e] == b) || (kEdgeA[e] == b && kEdgeB[e] == a)) return e;
    return -1;
}

McTable build_table()
{
    McTable T;
    memset(&T, 0, sizeof(T));
    for (int cs = 0; cs < 256; cs++) {
        int nb[12][2], deg[12] = {0};
        auto link = [&](int a, int b) {
            nb[a][deg[a]++] = b;
            nb[b][deg[b]++] = a;
        };
        for (const auto &f : kFaces) {
            int E[4];
            bool cut[4], below[4];
            int ncut = 0;
            for (int q = 0; q < 4; q++) {
                E[q] = edge_between(f[q], f[(q + 1) & 3]);
                below[q] = (cs >> f[q]) & 1;
            }
            for (int q = 0; q < 4; q++) {
                cut[q] = below[q] != below[(q + 1) & 3];
                ncut += cut[q];
            }
            if (ncut == 2) {
                int a = -1, b = -1;
                for (int q = 0; q < 4; q++)
                    if (cut[q]) (a < 0 ? a : b) = E[q];
                link(a, b);
            } else if (ncut == 4) {
                if (below[0]) {  // corners 0 and 2 below: cut around each
                    link(E[3], E[0]);
                    link(E[1], E[2]);
                } else {         // corners 1 and 3 below
                    link(E[0], E[1]);
                    link(E[2], E[3]);
                }
            }
        }
        bool seen[12] = {false};
        int nt = 0;
        for (int e = 0; e < 12; e++) {
            if (deg[e] == 0 || seen[e]) continue;
            int loop[12], len = 0, prev = e, cur = nb[e][0] < nb[e][1] ? nb[e][0] : nb[e][1];
            loop[len++] = e;
            seen[e] = true;
            while (cur != e) {
                loop[len++] = cur;
                seen[cur] = true;
                const int next = nb[cur][0] == prev ? nb[cur][1] : nb[cur][0];
                prev = cur;
                cur = next;
            }
            for (int q = 1; q + 1 < len; q++) {
                T.edge[cs][3 * nt + 0] = (uint8_t)loop[0];
                T.edge[cs][3 * nt + 1] = (uint8_t)loop[q];
                T.edge[cs][3 * nt + 2] = (uint8_t)loop[q + 1];
                nt++;
            }
        }
        T.ntri[cs] = (uint8_t)nt;
    }
    return T;
}

struct AlphaArgs {
    const uint8_t *mask;
    const uint32_t *labels;      // nullptr: the solid field alone
    const uint8_t *label_bits;   // per label: bit d = touches face d
    const McTable *table;
    double *partials;            // [blocks][kFields]
    uint32_t *bad;               // set when a voxel is neither 0 nor 255
    int nx, ny, nz, zc, tiles_x, tiles_y;
    float iso, vx, vy, vz;       // isovalue, voxel size 1/n per axis
    int thr;                     // corner below <=> count < thr (count = 8 x value)
};

// kEdgeA / kEdgeB packed one nibble per edge, for device code.
__device__ __forceinline__ int edge_a(int e) { return (int)((0x321076543210ULL >> (4 * e)) & 15u); }
__device__ __forceinline__ int edge_b(int e) { return (int)((0x765447650321ULL >> (4 * e)) & 15u); }

__device__ __forceinline__ uint32_t spread7(uint32_t c)
{
    return (c & 1u) | (c & 2u) << 3 | (c & 4u) << 6 | (c & 8u) << 9 | (c & 16u) << 12 | (c & 32u) << 15 |
           (c & 64u) << 18;
}

// One expanded voxel plane into shared memory; off[r] = the clamped (x, y)
// offset of this thread's r-th tile entry (fixed for the block).
template <bool LABELS>
__device__ __forceinline__ void load_plane(const AlphaArgs &A, uint32_t *dst, const int64_t off[NLOAD], int p)
{
    const int pz = p < 0 ? 0 : (p >= A.nz ? A.nz - 1 : p);
    const int64_t base = (int64_t)pz * A.nx * A.ny;
#pragma unroll
    for (int r = 0; r < NLOAD; r++) {
        const int e = threadIdx.x + r * NT;
        if (e < PW * PH) {
            const int64_t idx = base + off[r];
            const uint32_t m = A.mask[idx];
            if (m != 0 && m != 255) *A.bad = 1;
            uint32_t code;
            if (LABELS)
                code = spread7((m ? 64u : 0u) | A.label_bits[A.labels[idx]]);
            else
                code = m ? 1u : 0u;
            dst[e] = code;
        }
    }
}

// Float arithmetic as the reference's helpers (lerp, cross, length) write it,
// with no fused multiply-add so that every cell's area is reproducible.
__device__ __forceinline__ float lerp1(float a, float b, float t) { return __fadd_rn(a, __fmul_rn(t, __fsub_rn(b, a))); }

// Area of triangle `t` of corner pattern `cube` in the cell whose low corner
// is (px, py, pz) and high corner (qx, qy, qz); cnt = 8 corner counts
// (4 bits each, corner c at bits 4c).
__device__ __forceinline__ float triangle_area(const McTable &T, int cube, int t, uint32_t cnt, float iso, float px,
                                               float py, float pz, float qx, float qy, float qz)
{
    float v[3][3];
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const int e = T.edge[cube][3 * t + q];
        const int ca = edge_a(e), cb = edge_b(e);
        const float fa = __fmul_rn((float)((cnt >> (4 * ca)) & 15u), 0.125f);
        const float fb = __fmul_rn((float)((cnt >> (4 * cb)) & 15u), 0.125f);
        const int axa = (ca & 1) ^ ((ca >> 1) & 1), aya = (ca >> 1) & 1, aza = ca >> 2;
        const int axb = (cb & 1) ^ ((cb >> 1) & 1), ayb = (cb >> 1) & 1, azb = cb >> 2;
        const float x0 = axa ? qx : px, y0 = aya ? qy : py, z0 = aza ? qz : pz;
        const float x1 = axb ? qx : px, y1 = ayb ? qy : py, z1 = azb ? qz : pz;
        if (fa == fb) {
            v[q][0] = x0;
            v[q][1] = y0;
            v[q][2] = z0;
        } else {
            const float tt = __fdiv_rn(__fsub_rn(iso, fa), __fsub_rn(fb, fa));
            v[q][0] = lerp1(x0, x1, tt);
            v[q][1] = lerp1(y0, y1, tt);
            v[q][2] = lerp1(z0, z1, tt);
        }
    }
    const float ax = __fsub_rn(v[1][0], v[0][0]), ay = __fsub_rn(v[1][1], v[0][1]), az = __fsub_rn(v[1][2], v[0][2]);
    const float bx = __fsub_rn(v[2][0], v[0][0]), by = __fsub_rn(v[2][1], v[0][1]), bz = __fsub_rn(v[2][2], v[0][2]);
    const float cx = __fsub_rn(__fmul_rn(ay, bz), __fmul_rn(az, by));
    const float cy = __fsub_rn(__fmul_rn(az, bx), __fmul_rn(ax, bz));
    const float cz = __fsub_rn(__fmul_rn(ax, by), __fmul_rn(ay, bx));
    const float d = __fadd_rn(__fadd_rn(__fmul_rn(cx, cx), __fmul_rn(cy, cy)), __fmul_rn(cz, cz));
    return __fmul_rn(__fsqrt_rn(d), 0.5f);
}

// Counts of field f at the 8 corners, corner c at bits 4c.
__device__ __forceinline__ uint32_t field_counts(const uint32_t W[8], int f)
{
    uint32_t c = 0;
#pragma unroll
    for (int q = 0; q < 8; q++) c |= ((W[q] >> (4 * f)) & 15u) << (4 * q);
    return c;
}

__device__ __forceinline__ int cube_of(uint32_t cnt, int thr)
{
    int cube = 0;
#pragma unroll
    for (int q = 0; q < 8; q++) cube |= (int)(((cnt >> (4 * q)) & 15u) < (uint32_t)thr) << q;
    return cube;
}

// Triangles wait in a shared queue so that all lanes compute areas at once:
// a cell with a surface is rare and has one to five triangles per field, so
// evaluating them in the cell's own lane would leave most of the warp idle.
// Queue positions come from a block-wide exclusive scan (fixed order), and
// item q is always done by thread q mod NT, so the double sums are the same
// on every run.
constexpr int QCAP = 2048;

// Both passes are held to 64 registers (4 blocks per SM; the seven-field
// one spills a few hundred bytes): their memory waits want the warps more
// than the registers (1024^3: seven fields 62.9 ms at 128 registers and 2
// blocks, 61.3 at 3, 58.7 at 4; one field 16.1 ms at 75 registers and 3
// blocks, 14.7 at 4, 15.4 at 5).
template <bool LABELS>
__global__ void __launch_bounds__(NT, 4) alpha_kernel(AlphaArgs A)
{
    __shared__ uint32_t s_w[3][PH * PW];
    __shared__ McTable s_tab;
    __shared__ uint2 s_q[QCAP];     // x: corner counts, y: tx | cy << 5 | kk << 9 | fields << 14 | t << 21 | cube << 24
    __shared__ int s_warp[NT / 32];
    __shared__ double s_red[kFields][NT / 32];
    constexpr int NF = LABELS ? kFields : 1;

    reinterpret_cast<uint4 *>(&s_tab)[threadIdx.x] = reinterpret_cast<const uint4 *>(A.table)[threadIdx.x];

    const int tiles_xy = A.tiles_x * A.tiles_y;
    const int bz = blockIdx.x / tiles_xy;
    const int rem = blockIdx.x - bz * tiles_xy;
    const int by = rem / A.tiles_x, bx = rem - by * A.tiles_x;
    const int i0 = bx * TX, j0 = by * TY, k0 = bz * A.zc;
    const int k1 = min(k0 + A.zc, A.nz);
    const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    bool active[CY];
#pragma unroll
    for (int c = 0; c < CY; c++) active[c] = (i0 + tx) < A.nx && (j0 + ty + TYT * c) < A.ny;

    int64_t off[NLOAD];
#pragma unroll
    for (int r = 0; r < NLOAD; r++) {
        const int e = threadIdx.x + r * NT;
        const int ly = e / PW, lx = e - ly * PW;
        int gx = i0 - 1 + lx, gy = j0 - 1 + ly;
        gx = gx < 0 ? 0 : (gx >= A.nx ? A.nx - 1 : gx);
        gy = gy < 0 ? 0 : (gy >= A.ny ? A.ny - 1 : gy);
        off[r] = (int64_t)gy * A.nx + gx;
    }

    double acc[NF];
#pragma unroll
    for (int f = 0; f < NF; f++) acc[f] = 0.0;

    auto flush = [&](int n) {
        __syncthreads();
        for (int q = threadIdx.x; q < n; q += NT) {
            const uint2 it = s_q[q];
            const int ctx = it.y & 31, cy = (it.y >> 5) & 15, kk = (it.y >> 9) & 31;
            const int fields = (it.y >> 14) & 127, t = (it.y >> 21) & 7, cube = (it.y >> 24) & 255;
            const float px = __fmul_rn(A.vx, (float)(i0 + ctx)), py = __fmul_rn(A.vy, (float)(j0 + cy));
            const float pz = __fmul_rn(A.vz, (float)(k0 + kk));
            const float a = triangle_area(s_tab, cube, t, it.x, A.iso, px, py, pz, __fadd_rn(px, A.vx),
                                          __fadd_rn(py, A.vy), __fadd_rn(pz, A.vz));
#pragma unroll
            for (int g = 0; g < NF; g++)
                if ((fields >> g) & 1) acc[g] += (double)a;
        }
        __syncthreads();
    };

    load_plane<LABELS>(A, s_w[(k0 + 2) % 3], off, k0 - 1);
    load_plane<LABELS>(A, s_w[k0 % 3], off, k0);
    __syncthreads();
    // S[c][a + 2b] = sum of the 2x2 voxels around grid point (i + a, j + b)
    // of cell row c, in one plane.
    auto plane_sums = [&](int p, uint32_t S[CY][4]) {
        const uint32_t *w = s_w[(p + 3) % 3];
#pragma unroll
        for (int c = 0; c < CY; c++) {
            const int r0 = (ty + TYT * c) * PW + tx;
#pragma unroll
            for (int b = 0; b < 2; b++)
#pragma unroll
                for (int a = 0; a < 2; a++)
                    S[c][a + 2 * b] = w[r0 + b * PW + a] + w[r0 + b * PW + a + 1] + w[r0 + (b + 1) * PW + a] +
                                      w[r0 + (b + 1) * PW + a + 1];
        }
    };
    uint32_t Sp[CY][4], Sc[CY][4], Sn[CY][4];
    plane_sums(k0 - 1, Sp);
    plane_sums(k0, Sc);

    int queued = 0;  // block-uniform
    for (int k = k0; k < k1; k++) {
        __syncthreads();  // the slot of plane k - 2 is free
        load_plane<LABELS>(A, s_w[(k + 1) % 3], off, k + 1);
        __syncthreads();
        plane_sums(k + 1, Sn);
        // Corner counts per cell and field; fields with equal counts share
        // their triangles (queued once with the set of fields they serve).
        uint32_t cnt[CY][NF];
        int mine_c[CY];
        int mine = 0;
#pragma unroll
        for (int c = 0; c < CY; c++) {
            uint32_t W[8];
            W[0] = Sp[c][0] + Sc[c][0];
            W[1] = Sp[c][1] + Sc[c][1];
            W[2] = Sp[c][3] + Sc[c][3];
            W[3] = Sp[c][2] + Sc[c][2];
            W[4] = Sc[c][0] + Sn[c][0];
            W[5] = Sc[c][1] + Sn[c][1];
            W[6] = Sc[c][3] + Sn[c][3];
            W[7] = Sc[c][2] + Sn[c][2];
            bool flat = true;
#pragma unroll
            for (int q = 1; q < 8; q++) flat &= W[q] == W[0];
            mine_c[c] = 0;
#pragma unroll
            for (int f = 0; f < NF; f++) cnt[c][f] = 0;
            if (active[c] && !flat) {
#pragma unroll
                for (int f = 0; f < NF; f++) cnt[c][f] = field_counts(W, f);
#pragma unroll
                for (int f = 0; f < NF; f++) {
                    bool dup = false;
#pragma unroll
                    for (int g = 0; g < f; g++) dup |= cnt[c][g] == cnt[c][f];
                    if (!dup) mine_c[c] += s_tab.ntri[cube_of(cnt[c][f], A.thr)];
                }
            }
            mine += mine_c[c];
        }
        // Block-wide exclusive scan of the triangle counts.
        int inc = mine;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += v;
        }
        if (lane == 31) s_warp[warp] = inc;
        __syncthreads();
        int before = 0, total = 0;
#pragma unroll
        for (int w = 0; w < NT / 32; w++) {
            const int v = s_warp[w];
            before += w < warp ? v : 0;
            total += v;
        }
        const int off0 = before + inc - mine;
        for (int base = 0; base < total; base += QCAP) {
            const int chunk = min(total - base, QCAP);
            if (queued + chunk > QCAP) {
                flush(queued);
                queued = 0;
            }
            if (mine && off0 + mine > base && off0 < base + chunk) {
                int idx = off0;
#pragma unroll
                for (int c = 0; c < CY; c++) {
                    if (!mine_c[c]) continue;
#pragma unroll
                    for (int f = 0; f < NF; f++) {
                        bool dup = false;
                        uint32_t fields = 0;
#pragma unroll
                        for (int g = 0; g < NF; g++) {
                            dup |= g < f && cnt[c][g] == cnt[c][f];
                            fields |= (uint32_t)(g >= f && cnt[c][g] == cnt[c][f]) << g;
                        }
                        if (dup) continue;
                        const int cube = cube_of(cnt[c][f], A.thr);
                        const int nt = s_tab.ntri[cube];
                        const uint32_t meta = (uint32_t)tx | (uint32_t)(ty + TYT * c) << 5 | (uint32_t)(k - k0) << 9 |
                                              fields << 14 | (uint32_t)cube << 24;
                        for (int t = 0; t < nt; t++, idx++) {
                            if (idx >= base && idx < base + chunk)
                                s_q[queued + idx - base] = make_uint2(cnt[c][f], meta | (uint32_t)t << 21);
                        }
                    }
                }
            }
            queued += chunk;
        }
#pragma unroll
        for (int c = 0; c < CY; c++)
#pragma unroll
            for (int q = 0; q < 4; q++) {
                Sp[c][q] = Sc[c][q];
                Sc[c][q] = Sn[c][q];
            }
    }
    flush(queued);

    // Block sums in a fixed order.
#pragma unroll
    for (int f = 0; f < NF; f++) {
        double v = acc[f];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) s_red[f][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < NF) {
        double s = 0.0;
        for (int w = 0; w < NT / 32; w++) s += s_red[threadIdx.x][w];
        A.partials[(size_t)blockIdx.x * kFields + threadIdx.x] = s;
    }
}

// One block sums the per-block partials of every field in a fixed order.
__global__ void __launch_bounds__(NT) alpha_sum_kernel(const double *partials, int nblocks, double *out)
{
    __shared__ double s[NT];
    for (int f = 0; f < kFields; f++) {
        double v = 0.0;
        for (int b = threadIdx.x; b < nblocks; b += NT) v += partials[(size_t)b * kFields + f];
        s[threadIdx.x] = v;
        __syncthreads();
        for (int w = NT / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[f] = s[0];
        __syncthreads();
    }
}

std::once_flag g_table_once;
McTable g_table;

int check_args(int64_t nx, int64_t ny, int64_t nz, float iso)
{
    if (nx <= 0 || ny <= 0 || nz <= 0) return ft_fail(FAST_BAD_ARG, "dimensions must be positive");
    if (nx > INT32_MAX || ny > INT32_MAX || nz > INT32_MAX) return ft_fail(FAST_BAD_ARG, "dimension too large");
    if (iso != iso) return ft_fail(FAST_BAD_ARG, "isovalue is NaN");
    return FAST_OK;
}

// The whole area pass on device data; out[kFields] (host) gets the sums.
int area_device(const uint8_t *d_mask, const uint32_t *d_labels, const uint8_t *d_bits, int64_t nx, int64_t ny,
                int64_t nz, float iso, double *out, cudaStream_t st)
{
    std::call_once(g_table_once, [] { g_table = build_table(); });
    AlphaArgs A;
    memset(&A, 0, sizeof(A));
    A.mask = d_mask;
    A.labels = d_labels;
    A.label_bits = d_bits;
    A.nx = (int)nx;
    A.ny = (int)ny;
    A.nz = (int)nz;
    A.tiles_x = (int)((nx + TX - 1) / TX);
    A.tiles_y = (int)((ny + TY - 1) / TY);
    // z-slabs: 32 deep, halved while the grid has fewer than 8 blocks per SM.
    int sms = 152, dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t xy = (int64_t)A.tiles_x * A.tiles_y;
    int zc = kMaxSlab;
    while (zc > 1 && xy * ((nz + zc - 1) / zc) < 8LL * sms) zc /= 2;
    const int64_t nblocks = xy * ((nz + zc - 1) / zc);
    if (nblocks > INT32_MAX) return ft_fail(FAST_BAD_ARG, "volume too large for one area pass");
    A.zc = zc;
    A.iso = iso;
    A.vx = 1.0f / (float)nx;
    A.vy = 1.0f / (float)ny;
    A.vz = 1.0f / (float)nz;
    A.thr = 9;
    for (int c = 8; c >= 0; c--)
        if ((float)c * 0.125f >= iso) A.thr = c;

    const size_t part_bytes = (size_t)nblocks * kFields * sizeof(double);
    char *scratch = nullptr;
    const size_t need = sizeof(McTable) + 256 + part_bytes + 256 + kFields * sizeof(double) + 256 + 16;
    cudaError_t e = cudaMallocAsync((void **)&scratch, need, st);
    if (e != cudaSuccess) return ft_fail(FAST_NOMEM, "area scratch: %s", cudaGetErrorString(e));
    McTable *d_tab = (McTable *)scratch;
    double *d_part = (double *)(scratch + sizeof(McTable) + 256);
    double *d_out = (double *)((char *)d_part + part_bytes + 256);
    uint32_t *d_bad = (uint32_t *)((char *)d_out + kFields * sizeof(double) + 256);
    A.table = d_tab;
    A.partials = d_part;
    A.bad = d_bad;
    double h_out[kFields];
    uint32_t h_bad = 0;
    e = cudaMemcpyAsync(d_tab, &g_table, sizeof(McTable), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_bad, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) {
        if (d_labels)
            alpha_kernel<true><<<(unsigned)nblocks, NT, 0, st>>>(A);
        else
            alpha_kernel<false><<<(unsigned)nblocks, NT, 0, st>>>(A);
        alpha_sum_kernel<<<1, NT, 0, st>>>(d_part, (int)nblocks, d_out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_out, d_out, sizeof(h_out), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_bad, d_bad, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(scratch, st);
    const cudaError_t e2 = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return ft_fail(FAST_CUDA_ERROR, "area pass: %s", cudaGetErrorString(e));
    if (h_bad) return ft_fail(FAST_BAD_TYPE, "the volume must hold 0 and 255 only");
    if (!d_labels) {
        out[0] = h_out[0];
    } else {
        for (int f = 0; f < kFields; f++) out[f] = h_out[f];
    }
    return FAST_OK;
}

// getVolumeCCL(mask, 255) on the device, then the seven-field pass.
int tensor_device(const uint8_t *d_mask, int64_t nx, int64_t ny, int64_t nz, float iso, double *tensor,
                  double *area_solid, cudaStream_t st)
{
    if ((double)nx * ny * nz >= 4294967295.0) return ft_fail(FAST_BAD_ARG, "labelling is limited to 4294967294 voxels");
    const size_t n = (size_t)(nx * ny * nz);
    uint32_t *d_labels = nullptr;
    cudaError_t e = cudaMallocAsync((void **)&d_labels, n * 4, st);
    if (e != cudaSuccess) return ft_fail(FAST_NOMEM, "labels: %s", cudaGetErrorString(e));
    uint32_t num_labels = 0;
    int s = fast_ccl_label_device(d_mask, nx, ny, nz, 255, d_labels, &num_labels, nullptr, 0, st);
    std::vector<uint8_t> boundary;
    if (s == FAST_OK) {
        boundary.resize((size_t)7 * num_labels);
        s = fast_ccl_boundary_device(d_labels, nx, ny, nz, num_labels, boundary.data(), st);
    }
    uint8_t *d_bits = nullptr;
    if (s == FAST_OK) {
        std::vector<uint8_t> bits(num_labels, 0);
        for (int d = 0; d < 6; d++)
            for (uint32_t l = 1; l < num_labels; l++) bits[l] |= (uint8_t)(boundary[(size_t)d * num_labels + l] << d);
        e = cudaMallocAsync((void **)&d_bits, num_labels, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_bits, bits.data(), num_labels, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // bits is a stack buffer
        if (e != cudaSuccess) s = ft_fail(FAST_CUDA_ERROR, "label bits: %s", cudaGetErrorString(e));
    }
    double out[kFields];
    if (s == FAST_OK) s = area_device(d_mask, d_labels, d_bits, nx, ny, nz, iso, out, st);
    if (d_bits) cudaFreeAsync(d_bits, st);
    cudaFreeAsync(d_labels, st);
    cudaStreamSynchronize(st);
    if (s != FAST_OK) return s;
    for (int d = 0; d < 6; d++) tensor[d] = out[d];
    if (area_solid) *area_solid = out[6];
    return FAST_OK;
}

// Host mask -> device copy on a private stream, then `body`.
template <class F>
int with_device_mask(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, F body)
{
    const size_t n = (size_t)(nx * ny * nz);
    cudaStream_t st = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e != cudaSuccess) return ft_fail(FAST_CUDA_ERROR, "stream: %s", cudaGetErrorString(e));
    uint8_t *d = nullptr;
    int s;
    e = cudaMallocAsync((void **)&d, n, st);
    if (e != cudaSuccess) {
        s = ft_fail(FAST_NOMEM, "mask copy: %s", cudaGetErrorString(e));
    } else {
        e = cudaMemcpyAsync(d, mask, n, cudaMemcpyHostToDevice, st);
        s = e == cudaSuccess ? body(d, st) : ft_fail(FAST_CUDA_ERROR, "mask upload: %s", cudaGetErrorString(e));
        cudaFreeAsync(d, st);
    }
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    return s;
}

// ---------------------------------------------------------------------------
// Mesh export: the triangles themselves (getVolumeAreaMesh, fastlib/src/
// volume/VolumeSurface.cpp:38-68, ___generateTriangles in fastlib/src/cuda/
// VolumeSurface.cu:264-357).  Field = voxel != 0, corner values and cut
// vertices as for the area; positions in the reference's mesh frame: a voxel
// is dx = 1/max(n) wide on every axis and the grid is centred on the origin,
// p = (dx i - dx n / 2, ...); one face normal per triangle,
// normalize((v1 - v0) x (v2 - v0)).  Two passes with a fixed order: blocks
// of 256 cells count their triangles, the host scans the block totals, and
// each block writes its cells' triangles in cell order (12 floats each: three
// vertices, then the normal).
// ---------------------------------------------------------------------------
constexpr int kMeshBlock = 256;

struct MeshArgs {
    const uint8_t *mask;
    const McTable *table;
    int nx, ny, nz, thr;
    float iso, vx, vy, vz, dx;
};

__device__ __forceinline__ uint32_t mesh_counts(const MeshArgs &A, int64_t cell, int &cube, int &i, int &j, int &k)
{
    i = (int)(cell % A.nx);
    j = (int)((cell / A.nx) % A.ny);
    k = (int)(cell / ((int64_t)A.nx * A.ny));
    uint32_t cnt = 0;
    cube = 0;
#pragma unroll
    for (int c = 0; c < 8; c++) {
        const int ox = (c & 1) ^ ((c >> 1) & 1), oy = (c >> 1) & 1, oz = c >> 2;
        int n = 0;
        for (int dz = -1; dz <= 0; dz++)
            for (int dy = -1; dy <= 0; dy++)
                for (int dxx = -1; dxx <= 0; dxx++) {
                    int gx = i + ox + dxx, gy = j + oy + dy, gz = k + oz + dz;
                    gx = gx < 0 ? 0 : (gx >= A.nx ? A.nx - 1 : gx);
                    gy = gy < 0 ? 0 : (gy >= A.ny ? A.ny - 1 : gy);
                    gz = gz < 0 ? 0 : (gz >= A.nz ? A.nz - 1 : gz);
                    n += A.mask[((int64_t)gz * A.ny + gy) * A.nx + gx] != 0;
                }
        cnt |= (uint32_t)n << (4 * c);
        cube |= (n < A.thr) << c;
    }
    return cnt;
}

__global__ void __launch_bounds__(kMeshBlock) mesh_count_kernel(MeshArgs A, int64_t ncell, uint32_t *block_tri)
{
    __shared__ uint32_t s[kMeshBlock];
    const int64_t cell = (int64_t)blockIdx.x * kMeshBlock + threadIdx.x;
    uint32_t nt = 0;
    if (cell < ncell) {
        int cube, i, j, k;
        mesh_counts(A, cell, cube, i, j, k);
        nt = A.table->ntri[cube];
    }
    s[threadIdx.x] = nt;
    __syncthreads();
    for (int w = kMeshBlock / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) block_tri[blockIdx.x] = s[0];
}

__global__ void __launch_bounds__(kMeshBlock) mesh_emit_kernel(MeshArgs A, int64_t ncell, const uint64_t *block_off,
                                                               float *out)
{
    __shared__ uint32_t s[kMeshBlock];
    const int64_t cell = (int64_t)blockIdx.x * kMeshBlock + threadIdx.x;
    int cube = 0, i = 0, j = 0, k = 0;
    uint32_t cnt = 0, nt = 0;
    if (cell < ncell) {
        cnt = mesh_counts(A, cell, cube, i, j, k);
        nt = A.table->ntri[cube];
    }
    // exclusive scan of the counts in cell order (Hillis-Steele over the block)
    s[threadIdx.x] = nt;
    __syncthreads();
    for (int o = 1; o < kMeshBlock; o <<= 1) {
        const uint32_t v = threadIdx.x >= o ? s[threadIdx.x - o] : 0u;
        __syncthreads();
        s[threadIdx.x] += v;
        __syncthreads();
    }
    const uint64_t base = block_off[blockIdx.x] + s[threadIdx.x] - nt;
    if (nt == 0) return;
    // positions in the mesh frame (VolumeSurface.cu:291-297)
    const float px = __fsub_rn(__fmul_rn(A.dx, (float)i), __fmul_rn(0.5f, __fmul_rn(A.dx, (float)A.nx)));
    const float py = __fsub_rn(__fmul_rn(A.dx, (float)j), __fmul_rn(0.5f, __fmul_rn(A.dx, (float)A.ny)));
    const float pz = __fsub_rn(__fmul_rn(A.dx, (float)k), __fmul_rn(0.5f, __fmul_rn(A.dx, (float)A.nz)));
    const float qx = __fadd_rn(px, A.dx), qy = __fadd_rn(py, A.dx), qz = __fadd_rn(pz, A.dx);
    for (uint32_t t = 0; t < nt; t++) {
        float v[3][3];
        for (int q = 0; q < 3; q++) {
            const int e = A.table->edge[cube][3 * t + q];
            const int ca = edge_a(e), cb = edge_b(e);
            const float fa = __fmul_rn((float)((cnt >> (4 * ca)) & 15u), 0.125f);
            const float fb = __fmul_rn((float)((cnt >> (4 * cb)) & 15u), 0.125f);
            const float x0 = ((ca & 1) ^ ((ca >> 1) & 1)) ? qx : px, y0 = ((ca >> 1) & 1) ? qy : py, z0 = (ca >> 2) ? qz : pz;
            const float x1 = ((cb & 1) ^ ((cb >> 1) & 1)) ? qx : px, y1 = ((cb >> 1) & 1) ? qy : py, z1 = (cb >> 2) ? qz : pz;
            if (fa == fb) {
                v[q][0] = x0; v[q][1] = y0; v[q][2] = z0;
            } else {
                const float tt = __fdiv_rn(__fsub_rn(A.iso, fa), __fsub_rn(fb, fa));
                v[q][0] = lerp1(x0, x1, tt);
                v[q][1] = lerp1(y0, y1, tt);
                v[q][2] = lerp1(z0, z1, tt);
            }
        }
        const float ax = __fsub_rn(v[1][0], v[0][0]), ay = __fsub_rn(v[1][1], v[0][1]), az = __fsub_rn(v[1][2], v[0][2]);
        const float bx = __fsub_rn(v[2][0], v[0][0]), by = __fsub_rn(v[2][1], v[0][1]), bz = __fsub_rn(v[2][2], v[0][2]);
        const float cx = __fsub_rn(__fmul_rn(ay, bz), __fmul_rn(az, by));
        const float cy = __fsub_rn(__fmul_rn(az, bx), __fmul_rn(ax, bz));
        const float cz = __fsub_rn(__fmul_rn(ax, by), __fmul_rn(ay, bx));
        const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(cx, cx), __fmul_rn(cy, cy)), __fmul_rn(cz, cz)));
        const float inv = len > 0.f ? __fdiv_rn(1.0f, len) : 0.f;
        float *o = out + (base + t) * 12;
        for (int q = 0; q < 3; q++)
            for (int a = 0; a < 3; a++) o[3 * q + a] = v[q][a];
        o[9] = __fmul_rn(cx, inv);
        o[10] = __fmul_rn(cy, inv);
        o[11] = __fmul_rn(cz, inv);
    }
}

int mesh_device(const uint8_t *d_mask, int64_t nx, int64_t ny, int64_t nz, float iso, float *out, uint64_t capacity,
                uint64_t *ntri, cudaStream_t st)
{
    std::call_once(g_table_once, [] { g_table = build_table(); });
    const int64_t ncell = nx * ny * nz;
    const int64_t nblocks = (ncell + kMeshBlock - 1) / kMeshBlock;
    if (nblocks > INT32_MAX) return ft_fail(FAST_BAD_ARG, "volume too large for the mesh export");
    MeshArgs A;
    A.mask = d_mask;
    A.nx = (int)nx;
    A.ny = (int)ny;
    A.nz = (int)nz;
    A.iso = iso;
    A.thr = 9;
    for (int c = 8; c >= 0; c--)
        if ((float)c * 0.125f >= iso) A.thr = c;
    const int64_t maxdim = std::max(nx, std::max(ny, nz));
    A.dx = 1.0f / (float)maxdim;
    char *scratch = nullptr;
    const size_t need = sizeof(McTable) + 256 + (size_t)nblocks * 4 + 256 + (size_t)nblocks * 8;
    cudaError_t e = cudaMallocAsync((void **)&scratch, need, st);
    if (e != cudaSuccess) return ft_fail(FAST_NOMEM, "mesh scratch: %s", cudaGetErrorString(e));
    McTable *d_tab = (McTable *)scratch;
    uint32_t *d_cnt = (uint32_t *)(scratch + sizeof(McTable) + 256);
    uint64_t *d_off = (uint64_t *)((char *)d_cnt + ((size_t)nblocks * 4 + 255) / 256 * 256);
    A.table = d_tab;
    std::vector<uint32_t> cnt((size_t)nblocks);
    std::vector<uint64_t> off((size_t)nblocks);
    int s = FAST_OK;
    e = cudaMemcpyAsync(d_tab, &g_table, sizeof(McTable), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        mesh_count_kernel<<<(unsigned)nblocks, kMeshBlock, 0, st>>>(A, ncell, d_cnt);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(cnt.data(), d_cnt, (size_t)nblocks * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    uint64_t total = 0;
    if (e == cudaSuccess) {
        for (int64_t b = 0; b < nblocks; b++) {
            off[(size_t)b] = total;
            total += cnt[(size_t)b];
        }
        *ntri = total;
        if (out && total > capacity)
            s = ft_fail(FAST_BAD_ARG, "mesh buffer holds %llu triangles, %llu needed", (unsigned long long)capacity,
                        (unsigned long long)total);
        if (out && s == FAST_OK && total > 0) {
            float *d_out = nullptr;
            e = cudaMallocAsync((void **)&d_out, (size_t)total * 12 * sizeof(float), st);
            if (e != cudaSuccess) {
                s = ft_fail(FAST_NOMEM, "mesh triangles: %s", cudaGetErrorString(e));
            } else {
                e = cudaMemcpyAsync(d_off, off.data(), (size_t)nblocks * 8, cudaMemcpyHostToDevice, st);
                if (e == cudaSuccess) {
                    mesh_emit_kernel<<<(unsigned)nblocks, kMeshBlock, 0, st>>>(A, ncell, d_off, d_out);
                    e = cudaGetLastError();
                }
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(out, d_out, (size_t)total * 12 * sizeof(float), cudaMemcpyDeviceToHost, st);
                cudaFreeAsync(d_out, st);
            }
        }
    }
    cudaFreeAsync(scratch, st);
    const cudaError_t e2 = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = e2;
    if (s == FAST_OK && e != cudaSuccess) s = ft_fail(FAST_CUDA_ERROR, "mesh: %s", cudaGetErrorString(e));
    return s;
}

}  // namespace

extern "C" {

FAST_API int fast_reactive_area_mesh(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, float isovalue,
                                     float *triangles, uint64_t capacity, uint64_t *ntri)
{
    ft_clear_error();
    if (!mask) return ft_fail(FAST_NO_HOST_DATA, "mask is NULL");
    if (!ntri) return ft_fail(FAST_BAD_ARG, "ntri is NULL");
    int s = check_args(nx, ny, nz, isovalue);
    if (s != FAST_OK) return s;
    return with_device_mask(mask, nx, ny, nz, [&](const uint8_t *d, cudaStream_t st) {
        return mesh_device(d, nx, ny, nz, isovalue, triangles, capacity, ntri, st);
    });
}


FAST_API int fast_reactive_area_device(const uint8_t *d_mask, int64_t nx, int64_t ny, int64_t nz, float isovalue,
                                       double *area, void *stream)
{
    ft_clear_error();
    if (!d_mask) return ft_fail(FAST_NO_HOST_DATA, "mask is NULL");
    if (!area) return ft_fail(FAST_BAD_ARG, "area is NULL");
    int s = check_args(nx, ny, nz, isovalue);
    if (s != FAST_OK) return s;
    return area_device(d_mask, nullptr, nullptr, nx, ny, nz, isovalue, area, (cudaStream_t)stream);
}

FAST_API int fast_reactive_area(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, float isovalue, double *area)
{
    ft_clear_error();
    if (!mask) return ft_fail(FAST_NO_HOST_DATA, "mask is NULL");
    if (!area) return ft_fail(FAST_BAD_ARG, "area is NULL");
    int s = check_args(nx, ny, nz, isovalue);
    if (s != FAST_OK) return s;
    return with_device_mask(mask, nx, ny, nz, [&](const uint8_t *d, cudaStream_t st) {
        return area_device(d, nullptr, nullptr, nx, ny, nz, isovalue, area, st);
    });
}

FAST_API int fast_reactive_area_tensor_device(const uint8_t *d_mask, int64_t nx, int64_t ny, int64_t nz,
                                              float isovalue, double *tensor, double *area_solid, void *stream)
{
    ft_clear_error();
    if (!d_mask) return ft_fail(FAST_NO_HOST_DATA, "mask is NULL");
    if (!tensor) return ft_fail(FAST_BAD_ARG, "tensor is NULL");
    int s = check_args(nx, ny, nz, isovalue);
    if (s != FAST_OK) return s;
    return tensor_device(d_mask, nx, ny, nz, isovalue, tensor, area_solid, (cudaStream_t)stream);
}

FAST_API int fast_reactive_area_tensor(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, float isovalue,
                                       double *tensor, double *area_solid)
{
    ft_clear_error();
    if (!mask) return ft_fail(FAST_NO_HOST_DATA, "mask is NULL");
    if (!tensor) return ft_fail(FAST_BAD_ARG, "tensor is NULL");
    int s = check_args(nx, ny, nz, isovalue);
    if (s != FAST_OK) return s;
    return with_device_mask(mask, nx, ny, nz, [&](const uint8_t *d, cudaStream_t st) {
        return tensor_device(d, nx, ny, nz, isovalue, tensor, area_solid, st);
    });
}

}  // extern "C"
