/* CPU restatement of the reactive-area measure -- TEST INFRASTRUCTURE ONLY
 * (the checker of the engine's area pass; the product never links it).
 *
 * Follows the reference's marching-cubes area:
 *   getVolumeArea (fastlib/src/volume/VolumeSurface.cpp:10-36): res = the
 *     volume's dimensions, isovalue, cells over [0, res)^3;
 *   ___generateTrianglesSurfaceArea (fastlib/src/cuda/VolumeSurface.cu:198-262):
 *     corner samples, getCubeIndex (v < iso -> bit), vertexInterp
 *     (:176-184), triangleArea (:192-194), per-cell double sum;
 *   getVoxelCornerVals / getVoxelCornerPos (:78-114): corner order and
 *     positions p = (i/nx, j/ny, k/nz) + offsets of one voxel size;
 *   the texture read (fastlib/src/utility/DataPtr.cpp:565-595: normalized
 *     coordinates, linear filter, clamp) at a grid point = mean of the eight
 *     voxels around it, clamped at the faces;
 *   getReactiveAreaDensity(Tensor) (fastlib/src/volume/VolumeMeasures.cpp:
 *     294-335) sums the cell areas.
 *
 * The triangulation is generated by the rule the engine states, written
 * here on its own: the cut edges of each cube face are paired (a face with
 * four cut edges pairs the edges around each "below" corner), the pairs are
 * walked into loops starting at the smallest edge number and stepping to the
 * smaller neighbour first, and each loop is fanned from its first edge.
 * Parity with the reference's own published table is not claimed for cells
 * whose loop is not planar ("parity unpinned" there); planar interfaces give
 * table-independent areas and pin the rest.
 *
 * Build: -ffp-contract=off (oracle/Makefile), so every float operation is
 * rounded as written. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* Corner offsets in the reference's order (VolumeSurface.cu:102-114). */
static const int CX[8] = {0, 1, 1, 0, 0, 1, 1, 0};
static const int CY[8] = {0, 0, 1, 1, 0, 0, 1, 1};
static const int CZ[8] = {0, 0, 0, 0, 1, 1, 1, 1};
/* Edge endpoints in the order of the vertexInterp calls (VolumeSurface.cu:224-235). */
static const int EA[12] = {0, 1, 2, 3, 4, 5, 6, 7, 0, 1, 2, 3};
static const int EB[12] = {1, 2, 3, 0, 5, 6, 7, 4, 4, 5, 6, 7};
/* Cube faces, corners in cyclic order. */
static const int FACE[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4}, {3, 2, 6, 7}, {0, 3, 7, 4}, {1, 2, 6, 5}};

static int g_ntri[256];
static int g_tri[256][15];
static int g_ready = 0;

static int find_edge(int a, int b)
{
    int e;
    for (e = 0; e < 12; e++) {
        if (EA[e] == a && EB[e] == b) return e;
        if (EA[e] == b && EB[e] == a) return e;
    }
    return -1;
}

static void add_pair(int adj[12][2], int cnt[12], int a, int b)
{
    adj[a][cnt[a]++] = b;
    adj[b][cnt[b]++] = a;
}

static void make_table(void)
{
    int cs, f, q, e;
    for (cs = 0; cs < 256; cs++) {
        int adj[12][2], cnt[12], used[12];
        int n = 0;
        memset(cnt, 0, sizeof(cnt));
        memset(used, 0, sizeof(used));
        for (f = 0; f < 6; f++) {
            int c[4], b[4], k[4], m = 0;
            for (q = 0; q < 4; q++) {
                c[q] = FACE[f][q];
                b[q] = (cs >> c[q]) & 1;
            }
            for (q = 0; q < 4; q++) {
                if (b[q] != b[(q + 1) % 4]) k[m++] = find_edge(c[q], c[(q + 1) % 4]);
            }
            if (m == 2) {
                add_pair(adj, cnt, k[0], k[1]);
            } else if (m == 4) {
                /* k[] holds the face's four edges in cyclic order starting at
                 * edge (c0, c1); pair around the two "below" corners. */
                if (b[0]) {
                    add_pair(adj, cnt, k[3], k[0]);
                    add_pair(adj, cnt, k[1], k[2]);
                } else {
                    add_pair(adj, cnt, k[0], k[1]);
                    add_pair(adj, cnt, k[2], k[3]);
                }
            }
        }
        for (e = 0; e < 12; e++) {
            int ring[12], len = 0, prev, cur, i;
            if (cnt[e] == 0 || used[e]) continue;
            ring[len++] = e;
            used[e] = 1;
            prev = e;
            cur = adj[e][0] < adj[e][1] ? adj[e][0] : adj[e][1];
            while (cur != e) {
                int nxt;
                ring[len++] = cur;
                used[cur] = 1;
                nxt = (adj[cur][0] == prev) ? adj[cur][1] : adj[cur][0];
                prev = cur;
                cur = nxt;
            }
            for (i = 1; i + 1 < len; i++) {
                g_tri[cs][3 * n] = ring[0];
                g_tri[cs][3 * n + 1] = ring[i];
                g_tri[cs][3 * n + 2] = ring[i + 1];
                n++;
            }
        }
        g_ntri[cs] = n;
    }
    g_ready = 1;
}

static int64_t clampi(int64_t v, int64_t n) { return v < 0 ? 0 : (v >= n ? n - 1 : v); }

/* Value at grid point (gx, gy, gz): mean of the 8 clamped voxels around it. */
static float grid_value(const uint8_t *fld, int64_t nx, int64_t ny, int64_t nz, int64_t gx, int64_t gy, int64_t gz)
{
    float s = 0.0f;
    int a, b, c;
    for (c = 0; c < 2; c++)
        for (b = 0; b < 2; b++)
            for (a = 0; a < 2; a++) {
                const int64_t x = clampi(gx - 1 + a, nx), y = clampi(gy - 1 + b, ny), z = clampi(gz - 1 + c, nz);
                s += fld[(z * ny + y) * nx + x] ? 1.0f : 0.0f;
            }
    return s * 0.125f;
}

/* lerp(a, b, t) = a + t (b - a) (CUDA's helper_math form). */
static float lerpf1(float a, float b, float t) { return a + t * (b - a); }

/* Area of the isovalue surface of a 0/1 field (uint8, nonzero = 1). */
double oracle_area_field(const uint8_t *fld, int64_t nx, int64_t ny, int64_t nz, float iso)
{
    int64_t k;
    double total = 0.0;
    double *per_z;
    const float vx = 1.0f / (float)nx, vy = 1.0f / (float)ny, vz = 1.0f / (float)nz;
    if (!g_ready) make_table();
    per_z = (double *)calloc((size_t)nz, sizeof(double));
#pragma omp parallel for schedule(dynamic, 1)
    for (k = 0; k < nz; k++) {
        int64_t i, j;
        double zsum = 0.0;
        for (j = 0; j < ny; j++) {
            for (i = 0; i < nx; i++) {
                float val[8], P[8][3];
                int c, cube = 0, t;
                double cell = 0.0;
                const float px = vx * (float)i, py = vy * (float)j, pz = vz * (float)k;
                for (c = 0; c < 8; c++) {
                    val[c] = grid_value(fld, nx, ny, nz, i + CX[c], j + CY[c], k + CZ[c]);
                    if (val[c] < iso) cube |= 1 << c;
                    P[c][0] = CX[c] ? px + vx : px;
                    P[c][1] = CY[c] ? py + vy : py;
                    P[c][2] = CZ[c] ? pz + vz : pz;
                }
                for (t = 0; t < g_ntri[cube]; t++) {
                    float V[3][3], d1[3], d2[3], cr[3];
                    int q, ax;
                    for (q = 0; q < 3; q++) {
                        const int e = g_tri[cube][3 * t + q];
                        const int a = EA[e], b = EB[e];
                        if (val[a] == val[b]) {
                            for (ax = 0; ax < 3; ax++) V[q][ax] = P[a][ax];
                        } else {
                            const float tt = (iso - val[a]) / (val[b] - val[a]);
                            for (ax = 0; ax < 3; ax++) V[q][ax] = lerpf1(P[a][ax], P[b][ax], tt);
                        }
                    }
                    for (ax = 0; ax < 3; ax++) {
                        d1[ax] = V[1][ax] - V[0][ax];
                        d2[ax] = V[2][ax] - V[0][ax];
                    }
                    cr[0] = d1[1] * d2[2] - d1[2] * d2[1];
                    cr[1] = d1[2] * d2[0] - d1[0] * d2[2];
                    cr[2] = d1[0] * d2[1] - d1[1] * d2[0];
                    cell += (double)(sqrtf(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]) * 0.5f);
                }
                zsum += cell;
            }
        }
        per_z[k] = zsum;
    }
    for (k = 0; k < nz; k++) total += per_z[k];
    free(per_z);
    return total;
}

/* Triangle count of a corner pattern (for table checks). */
int oracle_mc_ntri(int cube)
{
    if (!g_ready) make_table();
    return (cube >= 0 && cube < 256) ? g_ntri[cube] : -1;
}
