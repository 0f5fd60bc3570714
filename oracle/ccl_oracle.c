/*
 * ccl_oracle.c -- CPU restatement of the reference's 6-connected component
 * labelling (fastlib/src/cuda/VolumeCCL.cu:381-620 VolumeCCL_Label,
 * :753-818 VolumeCCL_BoundaryLabels; fastlib/src/volume/VolumeSegmentation.cpp:
 * 14-64 getDirMask / getVolumeCCL).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA labelling kernels.
 *
 * Semantics restated:
 *   - foreground = voxels whose value differs from `background`; for binary
 *     volumes (every voxel either `background` or one other value) this is
 *     exactly the span set the reference's toggle scan builds (VolumeCCL.cu:
 *     87-169);
 *   - components are 6-connected (x-runs joined to x-overlapping runs in rows
 *     y+-1 and z+-1, VolumeCCL.cu:204-283);
 *   - every component converges to the minimum linear index of its voxels
 *     (atomicMin of span-begin indices); roots are marked and inclusive-scanned
 *     in (z, y, span) order, i.e. in increasing linear index (VolumeCCL.cu:
 *     326-375, 547-560), so label k is the component with the k-th smallest
 *     minimum linear index; 0 is background; num_labels = K + 1;
 *   - boundary[d*num_labels + l] = 1 when label l > 0 touches face d, in Dir
 *     order X_POS (x = nx-1), X_NEG (x = 0), ... ; row 6 is the AND of rows 0-5
 *     (VolumeCCL.cu:735-818).
 *
 * A sequential union-find with a raster-order relabel yields exactly this
 * numbering: the first voxel of a component met in raster order is its
 * minimum linear index.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static uint32_t uf_find(uint32_t *par, uint32_t a)
{
    uint32_t r = a;
    while (par[r] != r) r = par[r];
    while (par[a] != r) {
        const uint32_t n = par[a];
        par[a] = r;
        a = n;
    }
    return r;
}

static void uf_union(uint32_t *par, uint32_t a, uint32_t b)
{
    a = uf_find(par, a);
    b = uf_find(par, b);
    if (a == b) return;
    if (a < b) par[b] = a; else par[a] = b;
}

/* Returns num_labels (K + 1), or 0 on a bad argument / allocation failure. */
uint32_t oracle_ccl_label(const uint8_t *vol, int64_t nx, int64_t ny, int64_t nz,
                          uint8_t background, uint32_t *labels)
{
    const int64_t N = nx * ny * nz;
    if (nx <= 0 || ny <= 0 || nz <= 0 || N >= (int64_t)UINT32_MAX) return 0;
    uint32_t *par = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)N);
    if (!par) return 0;
    const int64_t sy = nx, sz = nx * ny;
    for (int64_t z = 0; z < nz; z++)
        for (int64_t y = 0; y < ny; y++)
            for (int64_t x = 0; x < nx; x++) {
                const int64_t i = x + sy * y + sz * z;
                par[i] = (uint32_t)i;
                if (vol[i] == background) continue;
                if (x > 0 && vol[i - 1] != background) uf_union(par, (uint32_t)i, (uint32_t)(i - 1));
                if (y > 0 && vol[i - sy] != background) uf_union(par, (uint32_t)i, (uint32_t)(i - sy));
                if (z > 0 && vol[i - sz] != background) uf_union(par, (uint32_t)i, (uint32_t)(i - sz));
            }
    /* Relabel in raster order; reuse `labels` for root -> label lookups. */
    uint32_t next = 1;
    for (int64_t i = 0; i < N; i++) {
        if (vol[i] == background) { labels[i] = 0; continue; }
        const uint32_t r = uf_find(par, (uint32_t)i);
        if ((int64_t)r == i) labels[i] = next++;
        else labels[i] = labels[r];
    }
    free(par);
    return next;
}

/* boundary: 7 * num_labels bytes. */
void oracle_ccl_boundary(const uint32_t *labels, int64_t nx, int64_t ny, int64_t nz,
                         uint32_t num_labels, uint8_t *boundary)
{
    memset(boundary, 0, (size_t)7 * num_labels);
    const int64_t res[3] = {nx, ny, nz};
    for (int d = 0; d < 6; d++) {
        const int k = d / 2;
        const int sgn = -((d % 2) * 2 - 1);
        const int64_t fixed = (sgn == 1) ? res[k] - 1 : 0;
        const int a = (k + 1) % 3, b = (k + 2) % 3;
        for (int64_t u = 0; u < res[b]; u++)
            for (int64_t v = 0; v < res[a]; v++) {
                int64_t p[3];
                p[k] = fixed; p[a] = v; p[b] = u;
                const uint32_t l = labels[p[0] + nx * (p[1] + ny * p[2])];
                if (l > 0) boundary[(size_t)d * num_labels + l] = 1;
            }
    }
    for (uint32_t l = 0; l < num_labels; l++) {
        uint8_t all = 1;
        for (int d = 0; d < 6; d++) all &= boundary[(size_t)d * num_labels + l];
        boundary[(size_t)6 * num_labels + l] = all;
    }
}
