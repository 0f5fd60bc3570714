// Host driver of the reference's own per-voxel assembly rule,
// getSystemTopKernel<T> (fastlib/src/cuda/Diffusion.cuh:54-148), compiled
// from the reference's source by oracle/Makefile's `ref` target (outputs in
// oracle/_ref/).  TEST INFRASTRUCTURE ONLY: it pins the oracle's restated
// assembly (tau_oracle_impl.h) to the reference's code; nothing in the
// product links it.
//
// The inputs getSystemTopKernel takes are formed here as the reference forms
// them elsewhere, in code that cannot be compiled here (Eigen, CUDA surface
// kernels):
//   * DiffusionSysParams as setupSysParams fills it (fastlib/src/solver/
//     Diffusion.cpp:16-35): concentrations 1 and 0 ordered by the
//     direction's sign, cellDim = the float h = 1/maxDim of
//     VolumeMeasures.cpp:68 for all three axes, faceArea products in double,
//     dirPrimary = the direction's axis;
//   * the per-voxel face diffusivity stencil of ___linearSysKernel
//     (fastlib/src/cuda/Diffusion.cu:30-71): D = mask > 0 ? d1 : d0 at the
//     voxel and its clamped neighbours, face D = (D_nbr + D_here) * 0.5.
#include <cstdint>
#include <cstring>

#include "Diffusion.cuh"

using namespace fast;

template <typename T>
static int assemble(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, int dir, double d0, double d1,
                    float cell_f, T *A, T *b, T *x0)
{
    if (dir < 0 || dir > 5) return 1;
    const int64_t N = nx * ny * nz;
    DiffusionSysParams sp;
    std::memset(&sp, 0, sizeof(sp));
    sp.highConc = 1.0;
    sp.lowConc = 0.0;
    const int sgn = _getDirSgn(Dir(dir));
    sp.concetrationBegin = sgn == 1 ? sp.highConc : sp.lowConc;
    sp.concetrationEnd = sgn == 1 ? sp.lowConc : sp.highConc;
    for (int k = 0; k < 3; k++) sp.cellDim[k] = (double)cell_f;
    sp.faceArea[0] = sp.cellDim[1] * sp.cellDim[2];
    sp.faceArea[1] = sp.cellDim[0] * sp.cellDim[2];
    sp.faceArea[2] = sp.cellDim[0] * sp.cellDim[1];
    sp.dirPrimary = (int)_getDirIndex(Dir(dir));
    sp.dir = Dir(dir);
    const ivec3 res{(int)nx, (int)ny, (int)nz};
    for (int64_t z = 0; z < nz; z++)
        for (int64_t y = 0; y < ny; y++)
            for (int64_t x = 0; x < nx; x++) {
                const int64_t i = x + nx * (y + ny * z);
                const ivec3 vox{(int)x, (int)y, (int)z};
                const T Dc = mask[i] > 0 ? (T)d1 : (T)d0;
                Stencil_7<T> diff;
                for (int d = 0; d < 6; d++) {
                    const int k = (int)_getDirIndex(Dir(d));
                    ivec3 p = vox;
                    const int nv = p[k] + _getDirSgn(Dir(d));
                    if (nv >= 0 && nv < res[k]) p[k] = nv;
                    const int64_t j = p.x + nx * (p.y + ny * (int64_t)p.z);
                    const T Dn = mask[j] > 0 ? (T)d1 : (T)d0;
                    diff.v[d] = (Dn + Dc) * T(0.5);
                }
                diff.v[DIR_NONE] = Dc;
                Stencil_7<T> out;
                T f, xv;
                getSystemTopKernel<T>(sp, diff, vox, res, &out, &f, &xv);
                for (int d = 0; d < 7; d++) A[(int64_t)d * N + i] = out.v[d];
                b[i] = f;
                x0[i] = xv;
            }
    return 0;
}

extern "C" int ref_assemble_f64(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, int dir, double d0,
                                double d1, float cell_f, double *A, double *b, double *x0)
{
    return assemble<double>(mask, nx, ny, nz, dir, d0, d1, cell_f, A, b, x0);
}

extern "C" int ref_assemble_f32(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, int dir, double d0,
                                double d1, float cell_f, float *A, float *b, float *x0)
{
    return assemble<float>(mask, nx, ny, nz, dir, d0, d1, cell_f, A, b, x0);
}
