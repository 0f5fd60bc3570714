// Drives include/fasttau.hpp the way fastlib's callers do (TauModule::getTau,
// fast/src/TauModule.h:34-118): a uint8 Volume, TortuosityParams with the
// CLI's coefficients, getPorosity<T> and getTortuosity<T> for T = float and
// double, with the concentration output and the iteration count.
//
// usage: shim_check <volume.bin> <dir 0..5> <solver 0=BICGSTAB|1=CG> <tol double> <tol float>
// prints one line per precision:  <T> <tau> <porosity> <iterations> <sum of c> <c at voxel 0>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "fasttau.hpp"

template <typename T>
static int run(const fast::Volume &mask, fast::Dir dir, fast::DiffusionSolverType solver, double tol, const char *name)
{
    fast::TortuosityParams tp;
    tp.dir = dir;
    tp.coeffs = fast::vec2(1.0f, 0.001f);
    tp.tolerance = tol;
    tp.maxIter = 100000;
    tp.porosity = fast::getPorosity<double>(mask);
    tp.porosityPrecomputed = true;
    fast::Volume conc(mask.dim(), fast::primitiveTypeof<T>());
    size_t iters = 0;
    const T tau = fast::getTortuosity<T>(mask, tp, solver, &conc, &iters);
    const T *c = static_cast<const T *>(conc.getPtr().getCPU());
    double sum = 0.0;
    for (size_t i = 0; i < conc.totalElems(); i++) sum += (double)c[i];
    std::printf("%s %.17g %.17g %zu %.17g %.17g\n", name, (double)tau, (double)fast::getPorosity<T>(mask), iters, sum,
                (double)c[0]);
    return tau > T(0) ? 0 : 1;
}

int main(int argc, char **argv)
{
    if (argc < 6) {
        std::fprintf(stderr, "usage: %s volume.bin dir solver tol_double tol_float\n", argv[0]);
        return 2;
    }
    // .bin: int32 PrimitiveType, int32 x3 dims, one byte, then the voxels
    // (fastlib/src/volume/VolumeIO.cpp:256-305)
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int32_t hdr[4];
    unsigned char flag = 0;
    if (std::fread(hdr, 4, 4, f) != 4 || std::fread(&flag, 1, 1, f) != 1 || hdr[0] != fast::TYPE_UCHAR) return 2;
    fast::Volume mask(fast::ivec3(hdr[1], hdr[2], hdr[3]), fast::TYPE_UCHAR);
    const size_t n = mask.totalElems();
    if (std::fread(mask.getPtr().getCPU(), 1, n, f) != n) return 2;
    std::fclose(f);
    if (mask.sumZeroElems() == 0) return 3;
    const fast::Dir dir = (fast::Dir)std::atoi(argv[2]);
    const fast::DiffusionSolverType solver = std::atoi(argv[3]) == 1 ? fast::DSOLVER_CG : fast::DSOLVER_BICGSTAB;
    int rc = run<double>(mask, dir, solver, std::atof(argv[4]), "double");
    rc |= run<float>(mask, dir, solver, std::atof(argv[5]), "float");
    // errors come back as T(0) with the cause on stderr, as in the reference
    fast::Volume wrong(mask.dim(), fast::TYPE_FLOAT);
    fast::TortuosityParams tp;
    if (fast::getTortuosity<double>(wrong, tp) != 0.0) rc |= 4;
    return rc;
}
