/*
 * tau_oracle.c -- CPU restatement of the reference tortuosity path
 * (krsvojte/fast, fastlib): the 7-point diffusion system assembly, Jacobi-PCG and
 * right-Jacobi BiCGSTAB with the reference stopping rules, the tau plane-flux
 * reduction, the porosity count and 6-connected component labels.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that tests/, the smoke
 * check and bench.py's CPU baseline leg compare the CUDA path against.  The
 * product library never links, loads or calls it.
 *
 * Parity status: the reference cannot be built here (Eigen and the glm
 * submodule are absent, the default arch is sm_30) and ships no tests, golden
 * vectors or fixtures.  This restatement is therefore pinned against
 * closed-form known answers of the reference discretisation (all-pore tau=1,
 * all-solid tau=0, parallel layers tau = phi/(phi+(1-phi)D1), series layers from
 * the 1-D arithmetic-mean resistor chain) and cross-checked against an
 * independent scipy assembly + direct solve; it is not pinned to outputs of
 * the reference binary itself.
 *
 * Built with -ffp-contract=off so x86-64 and aarch64 builds round identically.
 */
#include <math.h>
#include <float.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

enum { X_POS_ = 0, X_NEG_, Y_POS_, Y_NEG_, Z_POS_, Z_NEG_, DIR_NONE_ };
enum { ORACLE_OK = 0, ORACLE_BAD_ARG = 1, ORACLE_NOMEM = 3, ORACLE_NO_CONVERGENCE = 4 };
enum { ORACLE_DEVICE = 0, ORACLE_EIGEN = 1 };
enum { ORACLE_SOLVER_BICGSTAB = 0, ORACLE_SOLVER_CG = 1 };

/* PrimitiveTypes.h:142-177: getDirIndex, getDirSgn, getDir */
static inline int dir_index(int d) { return d / 2; }
static inline int dir_sgn(int d) { return -((d % 2) * 2 - 1); }
static inline int make_dir(int index, int sgn) { return index * 2 + (1 - (sgn + 1) / 2); }

/* Volume::sumZeroElems (fastlib/src/volume/Volume.cpp:261-272): count of zero voxels. */
uint64_t oracle_count_pores(const uint8_t *mask, int64_t N)
{
    uint64_t c = 0;
#pragma omp parallel for reduction(+ : c) schedule(static)
    for (int64_t i = 0; i < N; i++) c += (mask[i] == 0);
    return c;
}

#define REAL double
#define SFX(x) x##_f64
#define ORACLE_REAL_EPS DBL_EPSILON
#define ORACLE_REAL_MIN DBL_MIN
#include "tau_oracle_impl.h"
#undef REAL
#undef SFX
#undef ORACLE_REAL_EPS
#undef ORACLE_REAL_MIN

#define REAL float
#define SFX(x) x##_f32
#define ORACLE_REAL_EPS FLT_EPSILON
#define ORACLE_REAL_MIN FLT_MIN
#include "tau_oracle_impl.h"
#undef REAL
#undef SFX
#undef ORACLE_REAL_EPS
#undef ORACLE_REAL_MIN
