/*
 * fasttau.hpp -- header-only C++ front end of libfasttau.so with fastlib's
 * tortuosity API, so that a caller of fast::getTortuosity<T> /
 * fast::getPorosity<T> switches by changing its include and link line.
 *
 * Mirrors (reference paths inside the fastlib project):
 *   enum Dir, PrimitiveType      fastlib/include/fastlib/utility/PrimitiveTypes.h:11-24,142-150
 *   DiffusionSolverType,
 *   TortuosityParams,
 *   getTortuosity<T>,
 *   getPorosity<T>               fastlib/include/fastlib/volume/VolumeMeasures.h:15-61
 *   Volume (host side only)      fastlib/include/fastlib/volume/Volume.h:18-105
 *   ivec3 / vec2                 glm's, as fastlib/include/fastlib/utility/Types.h uses them
 *
 * Behaviour kept from fastlib/src/volume/VolumeMeasures.cpp:42-292: any
 * failure returns T(0) with the cause on stderr; the mask must be TYPE_UCHAR
 * with its host copy present; porosity is computed unless
 * params.porosityPrecomputed; `concetrationOutput`, when given with
 * params.onDevice, receives the solution (a Volume of T with the mask's
 * dimensions); `iterationsOut` receives the solver's iteration count.  Every
 * solve runs on the GPU through fast_tau_solve: params.onDevice = false (the
 * reference's Eigen path) and cpuThreads change nothing but the
 * concentration output, which the reference writes on its device path only.
 * useNonUniform (a path the reference's CLI never takes) is rejected.
 *
 * T = double solves in FP64 and T = float in FP32, as the reference's
 * template instantiations (VolumeMeasures.cpp:348-349).
 */
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <stdexcept>
#include <type_traits>
#include <vector>

#include "fasttau.h"

namespace fast {

enum Dir { X_POS = 0, X_NEG = 1, Y_POS = 2, Y_NEG = 3, Z_POS = 4, Z_NEG = 5, DIR_NONE = 6 };

enum PrimitiveType {
    TYPE_FLOAT = 0, TYPE_CHAR, TYPE_UCHAR, TYPE_INT, TYPE_UINT, TYPE_UINT64, TYPE_FLOAT3, TYPE_FLOAT4,
    TYPE_DOUBLE, TYPE_UCHAR3, TYPE_UCHAR4, TYPE_UNKNOWN
};

enum DiffusionSolverType { DSOLVER_BICGSTAB, DSOLVER_CG };

struct ivec3 {
    int x = 0, y = 0, z = 0;
    ivec3() = default;
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
    explicit ivec3(int v) : x(v), y(v), z(v) {}
    int &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    int operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

struct vec2 {
    float x = 0.f, y = 0.f;
    vec2() = default;
    vec2(float a, float b) : x(a), y(b) {}
    float &operator[](int i) { return i == 0 ? x : y; }
    float operator[](int i) const { return i == 0 ? x : y; }
};

inline size_t primitiveSizeof(PrimitiveType t)
{
    switch (t) {
    case TYPE_FLOAT: case TYPE_INT: case TYPE_UINT: return 4;
    case TYPE_CHAR: case TYPE_UCHAR: return 1;
    case TYPE_UINT64: case TYPE_DOUBLE: return 8;
    case TYPE_FLOAT3: return 12;
    case TYPE_FLOAT4: return 16;
    case TYPE_UCHAR3: return 3;
    case TYPE_UCHAR4: return 4;
    default: return 0;
    }
}

template <typename T>
inline PrimitiveType primitiveTypeof()
{
    if (std::is_same<T, float>::value) return TYPE_FLOAT;
    if (std::is_same<T, double>::value) return TYPE_DOUBLE;
    if (std::is_same<T, unsigned char>::value) return TYPE_UCHAR;
    if (std::is_same<T, int>::value) return TYPE_INT;
    if (std::is_same<T, unsigned int>::value) return TYPE_UINT;
    if (std::is_same<T, unsigned long long>::value) return TYPE_UINT64;
    return TYPE_UNKNOWN;
}

/* The host half of fastlib's Volume: a dense x-fastest buffer of dim.x *
 * dim.y * dim.z elements of one primitive type.  getPtr().getCPU() is the
 * host pointer (NULL until allocated, as a volume whose host copy was never
 * retrieved). */
class Volume {
public:
    class Ptr {
    public:
        void *getCPU() { return data_.empty() ? nullptr : data_.data(); }
        const void *getCPU() const { return data_.empty() ? nullptr : data_.data(); }
        void allocCPU(size_t bytes) { data_.assign(bytes, 0); }
        void freeCPU() { std::vector<unsigned char>().swap(data_); }

    private:
        std::vector<unsigned char> data_;
    };

    Volume(ivec3 dim, PrimitiveType type, bool alloc_cpu = true) : dim_(dim), type_(type)
    {
        if (dim.x <= 0 || dim.y <= 0 || dim.z <= 0) throw std::invalid_argument("Volume dimensions must be positive");
        if (alloc_cpu) ptr_.allocCPU(totalElems() * elementSize());
    }

    ivec3 dim() const { return dim_; }
    PrimitiveType type() const { return type_; }
    size_t totalElems() const { return (size_t)dim_.x * (size_t)dim_.y * (size_t)dim_.z; }
    size_t elementSize() const { return primitiveSizeof(type_); }
    Ptr &getPtr() { return ptr_; }
    const Ptr &getPtr() const { return ptr_; }

    /* Number of zero elements (Volume::sumZeroElems, Volume.cpp:261-272),
     * counted on the GPU for a uint8 volume. */
    size_t sumZeroElems() const
    {
        const void *d = ptr_.getCPU();
        if (type_ != TYPE_UCHAR || !d) throw std::runtime_error("sumZeroElems: needs a uint8 volume with host data");
        double phi = 0.0;
        uint64_t zeros = 0;
        const int st = fast_porosity(static_cast<const uint8_t *>(d), dim_.x, dim_.y, dim_.z, &phi, &zeros);
        if (st != FAST_OK) throw std::runtime_error(fast_last_error());
        return (size_t)zeros;
    }

private:
    ivec3 dim_;
    PrimitiveType type_;
    Ptr ptr_;
};

struct TortuosityParams {
    Dir dir = X_NEG;
    vec2 coeffs = vec2(1.0f, 0.001f);
    double tolerance = 1e-6;
    size_t maxIter = 10000;
    bool verbose = false;
    bool oversubscribeGPUMemory = false;
    bool useNonUniform = false;

    // Porosity
    bool porosityPrecomputed = false;
    double porosity = -1.0;
    bool onDevice = true;
    int cpuThreads = -1;
};

template <typename T>
inline T getPorosity(const Volume &mask)
{
    static_assert(std::is_same<T, float>::value || std::is_same<T, double>::value, "getPorosity<float|double>");
    if (mask.type() != TYPE_UCHAR || !mask.getPtr().getCPU()) {
        std::cerr << "Mask must by type uchar with its host copy present" << std::endl;
        return T(0);
    }
    const ivec3 d = mask.dim();
    double phi = 0.0;
    const int st = fast_porosity(static_cast<const uint8_t *>(mask.getPtr().getCPU()), d.x, d.y, d.z, &phi, nullptr);
    if (st != FAST_OK) {
        std::cerr << fast_last_error() << std::endl;
        return T(0);
    }
    return T(phi);
}

template <typename T>
inline T getTortuosity(const Volume &mask, const TortuosityParams &params,
                       DiffusionSolverType solverType = DSOLVER_BICGSTAB, Volume *concetrationOutput = nullptr,
                       size_t *iterationsOut = nullptr)
{
    static_assert(std::is_same<T, float>::value || std::is_same<T, double>::value, "getTortuosity<float|double>");
    if (mask.type() != TYPE_UCHAR) {
        std::cerr << "Mask must by type uchar" << std::endl;
        return T(0);
    }
    const void *data = mask.getPtr().getCPU();
    if (!data) {
        std::cerr << "Mask must be allocated and retrieved to CPU" << std::endl;
        return T(0);
    }
    if (params.useNonUniform) {
        std::cerr << "useNonUniform is not supported" << std::endl;
        return T(0);
    }
    const ivec3 d = mask.dim();
    void *conc = nullptr;
    if (concetrationOutput && params.onDevice) {
        const ivec3 cd = concetrationOutput->dim();
        if (concetrationOutput->type() != primitiveTypeof<T>() || cd.x != d.x || cd.y != d.y || cd.z != d.z) {
            std::cerr << "Concentration output must be a volume of T with the mask's dimensions" << std::endl;
            return T(0);
        }
        if (!concetrationOutput->getPtr().getCPU())
            concetrationOutput->getPtr().allocCPU(concetrationOutput->totalElems() * sizeof(T));
        conc = concetrationOutput->getPtr().getCPU();
    }
    fast_tau_params p;
    fast_tau_params_init(&p);
    p.dir = (int32_t)params.dir;
    p.solver = solverType == DSOLVER_CG ? FAST_SOLVER_CG : FAST_SOLVER_BICGSTAB;
    p.precision = std::is_same<T, double>::value ? FAST_PREC_F64 : FAST_PREC_F32;
    p.tolerance = params.tolerance;
    p.max_iter = (uint64_t)params.maxIter;
    p.d0 = (double)params.coeffs[0];
    p.d1 = (double)params.coeffs[1];
    p.porosity = params.porosityPrecomputed ? params.porosity : -1.0;
    p.verbose = params.verbose ? 1 : 0;
    double tau = 0.0;
    uint64_t iters = 0;
    const int st = fast_tau_solve(static_cast<const uint8_t *>(data), d.x, d.y, d.z, &p, &tau, &iters, nullptr, conc);
    if (iterationsOut) *iterationsOut = (size_t)iters;
    if (st != FAST_OK) {
        std::cerr << fast_last_error() << std::endl;
        return T(0);
    }
    return T(tau);
}

}  // namespace fast
