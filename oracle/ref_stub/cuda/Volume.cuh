// Stand-in for fastlib/src/cuda/Volume.cuh when the reference's assembly
// header (fastlib/src/cuda/Diffusion.cuh) is compiled for the host by
// oracle/Makefile's `ref` target.  TEST INFRASTRUCTURE ONLY.
//
// Diffusion.cuh needs from Volume.cuh only what the reference's own
// fastlib/src/cuda/VolumeTypes.cuh declares (Dir helpers _getDirIndex,
// _getDirSgn, _getDir, CUDA_Volume), which is included unchanged, and
// fast::ivec3, which the reference takes from glm (an empty submodule here):
// a minimal integer 3-vector with glm's .x/.y/.z layout and operator[].
#pragma once
#include "cuda/VolumeTypes.cuh"

namespace fast {
struct ivec3 {
    int x, y, z;
    __host__ __device__ int &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    __host__ __device__ const int &operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
}  // namespace fast
