// Stand-in for fastlib/src/cuda/LinearSystemDevice.cuh (thrust containers of
// the stored system), of which fastlib/src/cuda/Diffusion.cuh uses nothing in
// getSystemTopKernel.  TEST INFRASTRUCTURE ONLY; see Volume.cuh beside it.
#pragma once
