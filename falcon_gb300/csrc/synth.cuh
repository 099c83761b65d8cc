// synth.cuh -- seeded synthetic initial states generated on the device.
#pragma once
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "host_setup.h"
#include "kernels.cuh"

namespace falcon {
// kind 0: Gaussian entropy bump + axisymmetric dipole B, v = 0
// kind 1: kind 0 plus a random-phase Kolmogorov velocity field scaled to rms
//         Mach `mach` against the local sound speed
// Writes every cell of U (state layout of the context; FP32 if mixed).
std::string synth_initial_state(const Grid& g, const Geometry& geo, void* U, bool mixed, int kind, uint64_t seed,
                                double mach, cudaStream_t st);
}  // namespace falcon
