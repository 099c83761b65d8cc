// lcc.h -- internal interface of the learned coarse-correction network (lcc.cu)
// used by the solver (solver.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

struct falcon_lcc;

namespace falcon {
namespace lcc {
// y[v] = net(x)[v] for x [n][D][H][W][8] FP32 on the device, y [n][D][H][W]
// FP32 on the device, enqueued on `st` (the network's buffers are resized on
// the first call for a shape; later calls with the same shape allocate nothing).
cudaError_t forward_device(falcon_lcc* net, const float* x, int n, int D, int H, int W, float* y, cudaStream_t st);
}  // namespace lcc
}  // namespace falcon
