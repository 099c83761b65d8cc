// state_range.cu -- download a range of the state without allocating.
//
// falcon_download_state converts the device state (FP32 in MIXED mode, and
// always without psi's plane when GLM is off) through an FP64 device staging
// buffer of the whole host array, allocated on first use. The range download
// here gathers through one fixed array compiled into the library instead, so
// it needs no cudaMalloc, no cudaFree and no host allocation.
//
// The array is shared by every context on a device and keeps what the last
// call wrote into it. Each call overwrites the part it reads back (the first
// `count` elements), so no part of it has to start at zero. A call finishes
// with a stream synchronise, so calls made one after another never overlap;
// calls that overlap on the GPU (several host threads, several contexts on one
// device) race on the array and must be serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/falcon_gb300.h"
#include "kernels.cuh"

// FALCON_STATIC_SCRATCH_BYTES (16 MiB) of FP64 staging, 256-byte aligned.
static __device__ __align__(256) double g_range_scratch[FALCON_STATIC_SCRATCH_BYTES / sizeof(double)];

namespace falcon {

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
double* g_scratch_ptr[kMaxDevices] = {};

// The array's device address on device `dev`, which must be current. Resolved
// once per device (the first call may also load the library's device code on
// that device) and cached for the life of the process: the cache assumes that
// the device's primary context (which every context of this library uses)
// lives as long as the process. After a cudaDeviceReset, or another reset of
// the primary context in the same process, the cached address is stale; do not
// call this entry point after one.
cudaError_t scratch_on_device(int dev, double** out) {
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        double* ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_range_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = ptr;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}
}  // namespace

size_t static_scratch_elems() { return FALCON_STATIC_SCRATCH_BYTES / sizeof(double); }

// Copy host-layout elements [first, first + count) ([b][9][cell], psi last)
// of the device state (FP32 with its correction Ulo if mixed, else FP64) and
// psi (P, nullptr: 0) to host u as FP64, through the static array. The caller
// has checked the range and count <= static_scratch_elems(), and made `dev`
// current. Returns "" or the failing step.
std::string download_range_static(int dev, cudaStream_t st, const void* U, const int8_t* Ulo, const void* P,
                                  bool mixed, const StepDims& dm, size_t first, size_t count, double* u) {
    if (count == 0) return "";
    double* ptr = nullptr;
    cudaError_t e = scratch_on_device(dev, &ptr);
    if (e != cudaSuccess) return std::string("static scratch address: ") + cudaGetErrorString(e);
    e = launch_gather_host(U, mixed ? Ulo : nullptr, P, mixed, dm, (int64_t)first, (int64_t)count, (int64_t)dm.ncell, ptr,
                           st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(u, ptr, count * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return std::string("range download: ") + cudaGetErrorString(e);
    return "";
}

}  // namespace falcon
