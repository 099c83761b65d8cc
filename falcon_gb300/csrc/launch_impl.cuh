// launch_impl.cuh -- host launchers of the step kernels for one precision.
// Included once by mhd_fp64.cu (FALCON_T=double, FALCON_SFX=fp64) and once by
// mhd_mixed.cu (FALCON_T=float, FALCON_SFX=mixed).
#pragma once
#include "mhd_impl.cuh"

namespace falcon {
namespace impl {

template <class T> struct Cfg;   // KPAR per block size and precision
template <> struct Cfg<double> { static constexpr int K8 = 4, K16 = 2; };
template <> struct Cfg<float> { static constexpr int K8 = 8, K16 = 2; };

template <class T, int N, int KP>
cudaError_t stage_n(const StepDims& d, const Geometry& g, const T* in, const T* un, T* out, int stage,
                    int bcw, const StepScalars* sc, int heat, cudaStream_t st) {
    using S = Shape<T, N, N, N, KP>;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_stage<T, N, N, N, KP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)S::smem_stage);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    k_stage<T, N, N, N, KP><<<d.nblocks, S::NT, S::smem_stage, st>>>(in, un, out, g, sc, stage, bcw, heat);
    return cudaGetLastError();
}

template <class T, int N, int KP>
cudaError_t diff_n(const StepDims& d, const Geometry& g, T* u, const StepScalars* sc, cudaStream_t st) {
    using S = Shape<T, N, N, N, KP>;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_diffusion<T, N, N, N, KP>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::smem_diff);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    k_diffusion<T, N, N, N, KP><<<d.nblocks, S::NT, S::smem_diff, st>>>(u, g, sc);
    return cudaGetLastError();
}

template <class T>
cudaError_t stage_any(const StepDims& d, const Geometry& g, const T* in, const T* un, T* out, int stage, int bcw,
                      const StepScalars* sc, int heat, cudaStream_t st) {
    if (d.ni == 8 && d.nj == 8 && d.nk == 8) return stage_n<T, 8, Cfg<T>::K8>(d, g, in, un, out, stage, bcw, sc, heat, st);
    if (d.ni == 16 && d.nj == 16 && d.nk == 16)
        return stage_n<T, 16, Cfg<T>::K16>(d, g, in, un, out, stage, bcw, sc, heat, st);
    return cudaErrorInvalidValue;
}

template <class T>
cudaError_t diff_any(const StepDims& d, const Geometry& g, T* u, const StepScalars* sc, cudaStream_t st) {
    if (d.ni == 8 && d.nj == 8 && d.nk == 8) return diff_n<T, 8, Cfg<T>::K8>(d, g, u, sc, st);
    if (d.ni == 16 && d.nj == 16 && d.nk == 16) return diff_n<T, 16, Cfg<T>::K16>(d, g, u, sc, st);
    return cudaErrorInvalidValue;
}

template <class T>
cudaError_t cfl_any(const StepDims& d, const Geometry& g, const T* u, StepScalars* sc, cudaStream_t st) {
    const int nint = d.ni * d.nj * d.nk;
    dim3 grid((nint + 255) / 256, d.nblocks);
    k_cfl<T><<<grid, 256, 0, st>>>(u, g, sc, d);
    return cudaGetLastError();
}

template <class T>
cudaError_t ghost_any(const StepDims& d, const GhostCopyList& cp, const GhostInterpList& ip, T* u, cudaStream_t st) {
    if (cp.n > 0) {
        dim3 grid((unsigned)((cp.n + 255) / 256), NV);
        k_ghost_copy<T><<<grid, 256, 0, st>>>(u, cp, d.ncell);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (ip.n > 0) {
        k_ghost_interp<T><<<(unsigned)((ip.n + 127) / 128), 128, 0, st>>>(u, ip, d.ncell, d.nip, d.nip * d.njp);
        return cudaGetLastError();
    }
    return cudaSuccess;
}

}  // namespace impl
}  // namespace falcon
