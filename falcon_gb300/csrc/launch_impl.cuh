// launch_impl.cuh -- host launchers of the step kernels for one precision.
// Included once by mhd_fp64.cu (FALCON_T=double, FALCON_SFX=fp64) and once by
// mhd_mixed.cu (FALCON_T=float, FALCON_SFX=mixed).
#pragma once
#include "mhd_impl.cuh"

namespace falcon {
namespace impl {

// k-chunk depths (KPAR) instantiated per block size and precision; the
// context's autotuner times them on its own grid and keeps the fastest.
template <class T> struct Cand;
template <> struct Cand<double> {
    static constexpr int n8 = 2, n16 = 1;
    static constexpr int k8[2] = {2, 4};
    static constexpr int k16[1] = {1};
};
template <> struct Cand<float> {
    static constexpr int n8 = 3, n16 = 3;
    static constexpr int k8[3] = {2, 4, 8};
    static constexpr int k16[3] = {1, 2, 4};
};

template <class T, int N, int KP, int DIVB>
cudaError_t stage_nd(const StepDims& d, const Geometry& g, const T* in, const T* un, T* out, int8_t* lo,
                     const PushTable& push, const DivBArgs& psi, int stage, int bcw, StepScalars* sc, int heat,
                     cudaStream_t st) {
    using S = Shape<T, N, N, N, KP>;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_stage<T, N, N, N, KP, DIVB>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::smem_stage);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    k_stage<T, N, N, N, KP, DIVB>
        <<<d.nblocks, S::NT, S::smem_stage, st>>>(in, un, out, lo, push, psi, g, sc, stage, bcw, heat);
    return cudaGetLastError();
}

// The div-B mode is a template parameter: the plain stage keeps its register
// allocation free of the GLM/Powell terms.
template <class T, int N, int KP>
cudaError_t stage_n(const StepDims& d, const Geometry& g, const T* in, const T* un, T* out, int8_t* lo,
                    const PushTable& push, const DivBArgs& psi, int stage, int bcw, StepScalars* sc, int heat,
                    cudaStream_t st) {
    switch (psi.mode) {
    case 0: return stage_nd<T, N, KP, 0>(d, g, in, un, out, lo, push, psi, stage, bcw, sc, heat, st);
    case 1:
        if (!psi.in || !psi.un || !psi.out) return cudaErrorInvalidValue;
        return stage_nd<T, N, KP, 1>(d, g, in, un, out, lo, push, psi, stage, bcw, sc, heat, st);
    case 2: return stage_nd<T, N, KP, 2>(d, g, in, un, out, lo, push, psi, stage, bcw, sc, heat, st);
    default: return cudaErrorInvalidValue;
    }
}

template <class T, int N, int KP>
cudaError_t diff_n(const StepDims& d, const Geometry& g, const T* u, T* out, int8_t* lo, const PushTable& push,
                   StepScalars* sc, int cfl_next, cudaStream_t st) {
    using S = DShape<T, N, N, N, KP>;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_diffusion<T, N, N, N, KP>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    k_diffusion<T, N, N, N, KP><<<d.nblocks, S::NT, S::smem, st>>>(u, out, lo, push, g, sc, cfl_next);
    return cudaGetLastError();
}

template <class T>
cudaError_t stage_any(const StepDims& d, const Geometry& g, const T* in, const T* un, T* out, int8_t* lo,
                      const PushTable& push, const DivBArgs& psi, int stage, int bcw, StepScalars* sc, int heat, int kpar,
                      cudaStream_t st) {
#define FALCON_STAGE_CASE(N, K) \
    if (d.ni == N && kpar == K) return stage_n<T, N, K>(d, g, in, un, out, lo, push, psi, stage, bcw, sc, heat, st);
    if (d.ni != d.nj || d.ni != d.nk) return cudaErrorInvalidValue;
    FALCON_STAGE_CASE(8, 2) FALCON_STAGE_CASE(8, 4)
    FALCON_STAGE_CASE(16, 1)
    if constexpr (!Pol<T>::exact) { FALCON_STAGE_CASE(8, 8) FALCON_STAGE_CASE(16, 2) FALCON_STAGE_CASE(16, 4) }
#undef FALCON_STAGE_CASE
    return cudaErrorInvalidValue;
}

// FP32 16^3 blocks: the k-march kernel; the k-chunk depth asked for selects
// one thread per column (1) or two (2 and 4)
template <int TPC>
cudaError_t diff_march16(const StepDims& d, const Geometry& g, const float* u, float* out, int8_t* lo,
                         const PushTable& push, StepScalars* sc, int cfl_next, cudaStream_t st) {
    using S = MShape<16, 16, 16, TPC>;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_diffusion_march<16, 16, 16, TPC>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    k_diffusion_march<16, 16, 16, TPC><<<d.nblocks, S::NT, S::smem, st>>>(u, out, lo, push, g, sc, cfl_next);
    return cudaGetLastError();
}

// FP64 8^3 blocks: the k-march kernel, in place (any k-chunk depth asked for)
inline cudaError_t diff_march64_8(const StepDims& d, const Geometry& g, double* u, StepScalars* sc, cudaStream_t st) {
    using S = M64Shape<8, 8, 8>;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_diffusion_march64<8, 8, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)S::smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    k_diffusion_march64<8, 8, 8><<<d.nblocks, S::NT, S::smem, st>>>(u, g, sc);
    return cudaGetLastError();
}

template <class T>
cudaError_t diff_any(const StepDims& d, const Geometry& g, const T* u, T* out, int8_t* lo, const PushTable& push,
                     StepScalars* sc, int kpar, cudaStream_t st, int cfl_next = 0) {
    if (push.tgt != nullptr && out == u) return cudaErrorInvalidValue;   // pushing needs out != u
    if constexpr (Pol<T>::exact) {
        if (d.ni == 8 && d.nj == 8 && d.nk == 8 && out == u && push.tgt == nullptr)
            return diff_march64_8(d, g, out, sc, st);
    }
    if constexpr (!Pol<T>::exact) {
        if (d.ni == 16 && d.nj == 16 && d.nk == 16)
            return kpar == 1 ? diff_march16<1>(d, g, u, out, lo, push, sc, cfl_next, st)
                             : diff_march16<2>(d, g, u, out, lo, push, sc, cfl_next, st);
    }
#define FALCON_DIFF_CASE(N, K) \
    if (d.ni == N && kpar == K) return diff_n<T, N, K>(d, g, u, out, lo, push, sc, cfl_next, st);
    if (d.ni != d.nj || d.ni != d.nk) return cudaErrorInvalidValue;
    FALCON_DIFF_CASE(8, 2) FALCON_DIFF_CASE(8, 4)
    FALCON_DIFF_CASE(16, 1)
    // (16, 4) would need more than 227 KB of shared memory for its face arrays
    if constexpr (!Pol<T>::exact) { FALCON_DIFF_CASE(8, 8) }
#undef FALCON_DIFF_CASE
    return cudaErrorInvalidValue;
}

template <class T>
cudaError_t psi_diffusion_any(const StepDims& d, const Geometry& g, const T* u, const T* psi, T* psi_out,
                              StepScalars* sc, cudaStream_t st) {
    const int nint = d.ni * d.nj * d.nk;
    k_psi_diffusion<T><<<dim3((nint + 255) / 256, d.nblocks), 256, 0, st>>>(u, psi, psi_out, g, sc, d);
    return cudaGetLastError();
}

template <class T>
cudaError_t psi_ghost_any(const StepDims& d, const GhostLists& gl, T* psi, cudaStream_t st) {
    const int64_t n = gl.cp.n + gl.ln.n + gl.ip.n;
    if (n == 0) return cudaSuccess;
    k_psi_ghost<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(psi, gl, d.ncell, d.nip, d.nip * d.njp);
    return cudaGetLastError();
}

template <class T>
int candidates(const StepDims& d, int* out) {
    int n = 0;
    if (d.ni == 8) for (int q = 0; q < Cand<T>::n8; ++q) out[n++] = Cand<T>::k8[q];
    if (d.ni == 16) for (int q = 0; q < Cand<T>::n16; ++q) out[n++] = Cand<T>::k16[q];
    return n;
}

template <class T>
cudaError_t cfl_any(const StepDims& d, const Geometry& g, const T* u, StepScalars* sc, cudaStream_t st) {
    const int nint = d.ni * d.nj * d.nk;
    dim3 grid((nint + 255) / 256, d.nblocks);
    k_cfl<T><<<grid, 256, 0, st>>>(u, g, sc, d);
    return cudaGetLastError();
}

template <class T>
cudaError_t ghost_any(const StepDims& d, const GhostLists& gl, T* u, cudaStream_t st) {
    const int64_t nb_ip = (gl.ip.n + 127) / 128, nb_ln = (gl.ln.n + 127) / 128, nb_cp = (gl.cp.n + 127) / 128;
    if (nb_ip + nb_ln + nb_cp == 0) return cudaSuccess;
    if (nb_ip + nb_ln + nb_cp < (int64_t)INT32_MAX) {
        k_ghost_all<T><<<(unsigned)(nb_ip + nb_ln + nb_cp), 128, 0, st>>>(u, gl, d.ncell, d.nip, d.nip * d.njp,
                                                                          (int)nb_ip, (int)nb_ln);
        return cudaGetLastError();
    }
    if (gl.cp.n > 0) {
        k_ghost_copy<T><<<(unsigned)((gl.cp.n + 255) / 256), 256, 0, st>>>(u, gl.cp, d.ncell);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (gl.ln.n > 0) {
        k_ghost_lin<T><<<(unsigned)((gl.ln.n + 255) / 256), 256, 0, st>>>(u, gl.ln, d.ncell);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (gl.ip.n > 0) {
        k_ghost_interp<T><<<(unsigned)((gl.ip.n + 127) / 128), 128, 0, st>>>(u, gl.ip, d.ncell, d.nip, d.nip * d.njp);
        return cudaGetLastError();
    }
    return cudaSuccess;
}

}  // namespace impl
}  // namespace falcon
