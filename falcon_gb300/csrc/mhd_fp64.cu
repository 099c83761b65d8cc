// mhd_fp64.cu -- FP64 instantiation of the step kernels.
// Compiled with -fmad=false: no multiply-add contraction, so every result is
// rounded exactly where the reference rounds (it is built without FMA).
#include "launch_impl.cuh"

namespace falcon {
using impl::stage_any;
using impl::diff_any;
using impl::cfl_any;
using impl::ghost_any;

cudaError_t launch_stage_fp64(const StepDims& d, const Geometry& g, const double* in, const double* un, double* out,
                              const DivBArgs& psi, int stage, int bcw, StepScalars* sc, int heat, int kpar,
                              cudaStream_t st) {
    return stage_any<double>(d, g, in, un, out, nullptr, PushTable{}, psi, stage, bcw, sc, heat, kpar, st);
}
cudaError_t launch_psi_diffusion_fp64(const StepDims& d, const Geometry& g, const double* u, const double* psi,
                                      double* psi_out, StepScalars* sc, cudaStream_t st) {
    return impl::psi_diffusion_any<double>(d, g, u, psi, psi_out, sc, st);
}
cudaError_t launch_psi_ghost_fp64(const StepDims& d, const GhostLists& gl, double* psi, cudaStream_t st) {
    return impl::psi_ghost_any<double>(d, gl, psi, st);
}
cudaError_t launch_diffusion_fp64(const StepDims& d, const Geometry& g, double* u, StepScalars* sc,
                                  int kpar, cudaStream_t st) {
    return diff_any<double>(d, g, u, u, nullptr, PushTable{}, sc, kpar, st);
}
cudaError_t launch_cfl_fp64(const StepDims& d, const Geometry& g, const double* u, StepScalars* sc, cudaStream_t st) {
    return cfl_any<double>(d, g, u, sc, st);
}
cudaError_t launch_ghost_fp64(const StepDims& d, const GhostLists& gl, double* u, cudaStream_t st) {
    return ghost_any<double>(d, gl, u, st);
}
cudaError_t launch_shard_pack_fp64(const StepDims& d, const GhostInterpList& L, const double* u, double* pack,
                                   cudaStream_t st) {
    if (L.n == 0) return cudaSuccess;
    impl::k_shard_pack<double><<<(unsigned)((L.n + 127) / 128), 128, 0, st>>>(u, L, d.ncell, d.nip, d.nip * d.njp, pack);
    return cudaGetLastError();
}
cudaError_t launch_shard_unpack_fp64(const StepDims& d, const int32_t* dst, int64_t n, const double* pack, double* u,
                                     cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    impl::k_shard_unpack<double><<<(unsigned)((n + 127) / 128), 128, 0, st>>>(u, dst, n, d.ncell, pack);
    return cudaGetLastError();
}

// dt = min(1.e20, CFL*min(h/v_wave)) (3_6/ModTimeStep.f90:20-29); also the
// per-stage FP32 factors of the mixed path and the reset of the accumulator.
__global__ void k_finalize_dt(StepScalars* sc) { impl::finalize_dt_body(sc); }
cudaError_t launch_finalize_dt(StepScalars* sc, cudaStream_t st) {
    k_finalize_dt<<<1, 1, 0, st>>>(sc);
    return cudaGetLastError();
}

// Host block arrays carry FALCON_NVAR = 9 variables ([b][9][cell], psi last);
// the device state carries the 8 evolved ones ([b][8][cell]) and, with GLM,
// psi in an array of its own ([b][cell]).
__device__ __forceinline__ int64_t host_index(int64_t x, int64_t ncell) {   // device state element -> host element
    const int64_t b = x / (NV * ncell);
    return x + b * ncell;
}

// FP64 host array -> compensated FP32 state: hi = RN(u); interior cells get
// the correction of u - hi, ghost cells q = 0
__global__ void k_narrow(const double* s, float* d, int8_t* lo, int64_t n, StepDims dm) {
    for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
        const double u = s[host_index(x, dm.ncell)];
        const float hi = (float)u;
        d[x] = hi;
        if (lo) {
            const int64_t q = lo_index(x, dm);
            if (q >= 0) lo[q] = lo_encode64(hi, u - (double)hi);
        }
    }
}
// psi plane of the host array -> FP32 psi array (mixed GLM)
__global__ void k_narrow_psi(const double* s, float* psi, int64_t nb, int64_t ncell) {
    for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < nb * ncell; x += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = x / ncell;
        psi[x] = (float)s[(b * (NV + 1) + NV) * ncell + (x - b * ncell)];
    }
}
// flag = 1 if any psi value of the host array (already on the device) is
// not 0 (NaN counts as not 0)
__global__ void k_psi_nonzero(const double* s, int64_t nb, int64_t ncell, int32_t* flag) {
    int any = 0;
    for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < nb * ncell; x += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = x / ncell;
        any |= s[(b * (NV + 1) + NV) * ncell + (x - b * ncell)] != 0.0;
    }
    if (__any_sync(0xffffffffu, any) && (threadIdx.x & 31) == 0) *flag = 1;
}
// host elements [first, first + count) as FP64 from the device state (FP32
// with its correction, or FP64) and psi (nullptr: psi = 0)
template <class T>
__global__ void k_gather_host(const T* U, const int8_t* lo, const T* psi, StepDims dm, int64_t first, int64_t count,
                              int64_t ncell, double* out) {
    for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < count; x += (int64_t)gridDim.x * blockDim.x) {
        const int64_t h = first + x;
        const int64_t b = h / ((NV + 1) * ncell), r = h - b * (NV + 1) * ncell;
        double v;
        if (r < NV * ncell) {
            const int64_t e = b * NV * ncell + r;
            const T hi = U[e];
            v = (double)hi;
            if constexpr (sizeof(T) == 4) {
                const int64_t q = lo ? lo_index(e, dm) : -1;
                if (q >= 0) v += (double)lo[q] * (double)lo_unit((float)hi);
            }
        } else {
            v = psi ? (double)psi[b * ncell + (r - NV * ncell)] : 0.0;
        }
        out[x] = v;
    }
}
// Wide forms of the transfer kernels: each thread moves kWide elements per
// pass as kWide/2 16-byte accesses, all issued before any is used (a warp's
// access q covers 512 contiguous bytes), so that many bytes are in flight when
// the FP64 side is host memory read or written in place over the host link. They need 16-byte-aligned FP64
// arrays, an even cell count and even ranges (pairs never straddle a
// variable); the launchers fall back to the one-element kernels otherwise.
constexpr int kWide = 8;
__device__ __forceinline__ void narrow_one(double u, int64_t x, float* d, int8_t* lo, const StepDims& dm) {
    const float hi = (float)u;
    d[x] = hi;
    if (lo) {
        const int64_t q = lo_index(x, dm);
        if (q >= 0) lo[q] = lo_encode64(hi, u - (double)hi);
    }
}
__global__ void k_narrow_wide(const double* s, float* d, int8_t* lo, int64_t n, StepDims dm) {
    const int64_t lane2 = 2 * (threadIdx.x & 31);
    for (int64_t w0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32 * kWide; w0 < n;
         w0 += (((int64_t)gridDim.x * blockDim.x) >> 5) * 32 * kWide) {
        double2 v[kWide / 2];
#pragma unroll
        for (int q = 0; q < kWide / 2; ++q)
            if ((w0 + 64 * q + lane2) < n) v[q] = *reinterpret_cast<const double2*>(s + host_index((w0 + 64 * q + lane2), dm.ncell));
#pragma unroll
        for (int q = 0; q < kWide / 2; ++q)
            if ((w0 + 64 * q + lane2) < n) {
                narrow_one(v[q].x, (w0 + 64 * q + lane2), d, lo, dm);
                narrow_one(v[q].y, (w0 + 64 * q + lane2) + 1, d, lo, dm);
            }
    }
}
__device__ __forceinline__ int64_t psi_host_index(int64_t x, int64_t ncell) {   // psi element -> host element
    const int64_t b = x / ncell;
    return (b * (NV + 1) + NV) * ncell + (x - b * ncell);
}
__global__ void k_narrow_psi_wide(const double* s, float* psi, int64_t nb, int64_t ncell) {
    const int64_t n = nb * ncell;
    const int64_t lane2 = 2 * (threadIdx.x & 31);
    for (int64_t w0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32 * kWide; w0 < n;
         w0 += (((int64_t)gridDim.x * blockDim.x) >> 5) * 32 * kWide) {
        double2 v[kWide / 2];
#pragma unroll
        for (int q = 0; q < kWide / 2; ++q)
            if ((w0 + 64 * q + lane2) < n) v[q] = *reinterpret_cast<const double2*>(s + psi_host_index((w0 + 64 * q + lane2), ncell));
#pragma unroll
        for (int q = 0; q < kWide / 2; ++q)
            if ((w0 + 64 * q + lane2) < n) {
                psi[(w0 + 64 * q + lane2)] = (float)v[q].x;
                psi[(w0 + 64 * q + lane2) + 1] = (float)v[q].y;
            }
    }
}
__global__ void k_psi_nonzero_wide(const double* s, int64_t nb, int64_t ncell, int32_t* flag) {
    const int64_t n = nb * ncell;
    int any = 0;
    const int64_t lane2 = 2 * (threadIdx.x & 31);
    for (int64_t w0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32 * kWide; w0 < n;
         w0 += (((int64_t)gridDim.x * blockDim.x) >> 5) * 32 * kWide) {
        double2 v[kWide / 2];
#pragma unroll
        for (int q = 0; q < kWide / 2; ++q)
            if ((w0 + 64 * q + lane2) < n) v[q] = *reinterpret_cast<const double2*>(s + psi_host_index((w0 + 64 * q + lane2), ncell));
#pragma unroll
        for (int q = 0; q < kWide / 2; ++q)
            if ((w0 + 64 * q + lane2) < n) any |= (v[q].x != 0.0) | (v[q].y != 0.0);
    }
    if (__any_sync(0xffffffffu, any) && (threadIdx.x & 31) == 0) *flag = 1;
}
template <class T>
__device__ __forceinline__ double gather_one(const T* U, const int8_t* lo, const T* psi, int64_t h, int64_t ncell,
                                             const StepDims& dm) {
    const int64_t b = h / ((NV + 1) * ncell), r = h - b * (NV + 1) * ncell;
    if (r < NV * ncell) {
        const int64_t e = b * NV * ncell + r;
        const T hi = U[e];
        double v = (double)hi;
        if constexpr (sizeof(T) == 4) {
            const int64_t q = lo ? lo_index(e, dm) : -1;
            if (q >= 0) v += (double)lo[q] * (double)lo_unit((float)hi);
        }
        return v;
    }
    return psi ? (double)psi[b * ncell + (r - NV * ncell)] : 0.0;
}
template <class T>
__global__ void k_gather_host_wide(const T* U, const int8_t* lo, const T* psi, StepDims dm, int64_t first,
                                   int64_t count, int64_t ncell, double* out) {
    const int64_t lane2 = 2 * (threadIdx.x & 31);
    for (int64_t w0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32 * kWide; w0 < count;
         w0 += (((int64_t)gridDim.x * blockDim.x) >> 5) * 32 * kWide) {
        double2 v[kWide / 2];
#pragma unroll
        for (int q = 0; q < kWide / 2; ++q)
            if ((w0 + 64 * q + lane2) < count) {
                v[q].x = gather_one(U, lo, psi, first + (w0 + 64 * q + lane2), ncell, dm);
                v[q].y = gather_one(U, lo, psi, first + (w0 + 64 * q + lane2) + 1, ncell, dm);
            }
#pragma unroll
        for (int q = 0; q < kWide / 2; ++q)
            if ((w0 + 64 * q + lane2) < count) *reinterpret_cast<double2*>(out + (w0 + 64 * q + lane2)) = v[q];
    }
}
bool wide_ok(const void* p, int64_t ncell) { return ((uintptr_t)p % 16) == 0 && ncell % 2 == 0; }

// Core transfers: of every block and variable of the host array (9 per block,
// psi last), the interior planes and within them the interior rows, each
// row whole (its radial ghost columns, which hold the radial boundary
// condition, included). The interior rows of one plane are one contiguous
// run of (NJP-4)*NIP host elements: a warp moves one run at a time, block,
// variable and plane from the run number, the cell from the offset in the
// run, so no element pays a 64-bit division; each lane's 16-byte host
// accesses of a pass (kRunVec, a whole 16^3 run of 320 elements) are issued
// before any is used. Offsets are even and NIP is even, so a pair (ip, ip+1)
// is either two radial ghost columns or two interior cells, and its device
// side is one 8-byte (FP32) or 16-byte (FP64) access and one 2-byte access
// of the correction.
constexpr int kRunVec = 5;
struct CoreRun {
    int64_t host;   // host element of the run's first cell
    int64_t dev;    // state element of that cell ((b NV + v) ncell + cell0), v < NV
    int64_t psi;    // psi element of that cell (b ncell + cell0)
    int64_t lo0;    // correction element of the run's first interior row
    int v;          // 0..NV-1 state, NV psi
};
__device__ __forceinline__ CoreRun core_run(int64_t r, const StepDims& dm) {
    const int nkc = dm.nkp - 4;
    const int64_t bv = r / nkc, b = bv / (NV + 1);
    const int kp = 2 + (int)(r - bv * nkc);
    const int64_t cell0 = (int64_t)kp * dm.nip * dm.njp + 2 * dm.nip;
    CoreRun c;
    c.v = (int)(bv - b * (NV + 1));
    c.host = bv * dm.ncell + cell0;
    c.dev = (b * NV + c.v) * dm.ncell + cell0;
    c.psi = b * dm.ncell + cell0;
    c.lo0 = ((b * NV + c.v) * dm.nk + (kp - 2)) * (int64_t)dm.nj * dm.ni;
    return c;
}
// host core -> device: state cells narrowed (FP32 with its correction) or
// copied (FP64); psi converted into P, or, without P, tested for 0 (flag)
template <class T>
__global__ void k_core_up(const double* s, T* U, int8_t* lo, T* P, int32_t* flag, int64_t nruns, StepDims dm) {
    const int lane2 = 2 * (threadIdx.x & 31), len = (dm.njp - 4) * dm.nip;
    int any = 0;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < nruns;
         r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
        const CoreRun c = core_run(r, dm);
        for (int o0 = 0; o0 < len; o0 += 64 * kRunVec) {
            double2 v[kRunVec];
#pragma unroll
            for (int q = 0; q < kRunVec; ++q)
                if (o0 + 64 * q + lane2 < len) v[q] = *reinterpret_cast<const double2*>(s + c.host + o0 + 64 * q + lane2);
#pragma unroll
            for (int q = 0; q < kRunVec; ++q) {
                const int o = o0 + 64 * q + lane2;
                if (o >= len) continue;
                if (c.v < NV) {
                    if constexpr (sizeof(T) == 4) {
                        const float h0 = (float)v[q].x, h1 = (float)v[q].y;
                        *reinterpret_cast<float2*>(U + c.dev + o) = make_float2(h0, h1);
                        const int jr = o / dm.nip, ip = o - jr * dm.nip;
                        if (lo && ip >= 2 && ip < dm.nip - 2) {
                            char2 q2;
                            q2.x = lo_encode64(h0, v[q].x - (double)h0);
                            q2.y = lo_encode64(h1, v[q].y - (double)h1);
                            *reinterpret_cast<char2*>(lo + c.lo0 + jr * dm.ni + (ip - 2)) = q2;
                        }
                    } else {
                        *reinterpret_cast<double2*>(U + c.dev + o) = v[q];
                    }
                } else if (P) {
                    if constexpr (sizeof(T) == 4) *reinterpret_cast<float2*>(P + c.psi + o) = make_float2((float)v[q].x, (float)v[q].y);
                    else *reinterpret_cast<double2*>(P + c.psi + o) = v[q];
                } else {
                    any |= (v[q].x != 0.0) | (v[q].y != 0.0);
                }
            }
        }
    }
    if (flag && __any_sync(0xffffffffu, any) && (threadIdx.x & 31) == 0) *flag = 1;
}
// device -> host core (psi 0 without P)
template <class T>
__global__ void k_core_down(const T* U, const int8_t* lo, const T* P, double* out, int64_t nruns, StepDims dm) {
    const int lane2 = 2 * (threadIdx.x & 31), len = (dm.njp - 4) * dm.nip;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < nruns;
         r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
        const CoreRun c = core_run(r, dm);
        for (int o0 = 0; o0 < len; o0 += 64 * kRunVec) {
            double2 v[kRunVec];
#pragma unroll
            for (int q = 0; q < kRunVec; ++q) {
                const int o = o0 + 64 * q + lane2;
                if (o >= len) continue;
                if (c.v < NV) {
                    if constexpr (sizeof(T) == 4) {
                        const float2 h = *reinterpret_cast<const float2*>(U + c.dev + o);
                        v[q] = make_double2((double)h.x, (double)h.y);
                        const int jr = o / dm.nip, ip = o - jr * dm.nip;
                        if (lo && ip >= 2 && ip < dm.nip - 2) {
                            const char2 q2 = *reinterpret_cast<const char2*>(lo + c.lo0 + jr * dm.ni + (ip - 2));
                            v[q].x += (double)q2.x * (double)lo_unit(h.x);
                            v[q].y += (double)q2.y * (double)lo_unit(h.y);
                        }
                    } else {
                        v[q] = *reinterpret_cast<const double2*>(U + c.dev + o);
                    }
                } else if (P) {
                    if constexpr (sizeof(T) == 4) {
                        const float2 h = *reinterpret_cast<const float2*>(P + c.psi + o);
                        v[q] = make_double2((double)h.x, (double)h.y);
                    } else {
                        v[q] = *reinterpret_cast<const double2*>(P + c.psi + o);
                    }
                } else {
                    v[q] = make_double2(0.0, 0.0);
                }
            }
#pragma unroll
            for (int q = 0; q < kRunVec; ++q)
                if (o0 + 64 * q + lane2 < len) *reinterpret_cast<double2*>(out + c.host + o0 + 64 * q + lane2) = v[q];
        }
    }
}
int64_t core_runs(const StepDims& dm) { return (int64_t)dm.nblocks * (NV + 1) * (dm.nkp - 4); }
bool core_ok(const void* host, const StepDims& dm) {
    return ((uintptr_t)host % 16) == 0 && dm.ncell % 2 == 0 && dm.nip % 2 == 0;
}

cudaError_t launch_convert_state(const double* src, float* dst, int8_t* lo, int64_t n, const StepDims& dm,
                                 cudaStream_t st) {
    if (wide_ok(src, dm.ncell) && n % 2 == 0) k_narrow_wide<<<1216, 256, 0, st>>>(src, dst, lo, n, dm);
    else k_narrow<<<1216, 256, 0, st>>>(src, dst, lo, n, dm);
    return cudaGetLastError();
}
cudaError_t launch_convert_psi(const double* src, float* psi, int64_t nb, int64_t ncell, cudaStream_t st) {
    if (wide_ok(src, ncell)) k_narrow_psi_wide<<<1216, 256, 0, st>>>(src, psi, nb, ncell);
    else k_narrow_psi<<<1216, 256, 0, st>>>(src, psi, nb, ncell);
    return cudaGetLastError();
}
cudaError_t launch_psi_nonzero(const double* src, int64_t nb, int64_t ncell, int32_t* flag, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int32_t), st);
    if (e != cudaSuccess) return e;
    if (wide_ok(src, ncell)) k_psi_nonzero_wide<<<1216, 256, 0, st>>>(src, nb, ncell, flag);
    else k_psi_nonzero<<<1216, 256, 0, st>>>(src, nb, ncell, flag);
    return cudaGetLastError();
}
cudaError_t launch_gather_host(const void* U, const int8_t* lo, const void* psi, bool fp32, const StepDims& dm,
                               int64_t first, int64_t count, int64_t ncell, double* out, cudaStream_t st) {
    const bool wide = wide_ok(out, ncell) && first % 2 == 0 && count % 2 == 0;
    if (fp32) {
        if (wide)
            k_gather_host_wide<float><<<1216, 256, 0, st>>>((const float*)U, lo, (const float*)psi, dm, first, count, ncell,
                                                            out);
        else k_gather_host<float><<<1216, 256, 0, st>>>((const float*)U, lo, (const float*)psi, dm, first, count, ncell, out);
    } else {
        if (wide)
            k_gather_host_wide<double><<<1216, 256, 0, st>>>((const double*)U, nullptr, (const double*)psi, dm, first, count,
                                                             ncell, out);
        else
            k_gather_host<double><<<1216, 256, 0, st>>>((const double*)U, nullptr, (const double*)psi, dm, first, count,
                                                        ncell, out);
    }
    return cudaGetLastError();
}

cudaError_t launch_core_up(const double* host, void* U, int8_t* lo, void* P, int32_t* flag, bool fp32, const StepDims& dm,
                           cudaStream_t st) {
    if (!core_ok(host, dm)) return cudaErrorInvalidValue;
    const int64_t n = core_runs(dm);
    if (flag) {
        cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int32_t), st);
        if (e != cudaSuccess) return e;
    }
    if (fp32) k_core_up<float><<<1216, 256, 0, st>>>(host, (float*)U, lo, (float*)P, flag, n, dm);
    else k_core_up<double><<<1216, 256, 0, st>>>(host, (double*)U, nullptr, (double*)P, flag, n, dm);
    return cudaGetLastError();
}
cudaError_t launch_core_down(const void* U, const int8_t* lo, const void* P, bool fp32, double* host, const StepDims& dm,
                             cudaStream_t st) {
    if (!core_ok(host, dm)) return cudaErrorInvalidValue;
    const int64_t n = core_runs(dm);
    if (fp32) k_core_down<float><<<1216, 256, 0, st>>>((const float*)U, lo, (const float*)P, host, n, dm);
    else k_core_down<double><<<1216, 256, 0, st>>>((const double*)U, nullptr, (const double*)P, host, n, dm);
    return cudaGetLastError();
}

int kpar_candidates_fp64(const StepDims& d, int* out) { return impl::candidates<double>(d, out); }

}  // namespace falcon
