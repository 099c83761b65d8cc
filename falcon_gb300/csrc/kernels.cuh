// kernels.cuh -- device kernels of one RK4 step (templates).
//
// Instantiated twice:
//   mhd_fp64.cu  (T = double, compiled with -fmad=false): every operation in the
//                reference's order, bit-comparable with the CPU oracle;
//   mhd_mixed.cu (T = float): FP32 state and stencil RHS, p1 assembled in FP64.
//
// Data layout in HBM (one state buffer):
//   u[b][v][kp][jp][ip], ip fastest, padded extents nip=ni+4 etc. This is the
//   reference's per-block Fortran array primitive(i,j,k,var) laid end to end
//   (3_6/ModBlock.f90:275-277), so a block uploads/downloads with one memcpy.
//
// Stencil kernels run one CTA per block. The CTA owns an (i,j) interior column
// per thread (KPAR columns deep in k) and marches in k with a ring of KPAR+4
// shared-memory planes holding all 8 variables: every padded plane is read
// from HBM exactly once, and because a plane is only overwritten after the
// ring has moved past it, stages and the diffusion pass update in place.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace falcon {

enum { V_RHO1 = 0, V_VR = 1, V_VT = 2, V_VP = 3, V_BR = 4, V_BT = 5, V_BP = 6, V_S1 = 7, NV = 8 };

// ---- compensated FP32 state of the mixed path --------------------------------
// u^n is held as an FP32 value hi plus an 8-bit correction q (a second array
// with the state's layout): u = hi + q * unit(hi), unit(hi) = ulp(hi)/256 =
// 2^(e-158) for hi's biased exponent e. Rounding u^n to plain FP32 once a step
// is the dominant error of an FP32 state against FP64 (the stage buffers are
// transient and stay plain FP32); the correction keeps 8 more bits of u^n.
// Only interior cells carry a correction; ghost cells keep q = 0.
#ifdef __CUDACC__
__device__ __forceinline__ float lo_unit(float hi) {
    const int e = (__float_as_int(hi) >> 23) & 0xff;
    return e >= 32 ? __int_as_float((e - 31) << 23) : 0.f;
}
__device__ __forceinline__ float lo_inv_unit(float hi) {   // 1/unit(hi) = 2^(158-e)
    const int e = (__float_as_int(hi) >> 23) & 0xff;
    return e >= 32 ? __int_as_float((285 - e) << 23) : 0.f;
}
// q for the residual r = u - hi (|r| <= ulp(hi)/2); NaN residuals give -127.
// The clamp comes first (fmaxf of a NaN is -127) and the rounding to the
// nearest integer, ties to even, is the add of 1.5 * 2^23, whose ulp is 1:
// the same q as rintf then clamp then (int), on the full-rate FP32 and
// integer pipes instead of the conversion pipe.
__device__ __forceinline__ int8_t lo_encode(float hi, float r) {
    const float t = fminf(fmaxf(__fmul_rn(r, lo_inv_unit(hi)), -127.f), 127.f);
    return (int8_t)(__float_as_int(__fadd_rn(t, 12582912.f)) - 0x4B400000);
}
// (float)q of a correction, exactly: 2^23 + (q + 128) has ulp 1
__device__ __forceinline__ float lo_decode(int8_t q) {
    return __fsub_rn(__int_as_float(0x4B000000 + (int)q + 128), 8388736.f);
}
__device__ __forceinline__ int8_t lo_encode64(float hi, double r) {
    const double q = rint(r * (double)lo_inv_unit(hi));
    return (int8_t)(int)fmin(fmax(q, -127.0), 127.0);
}
// (hi + q*unit(hi)) + d, rounded to the nearest (hi', q') pair: two error-free
// FP32 sums (Knuth's TwoSum), no contraction (explicit _rn intrinsics)
__device__ __forceinline__ float ff_add(float hi, int8_t q, float d, int8_t& q_out) {
    const float l = __fmul_rn(lo_decode(q), lo_unit(hi));   // exact
    const float s = __fadd_rn(hi, d);
    const float bs = __fsub_rn(s, hi);
    const float es = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bs)), __fsub_rn(d, bs));
    const float t = __fadd_rn(es, l);
    const float h = __fadd_rn(s, t);
    const float bh = __fsub_rn(h, s);
    const float r = __fadd_rn(__fsub_rn(s, __fsub_rn(h, bh)), __fsub_rn(t, bh));
    q_out = lo_encode(h, r);
    return h;
}
#endif

// per-block radial (i) tables, padded length nip
enum {
    GI_R = 0,      // r (cell centres incl. ghosts)
    GI_R2,         // r*r
    GI_RINV,       // 1./r
    GI_R2INV,      // 1./(r*r)
    GI_A1,         // gamma1 * (p0/rho0)          (p1 coefficient of rho1)
    GI_A2,         // (gamma3-1) * (rho0*T0)      (p1 coefficient of s1)
    GI_RHO0,       // rho0
    GI_RHO0INV,    // 1./rho0
    GI_GOR0,       // g/rho0
    GI_HEAT,       // Artificial_heating_ratio*(diffusion+cooling)/(rho0*T0)
    GI_XI2INV,     // 1./(Xi*Xi)
    GI_CS,         // (1./Xi)*sqrt(gamma1*(p0/rho0))
    GI_COUNT
};
// per-block theta (j) tables, padded length njp
enum { GJ_SIN = 0, GJ_SININV, GJ_COT, GJ_COUNT };
// per-block scalars
enum { GS_C1 = 0, GS_C2, GS_C3, GS_DXI, GS_DXJ, GS_DXK, GS_COUNT };

struct Geometry {
    const double* gi;   // [b][GI_COUNT][nip]
    const double* gj;   // [b][GJ_COUNT][njp]
    const double* gs;   // [b][GS_COUNT]
    const float* gi_f;  // FP32 copies for the mixed path
    const float* gj_f;
    const float* gs_f;
    const int32_t* flags;  // bit0 yin, bit1 top, bit2 bottom
};

// Device-resident step scalars (written by the CFL finaliser, read by every
// stage kernel; nothing goes back to the host inside a step).
struct StepScalars {
    unsigned long long min_ratio_bits;  // atomicMin accumulator of h/v_wave (positive doubles)
    double dt;                          // CFL * min(h/v_wave), seeded with 1.e20 (FP32 literal)
    double cfl;
    float dt_stage_f[4];                // (float)(dt/(5-s)) for the mixed path
    float dt_half_f;                    // (float)(0.5*dt)
    int32_t nan_flag;                   // sticky: bit0 NaN seen in the state, bit1 a copy wait timed out
    int32_t nan_step;                   // step counter value when it was first seen
    int32_t step_counter;               // steps finalised so far (device side)
    int32_t wait_polls;                 // poll limit of the step kernels' bulk-copy waits
};

// Default poll limit of a bulk-copy wait (each poll may suspend briefly, so
// the wait is bounded in time as well as in count).
constexpr int32_t kDefaultWaitPolls = 1 << 22;

struct GhostCopyList {   // ghost cells that are exact copies (all weights zero, same panel)
    int64_t n;
    const int32_t* dst;  // element offset of var 0 of the target ghost cell
    const int32_t* src;  // element offset of var 0 of the source cell
};
struct GhostInterpList {  // trilinear (and/or Yin-Yang rotated) ghost cells
    int64_t n;
    const int32_t* dst;
    const int32_t* src;     // offset of the base cell (i0,j0,k0)
    const double* w;        // [n][3] weights wi, wj, wk
    const double* rot;      // [n][2] rotation coefficients (0 if not rotated)
    const uint8_t* kind;    // bit0: interpolate, bit1: rotate
    const float* wf;        // mixed path: FP32 copies of w and rot
    const float* rotf;
};

struct GhostLinList {     // 1-D linear ghost cells (mixed path)
    int64_t n;
    const int32_t* dst;
    const int32_t* src;
    const int32_t* stride;  // element distance to the second point (1, nip or nip*njp)
    const float* w;
};

struct GhostLists {
    GhostCopyList cp;
    GhostLinList ln;
    GhostInterpList ip;
};

// Ghost faces written by the stage kernel of the SOURCE block (mixed path).
// A face of a target block is pushed when all its ghost cells (2 layers x the
// full face) come from one source block of the same panel without rotation:
// theta/phi faces as a translation by the block extent (plain copies), radial
// faces as a 1-D blend per ghost layer of two adjacent source cells along i.
// Indexed by the source block and its side: face = 2*axis + side (side 0: the
// low side of the source, whose target lies below it on that axis).
struct PushTable {
    const int32_t* tgt;      // [b][6] target block, -1 = not pushed
    const int32_t* rad_src;  // [b][2 sides][2 layers] padded i of the first source cell
    const int32_t* rad_dst;  // [b][2][2] padded i of the target ghost cell
    const float* rad_w;      // [b][2][2] weight of the second source cell (0: copy)
};

struct StepDims {
    int nblocks, ni, nj, nk, nip, njp, nkp, ncell;
};

// The u^n correction of the mixed path is stored for interior cells only,
// [block][var][k][j][i] with the interior extents (1 byte per value, no
// padding: its rows are whole 16-byte runs for 16^3 blocks). Index of state
// element e (the state's padded layout), or -1 for a ghost cell.
__host__ __device__ __forceinline__ int64_t lo_index(int64_t e, const StepDims& d) {
    const int64_t bv = e / d.ncell;
    const int c = (int)(e - bv * d.ncell);
    const int ip = c % d.nip, jp = (c / d.nip) % d.njp, kp = c / (d.nip * d.njp);
    if (ip < 2 || ip >= d.nip - 2 || jp < 2 || jp >= d.njp - 2 || kp < 2 || kp >= d.nkp - 2) return -1;
    return ((bv * d.nk + (kp - 2)) * d.nj + (jp - 2)) * d.ni + (ip - 2);
}
inline size_t lo_elems(const StepDims& d) { return (size_t)d.nblocks * NV * d.ni * d.nj * d.nk; }

// div-B control of a stage (DivB_option): mode 0 none; 1 GLM cleaning
// (3_6/ModDivB.f90:13-38) with psi arrays [b][cell] of the stage input, of u^n
// and of the stage output -- psi is read from global memory (not the
// shared-memory ring), so out != in; 2 the Powell source term -(div B) v on
// the induction equation (3_5/ModEquation.f90:169-176), no psi.
struct DivBArgs {
    const void* in;
    const void* un;
    void* out;
    int mode;
};

// ---- launchers (defined in mhd_fp64.cu / mhd_mixed.cu) --------------------
// stage s = 1..4; in: u_s, un: u^n, out: u_{s+1}; bc_writeback: 1 writes the
// mirrored radial ghosts back into `in`, as ModBoundary does in place
// (3_6/ModBoundary.f90:10-55); the diffusion pass later reads those of u^n
// (3_6/ModAdvance.f90:101-108)
cudaError_t launch_stage_fp64(const StepDims& d, const Geometry& g, const double* in, const double* un,
                              double* out, const DivBArgs& psi, int stage, int bc_writeback, StepScalars* sc,
                              int heat_on, int kpar, cudaStream_t st);
// GLM: psi's artificial diffusion (into psi_out) and psi's ghost fill
cudaError_t launch_psi_diffusion_fp64(const StepDims& d, const Geometry& g, const double* u, const double* psi,
                                      double* psi_out, StepScalars* sc, cudaStream_t st);
cudaError_t launch_psi_ghost_fp64(const StepDims& d, const GhostLists& gl, double* psi, cudaStream_t st);
cudaError_t launch_diffusion_fp64(const StepDims& d, const Geometry& g, double* u, StepScalars* sc,
                                  int kpar, cudaStream_t st);
cudaError_t launch_cfl_fp64(const StepDims& d, const Geometry& g, const double* u, StepScalars* sc,
                            cudaStream_t st);
cudaError_t launch_ghost_fp64(const StepDims& d, const GhostLists& gl, double* u, cudaStream_t st);
// block sharding (FP64): outgoing entries of L into pack[n][8]; pack into the ghost cells dst[n]
cudaError_t launch_shard_pack_fp64(const StepDims& d, const GhostInterpList& L, const double* u, double* pack,
                                   cudaStream_t st);
cudaError_t launch_shard_unpack_fp64(const StepDims& d, const int32_t* dst, int64_t n, const double* pack, double* u,
                                     cudaStream_t st);

// lo: the correction array of u^n (see lo_unit); the stage kernel updates it
// at stage 4 only, the diffusion pass always; nullptr leaves u^n plain FP32.
// push: faces written into `out` by the stage kernel (tgt == nullptr: none);
// pushing needs out != in, since a target block may still be reading `in`.
cudaError_t launch_stage_mixed(const StepDims& d, const Geometry& g, const float* in, const float* un,
                               float* out, int8_t* lo, const PushTable& push, const DivBArgs& psi, int stage,
                               int bc_writeback, StepScalars* sc, int heat_on, int kpar, cudaStream_t st);
cudaError_t launch_psi_diffusion_mixed(const StepDims& d, const Geometry& g, const float* u, const float* psi,
                                       float* psi_out, StepScalars* sc, cudaStream_t st);
cudaError_t launch_psi_ghost_mixed(const StepDims& d, const GhostLists& gl, float* psi, cudaStream_t st);
// diffusion of u into out: in place (out == u, push.tgt == nullptr) or out of
// place with the regular faces pushed into out and the radial boundary ghost
// columns copied (see k_diffusion)
// One whole mixed step of 16^3 blocks as one persistent cooperative launch
// (after the CFL minimum of u^n is formed): dt, four stages with their face
// exchanges, diffusion into R2, the final exchange. bar: 8 device words
// (reset here): grid-barrier counter and generation, the 5 block tickets.
// every cell outside the core of each block and variable set to 0 (nvar
// variables per block: NV for the state, 1 for psi)
cudaError_t launch_clear_outside_core_mixed(const StepDims& d, float* u, int nvar, cudaStream_t st);
// the regular faces of a mixed state pushed and its CFL minimum formed, as the
// diffusion pass closing a step leaves them (after a core upload)
cudaError_t launch_push_state_mixed(const StepDims& d, const Geometry& g, float* u, const PushTable& push,
                                    StepScalars* sc, cudaStream_t st);
cudaError_t launch_step_persistent_mixed(const StepDims& d, const Geometry& g, float* U, float* RK, float* R2,
                                         int8_t* lo, const PushTable& push, const GhostLists& gl_stage,
                                         const GhostLists& gl_final, StepScalars* sc, unsigned int* bar,
                                         cudaStream_t st);
cudaError_t launch_diffusion_mixed(const StepDims& d, const Geometry& g, const float* u, float* out, int8_t* lo,
                                   const PushTable& push, StepScalars* sc, int kpar, cudaStream_t st,
                                   int cfl_next = 0);
cudaError_t launch_cfl_mixed(const StepDims& d, const Geometry& g, const float* u, StepScalars* sc,
                             cudaStream_t st);
cudaError_t launch_ghost_mixed(const StepDims& d, const GhostLists& gl, float* u, cudaStream_t st);

cudaError_t launch_finalize_dt(StepScalars* sc, cudaStream_t st);
// k-chunk depths instantiated for this block size (returns the count)
int kpar_candidates_fp64(const StepDims& d, int* out);
int kpar_candidates_mixed(const StepDims& d, int* out);
// Host block arrays ([b][FALCON_NVAR = 9][cell] FP64) <-> device state
// ([b][8][cell], FP32 compensated or FP64) and the optional psi array.
// convert: n = device state elements; gather: host elements [first, first+count)
cudaError_t launch_convert_state(const double* src, float* dst, int8_t* lo, int64_t n, const StepDims& dm,
                                 cudaStream_t st);
cudaError_t launch_convert_psi(const double* src, float* psi, int64_t nb, int64_t ncell, cudaStream_t st);
// *flag = 1 if the psi planes of a host-layout FP64 array on the device hold a non-zero value
cudaError_t launch_psi_nonzero(const double* src, int64_t nb, int64_t ncell, int32_t* flag, cudaStream_t st);
// AllCells output (output.cu): per-block face table [r (ni+1) | sin theta,
// cos theta (nj+1 each) | sin phi, cos phi (nk+1 each) | yin], and the
// kernel writing 12 doubles per corner (x, y, z, then the 9 variables with
// Cartesian vectors) for blocks [b0, b0 + nbb)
__host__ __device__ inline int allcells_table_stride(const StepDims& d) {
    return (d.ni + 1) + 2 * (d.nj + 1) + 2 * (d.nk + 1) + 1;
}
cudaError_t launch_allcells(const StepDims& d, const void* U, const int8_t* lo, const void* psi, bool fp32,
                            const double* tab, int b0, int nbb, double* out, cudaStream_t st);

// Core transfers (interior planes x interior rows of every block and
// variable of the host array, radial ghost columns included), host array
// 16-byte aligned; U is FP32 (with its correction lo) or FP64.
cudaError_t launch_core_up(const double* host, void* U, int8_t* lo, void* P, int32_t* flag, bool fp32, const StepDims& dm,
                           cudaStream_t st);
cudaError_t launch_core_down(const void* U, const int8_t* lo, const void* P, bool fp32, double* host, const StepDims& dm,
                             cudaStream_t st);
cudaError_t launch_gather_host(const void* U, const int8_t* lo, const void* psi, bool fp32, const StepDims& dm,
                               int64_t first, int64_t count,
                               int64_t ncell, double* out, cudaStream_t st);

// names of the kernels as they appear in profiles
const char* const* kernel_names();

}  // namespace falcon
