// mhd_impl.cuh -- kernel bodies shared by the FP64 and mixed instantiations.
// Included by mhd_fp64.cu (T=double, -fmad=false) and mhd_mixed.cu (T=float).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "kernels.cuh"

namespace falcon {
namespace impl {

// Precision policy. Exact: the reference's divisions stay divisions; the
// mixed path multiplies by reciprocals tabulated on the host.
template <class T> struct Pol;
template <> struct Pol<double> {
    static constexpr bool exact = true;
    __device__ static __forceinline__ double dv(double a, double b, double binv) { return a / b; }
    __device__ static __forceinline__ double mmthr() { return (double)1.e-30f; }
    __device__ static __forceinline__ double mmscale() { return 1.e10; }
    __device__ static __forceinline__ double ratio(double a, double b) { return a / b; }
};
template <> struct Pol<float> {
    static constexpr bool exact = false;
    __device__ static __forceinline__ float dv(float a, float, float binv) { return a * binv; }
    __device__ static __forceinline__ float mmthr() { return 1.e-30f; }
    __device__ static __forceinline__ float mmscale() { return 1.e10f; }
    // limiter ratio: an approximate quotient is enough (0/0 still gives NaN -> phi = 0)
    __device__ static __forceinline__ float ratio(float a, float b) { return __fdividef(a, b); }
};

// ModLinReconstruct_minmod for one value (3_6/ModLinReconstruct.f90:44-48).
template <class T>
__device__ __forceinline__ T minmod(T ul, T u, T ur) {
    const T a = (ur - ul) * T(0.5);
    const T b = T(2) * (ur - u);
    const T c = T(2) * (u - ul);
    T t;
    if (Pol<T>::exact) {
        t = fmax(T(0), a * b) * fmax(T(0), b * c) * Pol<T>::mmscale() - Pol<T>::mmthr();
    } else {
        // same test, factors reordered so the FP32 product stays in the normal range
        t = (fmax(T(0), a * b) * Pol<T>::mmscale()) * fmax(T(0), b * c) - Pol<T>::mmthr();
    }
    const T s = copysign(T(0.5), t);
    const T m = fmin(fmin(fabs(a), fabs(b)), fabs(c));
    return (s + T(0.5)) * copysign(m, a);
}

// FP32 minmod with the reference's selector written as a compare: the
// reference forms t = max(0,ab)max(0,bc)*1e10 - 1e-30 and returns
// (sign(t)/2 + 1/2) * sign(a) min(|a|,|b|,|c|), which is min(...) with a's
// sign when t >= 0 and zero otherwise
__device__ __forceinline__ float minmod_sel(float ul, float u, float ur) {
    const float a = (ur - ul) * 0.5f;
    const float b = 2.f * (ur - u);
    const float c = 2.f * (u - ul);
    // max(0, ab) 1e10 max(0, bc) >= 1e-30 is the same test as ab > 0 and
    // (ab 1e10) bc >= 1e-30: with ab > 0 the first max is ab, and with bc <= 0
    // or NaN both products are <= 0 or NaN (0 or -0 times an infinity)
    const float ab = a * b;
    const float x = (ab * 1.e10f) * (b * c);
    const float m = fminf(fminf(fabsf(a), fabsf(b)), fabsf(c));
    return ab > 0.f && x >= 1.e-30f ? copysignf(m, a) : 0.f;
}

// The per-cell CFL ratio h_LLL / v_wave of the mixed path, shared by k_cfl and
// the diffusion pass that forms it for the next step: explicitly rounded FP32
// operations, so both give the same bits whatever the compiler contracts.
__device__ __forceinline__ float cfl_sq3(float x, float y, float z) {
    return __fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z));
}
__device__ __forceinline__ float cfl_ratio_f(float v2, float b2, float cs, float rho0, float r, float sin_t,
                                             float dxi, float dxj, float dxk) {
    // h_LLL = min(dxi, r*dxj, r*sin(theta)*dxk) (3_6/ModBlock.f90:416-425)
    const float h = fminf(fminf(dxi, __fmul_rn(r, dxj)), __fmul_rn(__fmul_rn(r, sin_t), dxk));
    float w = __fadd_rn(cs, __fsqrt_rn(v2));
    w = __fadd_rn(w, __fdiv_rn(__fsqrt_rn(b2), __fsqrt_rn(rho0)));
    return __fdiv_rn(h, w);
}
// block minimum of the ratios (FP64 bit order for positive values) and NaN flag
__device__ __forceinline__ void cfl_commit(float ratio, int nan, StepScalars* sc) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ratio = fminf(ratio, __shfl_xor_sync(0xffffffffu, ratio, o));
        nan |= __shfl_xor_sync(0xffffffffu, nan, o);
    }
    __shared__ float wmin[32];
    __shared__ int wnan[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { wmin[wid] = ratio; wnan[wid] = nan; }
    __syncthreads();
    if (threadIdx.x == 0) {
        float m = wmin[0];
        int n = wnan[0];
        for (int w2 = 1; w2 < (int)(blockDim.x >> 5); ++w2) { m = fminf(m, wmin[w2]); n |= wnan[w2]; }
        atomicMin(&sc->min_ratio_bits, (unsigned long long)__double_as_longlong((double)m));
        if (n) atomicOr(&sc->nan_flag, 1);
    }
}

template <class T> __device__ __forceinline__ const T* gi_ptr(const Geometry& g);
template <> __device__ __forceinline__ const double* gi_ptr<double>(const Geometry& g) { return g.gi; }
template <> __device__ __forceinline__ const float* gi_ptr<float>(const Geometry& g) { return g.gi_f; }
template <class T> __device__ __forceinline__ const T* gj_ptr(const Geometry& g);
template <> __device__ __forceinline__ const double* gj_ptr<double>(const Geometry& g) { return g.gj; }
template <> __device__ __forceinline__ const float* gj_ptr<float>(const Geometry& g) { return g.gj_f; }
template <class T> __device__ __forceinline__ const T* gs_ptr(const Geometry& g);
template <> __device__ __forceinline__ const double* gs_ptr<double>(const Geometry& g) { return g.gs; }
template <> __device__ __forceinline__ const float* gs_ptr<float>(const Geometry& g) { return g.gs_f; }

// ---- TMA (bulk async copy) and mbarrier helpers ---------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// a barrier object is invalidated before its shared memory is used for
// anything else (the persistent step runs several kernel bodies in one CTA)
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// 1-D bulk copy global -> shared, completion counted on `bar` (16-byte aligned, size % 16 == 0)
// Hint: pull `bytes` (a multiple of 16, 16-byte aligned) of global memory into
// L2 ahead of plain loads.
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// bounded wait on an mbarrier phase; false if it did not complete in max_iter polls
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int max_iter) {
    for (int it = 0; it < max_iter; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}
constexpr int kWaitPolls = kDefaultWaitPolls;

// A CTA whose wait for a chunk's planes ran out leaves cleanly: every thread
// learns it at the next chunk's leading barrier (__syncthreads_or, so the exit
// is uniform over the CTA and no thread is left at a barrier), then thread 0
// flags the step (bit 1 of nan_flag: the host returns FALCON_ERR_TIMEOUT) and
// waits, with the default bound, for the bulk copies still in flight into
// this CTA's shared memory -- chunks c0..c1 -- before the CTA exits.
__device__ __forceinline__ void copy_wait_abort(StepScalars* sc, uint64_t* bars, int c0, int c1) {
    if (threadIdx.x != 0) return;
    atomicOr(&sc->nan_flag, 2);
    for (int c = c0 < 0 ? 0 : c0; c <= c1; ++c) mbar_wait(&bars[c & 1], (uint32_t)((c >> 1) & 1), kWaitPolls);
    mbar_inval(&bars[0]);
    mbar_inval(&bars[1]);
}

template <class T, int NI, int NJ, int NK, int KPAR>
struct Shape {
    static constexpr int NG = 2, NIP = NI + 4, NJP = NJ + 4, NKP = NK + 4;
    static constexpr int PL = NIP * NJP, NT = NI * NJ * KPAR;
    static constexpr int W = 2 * KPAR + 4;    // ring: current window (KPAR+4) + the prefetched KPAR planes
    static constexpr int WP = KPAR + 4;       // p1 window
    static constexpr int NCELL = PL * NKP;
    static constexpr int PLI = NI * NJ, NINT = PLI * NK;   // the u^n correction's (interior-only) plane and block
    static constexpr uint32_t PLB = PL * (uint32_t)sizeof(T);   // bytes of one variable plane
    static_assert(PLB % 16 == 0, "plane must be a multiple of 16 bytes");
    static_assert(NK % KPAR == 0, "KPAR must divide NK");
    // FP64 path: Br/sin(theta) and (v x B)_r/sin(theta) per point, [2][WP][PL]
    // (the k-derivatives of the curls divide them by the cell's sin(theta),
    // which its k-neighbours share: formed once per point, not per use)
    static constexpr int NXS = sizeof(T) == 8 ? 2 : 0;
    // shared memory: mbarriers | A1/A2 (double) | tile[NV][W][PL] | p1[WP][PL] | xs[NXS][WP][PL] | gi | gj | gs
    static constexpr size_t off_a12 = 16;
    static constexpr size_t off_tile = off_a12 + ((2 * NIP * sizeof(double) + 15) / 16) * 16;
    static constexpr size_t off_p1 = off_tile + (size_t)NV * W * PL * sizeof(T);
    static constexpr size_t off_xs = off_p1 + (size_t)WP * PL * sizeof(T);
    static constexpr size_t off_gi = off_xs + (size_t)NXS * WP * PL * sizeof(T);
    static constexpr size_t off_gj = off_gi + (size_t)GI_COUNT * NIP * sizeof(T);
    static constexpr size_t off_gs = off_gj + (size_t)GJ_COUNT * NJP * sizeof(T);
    static constexpr size_t smem_stage = off_gs + GS_COUNT * sizeof(T);
    static constexpr size_t smem_diff = smem_stage;
    // FP32 stage: as many CTAs per SM as the shared memory holds (228 KB per
    // SM, 1 KB reserved per CTA), so the register allocation must fit them
    // too (at least 32 registers a thread). FP64 keeps the compiler's choice.
    static constexpr int by_smem = (int)(233472 / (smem_stage + 1024));
    static constexpr int reg_cap = 2048 / NT;
    static constexpr int min_blocks =
        sizeof(T) != 4 || by_smem < 2 ? 1 : (by_smem < reg_cap ? by_smem : (reg_cap < 1 ? 1 : reg_cap));
};

// Thread 0: bulk-copy planes kp in [lo,hi) of all variables of the block into
// their ring slots, completing on `bar`.
template <class T, class S>
__device__ __forceinline__ void issue_planes(const T* blk, T* tile, int lo, int hi, uint64_t* bar) {
    mbar_expect_tx(bar, (uint32_t)(NV * (hi - lo)) * S::PLB);
    for (int v = 0; v < NV; ++v)
        for (int kp = lo; kp < hi; ++kp)
            tma_load_1d(tile + ((size_t)v * S::W + (kp % S::W)) * S::PL, blk + ((size_t)v * S::NKP + kp) * S::PL,
                        S::PLB, bar);
}

template <class T, class S>
__device__ __forceinline__ void load_geometry(const Geometry& g, int b, T* gi, T* gj, T* gs, double* a12) {
    const T* Gi = gi_ptr<T>(g) + (size_t)b * GI_COUNT * S::NIP;
    const T* Gj = gj_ptr<T>(g) + (size_t)b * GJ_COUNT * S::NJP;
    const T* Gs = gs_ptr<T>(g) + (size_t)b * GS_COUNT;
    for (int x = threadIdx.x; x < GI_COUNT * S::NIP; x += S::NT) gi[x] = Gi[x];
    for (int x = threadIdx.x; x < GJ_COUNT * S::NJP; x += S::NT) gj[x] = Gj[x];
    for (int x = threadIdx.x; x < GS_COUNT; x += S::NT) gs[x] = Gs[x];
    if (a12) {
        const double* Gd = g.gi + (size_t)b * GI_COUNT * S::NIP;
        for (int x = threadIdx.x; x < 2 * S::NIP; x += S::NT) {
            const double a = Gd[(x < S::NIP ? GI_A1 * S::NIP : GI_A2 * S::NIP - S::NIP) + x];
            if constexpr (Pol<T>::exact) {
                a12[x] = a;
            } else {
                // FP32 pairs (hi, lo) with hi + lo = a to about 2^-48:
                // [a1 hi | a1 lo | a2 hi | a2 lo], NIP floats each
                float* f = reinterpret_cast<float*>(a12);
                const int c = x % S::NIP, which = x / S::NIP;
                const float hi = (float)a;
                f[(2 * which) * S::NIP + c] = hi;
                f[(2 * which + 1) * S::NIP + c] = (float)(a - (double)hi);
            }
        }
    }
}

// p1 = a1*rho1 + a2*s1 for the mixed path in float-float arithmetic: the
// two products are formed exactly with FMA (plus the coefficients' low
// parts), summed with an error-free two-sum, and rounded once to FP32. The
// terms nearly cancel, so a plain FP32 sum would lose digits; this keeps the
// accuracy of an FP64 assembly on the FP32 pipe (GB300's FP64 rate is a
// small fraction of its FP32 rate).
__device__ __forceinline__ float p1_ff(float a1h, float a1l, float a2h, float a2l, float r1, float s1) {
    const float ph = __fmul_rn(a1h, r1);
    const float pl = __fmaf_rn(a1h, r1, -ph);
    const float qh = __fmul_rn(a2h, s1);
    const float ql = __fmaf_rn(a2h, s1, -qh);
    const float sh = __fadd_rn(ph, qh);
    const float bb = __fsub_rn(sh, ph);
    const float se = __fadd_rn(__fsub_rn(ph, __fsub_rn(sh, bb)), __fsub_rn(qh, bb));
    const float lo = __fmaf_rn(a1l, r1, __fmaf_rn(a2l, s1, __fadd_rn(pl, ql)));
    return __fadd_rn(sh, __fadd_rn(se, lo));
}

// Radial mirror boundary (3_6/ModBoundary.f90:10-55) on planes [lo,hi) of the
// ring, whole rows including their theta ghosts; optionally written back.
template <class T, class S>
__device__ __forceinline__ void apply_bc(T* tile, int lo, int hi, int fl, T* wb) {
    const bool top = fl & 2, bot = fl & 4;
    if (!top && !bot) return;
    const int np = hi - lo;
    const int NI = S::NIP - 4;
    // per variable sign: top mirrors rho1,vt,vp,s1,br; anti-mirrors vr,bt,bp.
    // bottom mirrors rho1,vt,vp,s1,bt,bp; anti-mirrors vr,br.
    const int total = np * S::NJP * NV * 2;
    for (int x = threadIdx.x; x < total; x += S::NT) {
        const int g = x & 1;
        const int rest = x >> 1;
        const int v = rest % NV;
        const int rest2 = rest / NV;
        const int j = rest2 % S::NJP;
        const int kp = lo + rest2 / S::NJP;
        T* row = tile + ((size_t)v * S::W + (kp % S::W)) * S::PL + j * S::NIP;
        if (top) {
            // Fortran i = ni+1+g <- 2*ni+1-i = ni-g ; padded index = Fortran + 1
            const bool neg = (v == V_VR) || (v == V_BT) || (v == V_BP);
            const T s = row[NI - g + 1];
            const T val = neg ? -s : s;
            row[NI + 2 + g] = val;
            if (wb) wb[((size_t)v * S::NKP + kp) * S::PL + j * S::NIP + NI + 2 + g] = val;
        }
        if (bot) {
            // Fortran i = -g <- 1-i = 1+g ; padded index = Fortran + 1
            const bool neg = (v == V_VR) || (v == V_BR);
            const T s = row[2 + g];
            const T val = neg ? -s : s;
            row[1 - g] = val;
            if (wb) wb[((size_t)v * S::NKP + kp) * S::PL + j * S::NIP + 1 - g] = val;
        }
    }
}

// 1-D blend a*(1-w) + b*w with one fixed rounding sequence, so the ghost
// fill and the stage kernel's pushed faces give identical values
__device__ __forceinline__ float blend(float a, float b, float uw, float w) { return __fmaf_rn(a, uw, __fmul_rn(b, w)); }
__device__ __forceinline__ double blend(double a, double b, double uw, double w) { return a * uw + b * w; }

// Write this cell's new values into the ghost cells of the neighbours whose
// faces are pushed (PushTable). (ii, jj, kp): padded indices of the cell; o:
// its 8 new values. Theta/phi faces: the two interior layers next to the side
// are copied to the target's opposite ghost layers (a shift of one block
// extent). Radial faces: the thread at the first source cell of a ghost layer
// blends it with the next cell along i, taken from the next lane (i is the
// fastest thread index, and the second cell is never beyond the row). Every
// thread of the CTA calls this (the shuffle needs the full warp).
// The push-table entries of one block, staged in shared memory before the
// kernel's first barrier: they are read at the end of every k-chunk, and as
// global loads their latency held every warp at the chunk's end.
struct PushBlock {
    int32_t tgt[6];
    int32_t src[4], dst[4];   // [side][layer]
    float w[4];
};
__device__ __forceinline__ void load_push_block(const PushTable& P, int b, PushBlock* s) {
    const int t = threadIdx.x;
    if (P.tgt == nullptr) return;
    if (t < 6) {
        s->tgt[t] = P.tgt[6 * b + t];
    } else if (t < 10) {
        const int q = t - 6;
        s->src[q] = P.rad_src[4 * b + q];
        s->dst[q] = P.rad_dst[4 * b + q];
        s->w[q] = P.rad_w[4 * b + q];
    }
}

template <class T, class S, int VN>
__device__ __forceinline__ void push_faces_part(T* out, const PushBlock& P, int ii, int jj, int kp,
                                                const T (&o)[VN], int v0) {
    constexpr int NJ = S::NJP - 4, NK = S::NKP - 4;
    const int32_t* tg = P.tgt;
    auto put = [&](int tb, int kt, int jt, int it, const T (&val)[VN]) {
        T* dst = out + ((size_t)tb * NV + v0) * S::NCELL + ((size_t)kt * S::NJP + jt) * S::NIP + it;
#pragma unroll
        for (int v = 0; v < VN; ++v) dst[(size_t)v * S::NCELL] = val[v];
    };
    if (jj <= 3 && tg[2] >= 0) put(tg[2], kp, jj + NJ, ii, o);
    if (jj >= NJ && tg[3] >= 0) put(tg[3], kp, jj - NJ, ii, o);
    if (kp <= 3 && tg[4] >= 0) put(tg[4], kp + NK, jj, ii, o);
    if (kp >= NK && tg[5] >= 0) put(tg[5], kp - NK, jj, ii, o);
    if (tg[0] >= 0 || tg[1] >= 0) {   // uniform over the CTA
        if constexpr (S::NIP == 20 && 2 * VN <= 16) {
            // 16-wide rows: every half-warp holds one full row (i = lane % 16).
            // Lane (v, layer) = (lh / 2, lh % 2) of the half gathers its value
            // from the row's source lanes, so a side takes one store per row
            // instead of a divergent store per variable and layer.
            const int lane = threadIdx.x & 31, lh = lane & 15, hb = lane & 16;
            const int v = lh >> 1, layer = lh & 1;
#pragma unroll
            for (int side = 0; side < 2; ++side) {
                if (tg[side] < 0) continue;
                const int q = side * 2 + layer;
                const int s0 = hb + P.src[q] - 2;
                const bool two = P.w[side * 2] != 0.f || P.w[side * 2 + 1] != 0.f;   // uniform
                T a = T(0), c = T(0);
#pragma unroll
                for (int u = 0; u < VN; ++u) {
                    const T x0 = __shfl_sync(0xffffffffu, o[u], s0);
                    T x1 = T(0);
                    if (two) x1 = __shfl_sync(0xffffffffu, o[u], s0 + 1);
                    if (u == v) { a = x0; c = x1; }
                }
                if (v < VN) {
                    const T w = (T)P.w[q];
                    const T val = w == T(0) ? a : blend(a, c, T(1) - w, w);
                    out[((size_t)tg[side] * NV + v0 + v) * S::NCELL + ((size_t)kp * S::NJP + jj) * S::NIP + P.dst[q]] = val;
                }
            }
            return;
        }
        T nx[VN];
#pragma unroll
        for (int v = 0; v < VN; ++v) nx[v] = __shfl_down_sync(0xffffffffu, o[v], 1);
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            if (tg[side] < 0) continue;
#pragma unroll
            for (int layer = 0; layer < 2; ++layer) {
                const int q = side * 2 + layer;
                if (ii != P.src[q]) continue;
                const T w = (T)P.w[q], uw = T(1) - w;
                T val[VN];
#pragma unroll
                for (int v = 0; v < VN; ++v) val[v] = w == T(0) ? o[v] : blend(o[v], nx[v], uw, w);
                put(tg[side], kp, jj, P.dst[q], val);
            }
        }
    }
}
template <class T, class S>
__device__ __forceinline__ void push_faces(T* out, const PushBlock& P, int ii, int jj, int kp, const T (&o)[NV]) {
    push_faces_part<T, S, NV>(out, P, ii, jj, kp, o, 0);
}

// Cell (i, j, kq) of a thread in a k-chunk. With 16-wide rows and an even
// chunk depth a warp takes one row of two adjacent planes (lanes 0-15 plane
// kq, 16-31 plane kq+1): a plane is 400 floats, 16 banks apart, so every
// shared-memory access of the stencil is free of bank conflicts (two rows of
// one plane, 20 floats apart, share 4 banks). Otherwise rows of one plane.
// i stays the fastest index within 16 or 8 lanes either way.
template <int NI, int NJ, int KPAR>
__device__ __forceinline__ void cell_of_thread(int tid, int& i, int& j, int& kq) {
    if constexpr (NI == 16 && KPAR % 2 == 0) {
        i = tid % NI;
        const int pair = (tid / NI) % 2;
        j = (tid / (2 * NI)) % NJ;
        kq = 2 * (tid / (2 * NI * NJ)) + pair;
    } else {
        i = tid % NI;
        j = (tid / NI) % NJ;
        kq = tid / (NI * NJ);
    }
}

// ---------------------------------------------------------------------------
// Packed FP32 pairs (Blackwell's two-lane FFMA2/FADD2/FMUL2): the diffusion
// march runs its slopes, fluxes and update on variables v and v+1 at once,
// the stage its stage-4 update. Each helper gives bit for bit what its scalar counterpart gives (a
// difference a - b is formed as fma(b, -1, a), one rounding of the exact
// difference, as FADD does).
__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 f2(float x) { return make_float2(x, x); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.f), a); }
__device__ __forceinline__ float2 max02(float2 a) { return f2(fmaxf(0.f, a.x), fmaxf(0.f, a.y)); }
// minmod_sel for two variables
__device__ __forceinline__ float2 minmod_sel2(float2 ul, float2 u, float2 ur) {
    const float2 a = __fmul2_rn(sub2(ur, ul), f2(0.5f));
    const float2 b = __fmul2_rn(sub2(ur, u), f2(2.f));
    const float2 c = __fmul2_rn(sub2(u, ul), f2(2.f));
    const float2 ab = __fmul2_rn(a, b);   // the test of minmod_sel
    const float2 x = __fmul2_rn(__fmul2_rn(ab, f2(1.e10f)), __fmul2_rn(b, c));
    const float mx = fminf(fminf(fabsf(a.x), fabsf(b.x)), fabsf(c.x));
    const float my = fminf(fminf(fabsf(a.y), fabsf(b.y)), fabsf(c.y));
    return f2(ab.x > 0.f && x.x >= 1.e-30f ? copysignf(mx, a.x) : 0.f,
              ab.y > 0.f && x.y >= 1.e-30f ? copysignf(my, a.y) : 0.f);
}
// face_flux_s<float> for two variables; cc = -0.25 (cR + cL), the face's
// speed factor (the same for every variable; -0.25 scales exactly, so
// (phi num) cc is the scalar form's ((-0.25 phi) num)(cR + cL) bit for bit)
__device__ __forceinline__ float2 face_flux2(float2 fl, float2 fr, float2 dL, float2 dR, float2 cc) {
    const float2 num = __ffma2_rn(dL, f2(-0.5f), sub2(__ffma2_rn(dR, f2(-0.5f), fr), fl));
    const float2 den = sub2(fr, fl);
    const float2 r = __ffma2_rn(f2(__fdividef(num.x, den.x), __fdividef(num.y, den.y)), f2(2.f), f2(-1.f));
    return __fmul2_rn(__fmul2_rn(max02(r), num), cc);
}
// ff_add for two variables
__device__ __forceinline__ float2 ff_add2(float2 hi, int8_t q0, int8_t q1, float2 d, int8_t& o0, int8_t& o1) {
    const float2 l = __fmul2_rn(f2(lo_decode(q0), lo_decode(q1)), f2(lo_unit(hi.x), lo_unit(hi.y)));
    const float2 s = __fadd2_rn(hi, d);
    const float2 bs = sub2(s, hi);
    const float2 es = __fadd2_rn(sub2(hi, sub2(s, bs)), sub2(d, bs));
    const float2 t = __fadd2_rn(es, l);
    const float2 h = __fadd2_rn(s, t);
    const float2 bh = sub2(h, s);
    const float2 r = __fadd2_rn(sub2(s, sub2(h, bh)), sub2(t, bh));
    o0 = lo_encode(h.x, r.x);
    o1 = lo_encode(h.y, r.y);
    return h;
}

// ---------------------------------------------------------------------------
// One RK stage of one block: boundary -> RHS (3_6/ModEquation.f90:24-162) ->
// u_out = u^n + dt*R/(5-s) (3_6/ModAdvance.f90:87-93).
// The body runs block b with the CTA's threads (NI*NJ*KPAR of them): k_stage
// calls it for blockIdx.x, the persistent step for each block it takes.
template <class T, int NI, int NJ, int NK, int KPAR, int DIVB>
__device__ __forceinline__ void stage_body(int b, const T* in, const T* un, T* out, int8_t* ulo, PushTable push,
                                           DivBArgs psi, Geometry g, StepScalars* sc, int stage, int bc_writeback,
                                           int heat_on) {
    using S = Shape<T, NI, NJ, NK, KPAR>;
    constexpr int NIP = S::NIP, PL = S::PL, W = S::W, WP = S::WP, NCELL = S::NCELL;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
    double* a12 = reinterpret_cast<double*>(smem + S::off_a12);
    T* tile = reinterpret_cast<T*>(smem + S::off_tile);
    T* tp1 = reinterpret_cast<T*>(smem + S::off_p1);
    T* txs = reinterpret_cast<T*>(smem + S::off_xs);   // FP64: [0] Br/sin, [1] E_r/sin (E = v x B)
    T* gi = reinterpret_cast<T*>(smem + S::off_gi);
    T* gj = reinterpret_cast<T*>(smem + S::off_gj);
    T* gs = reinterpret_cast<T*>(smem + S::off_gs);

    const int fl = g.flags[b];
    const T* blk_in = in + (size_t)b * NV * NCELL;
    T* wb = bc_writeback ? const_cast<T*>(blk_in) : nullptr;
    __shared__ PushBlock pb;
    load_push_block(push, b, &pb);
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) issue_planes<T, S>(blk_in, tile, 0, KPAR + 4, &bars[0]);
    // u^n (and its int8 correction at stage 4) is read with plain loads at
    // stages 2-4: warm L2 with the planes of the first chunk, then one chunk ahead
    const T* blk_un = un + (size_t)b * NV * NCELL;
    const int8_t* blk_lo = ulo != nullptr ? ulo + (size_t)b * NV * S::NINT : nullptr;
    T* blk_out = out + (size_t)b * NV * NCELL;
    auto prefetch_un = [&](int kp_first) {
        if (threadIdx.x >= NV) return;
        const int v = threadIdx.x;
        // the output rows are written in part (interior cells only): their lines into L2 first
        if (out != un || stage == 1) prefetch_l2(blk_out + ((size_t)v * S::NKP + kp_first) * PL, KPAR * S::PLB);
        if (stage == 1) return;
        // u^n is read at interior cells only: its interior rows (2 .. NJ+1 of
        // each plane, one contiguous run) are enough
#pragma unroll
        for (int q = 0; q < KPAR; ++q)
            prefetch_l2(blk_un + ((size_t)v * S::NKP + kp_first + q) * PL + 2 * NIP, (uint32_t)(NJ * NIP * sizeof(T)));
        if (blk_lo != nullptr && stage == 4)
            prefetch_l2(blk_lo + ((size_t)v * NK + (kp_first - 2)) * S::PLI, KPAR * S::PLI);
    };
    prefetch_un(2);
    load_geometry<T, S>(g, b, gi, gj, gs, a12);
    __syncthreads();   // the geometry tables are read by every thread below

    const int tid = threadIdx.x;
    int i, j, kq;
    cell_of_thread<NI, NJ, KPAR>(tid, i, j, kq);
    const int ii = i + 2, jj = j + 2;
    const T c1 = gs[GS_C1], c2 = gs[GS_C2], c3 = gs[GS_C3];
    const T* GR = gi + GI_R * NIP;
    const T* GR2 = gi + GI_R2 * NIP;
    const T* GRHO0 = gi + GI_RHO0 * NIP;
    const T* GSIN = gj + GJ_SIN * S::NJP;
    const T rinv = gi[GI_RINV * NIP + ii], r2inv = gi[GI_R2INV * NIP + ii];
    const T sinv = gj[GJ_SININV * S::NJP + jj], cot = gj[GJ_COT * S::NJP + jj];
    const T sin_c = GSIN[jj];
    const T rho0c = GRHO0[ii], rho0inv = gi[GI_RHO0INV * NIP + ii];
    const T gor0 = gi[GI_GOR0 * NIP + ii], heat = gi[GI_HEAT * NIP + ii], xi2inv = gi[GI_XI2INV * NIP + ii];
    const double dt = sc->dt;
    const double divs = (double)(5.0f - (float)stage);
    // x / divs for divs = 4, 2, 1 (stages 1, 3, 4) is x times the exact
    // reciprocal, the same bits without an FP64 division; stage 2 divides by 3
    const bool div_pow2 = stage != 2;
    const double rdivs = 1.0 / divs;
    auto over_divs = [&](double x) { return div_pow2 ? x * rdivs : x / divs; };
    const float dtk = sc->dt_stage_f[stage - 1];

    constexpr int nchunk = NK / KPAR;
    const int polls = sc->wait_polls;
    int late = 0;   // a wait of this thread for a chunk's planes ran out
    for (int ch = 0; ch < nchunk; ++ch) {
        const int k0 = 1 + ch * KPAR;  // first Fortran k of the chunk
        const int lo = (ch == 0) ? 0 : k0 + 3;   // first padded plane new to this chunk
        const int hi = k0 + KPAR + 3;            // one past the last plane it needs
        // chunk ch-1 is done with the slots the prefetch below overwrites; a
        // wait of chunk ch-1 that ran out ends the CTA here (chunks ch-1 and ch
        // are in flight)
        if (__syncthreads_or(late)) {
            copy_wait_abort(sc, bars, ch - 1, ch);
            return;
        }
        if (threadIdx.x == 0 && ch + 1 < nchunk)
            issue_planes<T, S>(blk_in, tile, hi, hi + KPAR, &bars[(ch + 1) & 1]);
        if (ch + 1 < nchunk) prefetch_un(k0 + KPAR + 1);
        // a wait that runs out does not leave the chunk (its barriers must be
        // reached by every thread): the chunk computes on whatever the slots
        // hold, the step is flagged and its results are discarded
        late |= mbar_wait(&bars[ch & 1], (uint32_t)((ch >> 1) & 1), polls) ? 0 : 1;
        // u^n for the update (stages 2-4), loaded here so that the latency of
        // these plain loads overlaps the boundary and p1 phases below
        const int kp = k0 + kq + 1;
        const size_t base = (size_t)b * NV * NCELL + (size_t)kp * PL + jj * NIP + ii;
        T u0s[NV];
        if (stage != 1) {
#pragma unroll
            for (int v = 0; v < NV; ++v) u0s[v] = un[base + (size_t)v * NCELL];
        }
        if (fl & 6) {   // radial boundary block (uniform over the CTA)
            apply_bc<T, S>(tile, lo, hi, fl, wb);
            fence_proxy_async();   // order these generic writes before later bulk copies into the slots
            __syncthreads();
        }
        // p1 = gamma1*(p0/rho0)*rho1 + (gamma3-1)*(rho0*T0)*s1, assembled in FP64
        // (3_6/ModEquation.f90:40-46)
        for (int x = tid; x < (hi - lo) * PL; x += S::NT) {
            const int kp = lo + x / PL, c = x % PL, ic = c % NIP;
            const int slot = kp % W;
            if constexpr (Pol<T>::exact) {
                const double r1 = (double)tile[(V_RHO1 * W + slot) * PL + c];
                const double s1v = (double)tile[(V_S1 * W + slot) * PL + c];
                tp1[(kp % WP) * PL + c] = (T)(a12[ic] * r1 + a12[NIP + ic] * s1v);
                const int jc = c / NIP;
                if (ic >= 2 && ic < NI + 2 && jc >= 2 && jc < NJ + 2) {   // the k-neighbours of interior cells
                    auto at = [&](int v) { return tile[(v * W + slot) * PL + c]; };
                    const T sn = gj[GJ_SIN * S::NJP + jc];
                    txs[(0 * WP + kp % WP) * PL + c] = Pol<T>::dv(at(V_BR), sn, T(0));
                    txs[(1 * WP + kp % WP) * PL + c] =
                        Pol<T>::dv(at(V_VT) * at(V_BP) - at(V_VP) * at(V_BT), sn, T(0));
                }
            } else {
                const float* f = reinterpret_cast<const float*>(a12);
                tp1[(kp % WP) * PL + c] = p1_ff(f[ic], f[NIP + ic], f[2 * NIP + ic], f[3 * NIP + ic],
                                                (float)tile[(V_RHO1 * W + slot) * PL + c],
                                                (float)tile[(V_S1 * W + slot) * PL + c]);
            }
        }
        __syncthreads();

        int sl[5], sp[5];
#pragma unroll
        for (int d = 0; d < 5; ++d) { sl[d] = (kp + d - 2) % W; sp[d] = (kp + d - 2) % WP; }
        auto A = [&](int v, int di, int dj, int dk) -> T {
            return tile[(v * W + sl[dk + 2]) * PL + (jj + dj) * NIP + ii + di];
        };
        auto P = [&](int di, int dj, int dk) -> T { return tp1[sp[dk + 2] * PL + (jj + dj) * NIP + ii + di]; };
        // ModDerivative_1st_O4_3D (3_6/ModDerivative.f90:16-32)
        auto D = [&](T c, auto f) -> T { return c * (((-f(2) + T(8) * f(1)) - T(8) * f(-1)) + f(-2)); };
        const T vr = A(V_VR, 0, 0, 0), vt = A(V_VT, 0, 0, 0), vp = A(V_VP, 0, 0, 0);
        const T br = A(V_BR, 0, 0, 0), bt = A(V_BT, 0, 0, 0), bp = A(V_BP, 0, 0, 0);
        const T rho1 = A(V_RHO1, 0, 0, 0);
        // at stage 1 the input is u^n and sits in the ring
        if (stage == 1) {
#pragma unroll
            for (int v = 0; v < NV; ++v) u0s[v] = A(v, 0, 0, 0);
        }

        // Mass conservation: -div(rho0 v)/Xi^2 (3_6/ModEquation.f90:50-61, ModSpherical_div :104-159)
        T Rrho;
        {
            T dA = D(c1, [&](int m) { return (GRHO0[ii + m] * A(V_VR, m, 0, 0)) * GR2[ii + m]; });
            dA = dA * r2inv;
            T d23 = D(c2, [&](int m) { return (rho0c * A(V_VT, 0, m, 0)) * GSIN[jj + m]; });
            d23 = d23 + D(c3, [&](int m) { return rho0c * A(V_VP, 0, 0, m); });
            d23 = d23 * sinv;
            d23 = d23 * rinv;
            Rrho = -(xi2inv * (dA + d23));
        }
        // A_dot_Grad_f (3_6/ModSpherical.f90:241-279)
        auto adg = [&](int var) -> T {
            T a = vr * D(c1, [&](int m) { return A(var, m, 0, 0); });
            T t = vt * D(c2, [&](int m) { return A(var, 0, m, 0); });
            a = a + t * rinv;
            t = vp * D(c3, [&](int m) { return A(var, 0, 0, m); });
            t = t * rinv;
            a = a + sinv * t;
            return a;
        };
        // Inertial force -(v.grad)v with curvature terms (3_6/ModSpherical.f90:281-343)
        T Rvr, Rvt, Rvp;
        {
            T a1 = adg(V_VR), a2 = adg(V_VT), a3 = adg(V_VP);
            T tmp = -(vt * vt) - vp * vp;
            a1 = a1 + tmp * rinv;
            tmp = -(vp * vp);
            tmp = tmp * cot;
            tmp = tmp + vt * vr;
            a2 = a2 + tmp * rinv;
            tmp = vp * vt;
            tmp = tmp * cot;
            tmp = tmp + vp * vr;
            a3 = a3 + tmp * rinv;
            Rvr = -a1; Rvt = -a2; Rvp = -a3;
        }
        // Pressure gradient -grad(p1)/rho0 (3_6/ModEquation.f90:79-92)
        {
            const T g1 = D(c1, [&](int m) { return P(m, 0, 0); });
            T g2 = D(c2, [&](int m) { return P(0, m, 0); });
            g2 = g2 * rinv;
            T g3 = D(c3, [&](int m) { return P(0, 0, m); });
            g3 = g3 * rinv;
            g3 = g3 * sinv;
            Rvr = Rvr - Pol<T>::dv(g1, rho0c, rho0inv);
            Rvt = Rvt - Pol<T>::dv(g2, rho0c, rho0inv);
            Rvp = Rvp - Pol<T>::dv(g3, rho0c, rho0inv);
        }
        // Lorentz force (curl B) x B / rho0 (3_6/ModEquation.f90:97-116, curl :38-102)
        {
            T k1 = D(c2, [&](int m) { return A(V_BP, 0, m, 0) * GSIN[jj + m]; }) -
                   D(c3, [&](int m) { return A(V_BT, 0, 0, m); });
            auto brs = [&](int m) -> T {   // Br / sin(theta) at the k-neighbour m
                if constexpr (Pol<T>::exact) return txs[(0 * WP + sp[m + 2]) * PL + jj * NIP + ii];
                else return Pol<T>::dv(A(V_BR, 0, 0, m), sin_c, sinv);
            };
            T k2 = D(c3, brs) -
                   D(c1, [&](int m) { return A(V_BP, m, 0, 0) * GR[ii + m]; });
            T k3 = D(c1, [&](int m) { return A(V_BT, m, 0, 0) * GR[ii + m]; }) -
                   D(c2, [&](int m) { return A(V_BR, 0, m, 0); });
            k1 = k1 * rinv; k2 = k2 * rinv; k3 = k3 * rinv;
            k1 = k1 * sinv;
            const T x1 = k2 * bp - k3 * bt;
            const T x2 = k3 * br - k1 * bp;
            const T x3 = k1 * bt - k2 * br;
            Rvr = Rvr + Pol<T>::dv(x1, rho0c, rho0inv);
            Rvt = Rvt + Pol<T>::dv(x2, rho0c, rho0inv);
            Rvp = Rvp + Pol<T>::dv(x3, rho0c, rho0inv);
        }
        // Buoyancy -(g/rho0) rho1 (3_6/ModEquation.f90:121-127)
        Rvr = Rvr - gor0 * rho1;
        // Entropy advection and heating (3_6/ModEquation.f90:132-151)
        T Rs = -adg(V_S1);
        Rs = Rs + heat;
        (void)heat_on;
        // Induction curl(v x B) (3_6/ModEquation.f90:154-162)
        T RBr, RBt, RBp;
        {
            auto E1 = [&](int a, int bq, int c) { return A(V_VT, a, bq, c) * A(V_BP, a, bq, c) - A(V_VP, a, bq, c) * A(V_BT, a, bq, c); };
            auto E2 = [&](int a, int bq, int c) { return A(V_VP, a, bq, c) * A(V_BR, a, bq, c) - A(V_VR, a, bq, c) * A(V_BP, a, bq, c); };
            auto E3 = [&](int a, int bq, int c) { return A(V_VR, a, bq, c) * A(V_BT, a, bq, c) - A(V_VT, a, bq, c) * A(V_BR, a, bq, c); };
            T q1 = D(c2, [&](int m) { return E3(0, m, 0) * GSIN[jj + m]; }) - D(c3, [&](int m) { return E2(0, 0, m); });
            auto e1s = [&](int m) -> T {   // E1 / sin(theta) at the k-neighbour m
                if constexpr (Pol<T>::exact) return txs[(1 * WP + sp[m + 2]) * PL + jj * NIP + ii];
                else return Pol<T>::dv(E1(0, 0, m), sin_c, sinv);
            };
            T q2 = D(c3, e1s) -
                   D(c1, [&](int m) { return E3(m, 0, 0) * GR[ii + m]; });
            T q3 = D(c1, [&](int m) { return E2(m, 0, 0) * GR[ii + m]; }) - D(c2, [&](int m) { return E1(0, m, 0); });
            q1 = q1 * rinv; q2 = q2 * rinv; q3 = q3 * rinv;
            q1 = q1 * sinv;
            RBr = q1; RBt = q2; RBp = q3;
        }

        // div-B control. GLM cleaning (3_6/ModDivB.f90:13-38), after the
        // equation terms as 3_6/ModAdvance.f90:82-84 orders it: dB += -grad(psi);
        // dpsi = -v_wave^2 div(B) - v_wave/h_LLL psi, v_wave from u^n. Powell
        // (3_5/ModEquation.f90:169-176): dB += -(div B) v.
        T divB = T(0);
        if constexpr (DIVB != 0) {
            // ModSpherical_div of B (3_6/ModSpherical.f90:104-159)
            T dB = D(c1, [&](int m) { return A(V_BR, m, 0, 0) * GR2[ii + m]; });
            dB = dB * r2inv;
            T e23 = D(c2, [&](int m) { return A(V_BT, 0, m, 0) * GSIN[jj + m]; });
            e23 = e23 + D(c3, [&](int m) { return A(V_BP, 0, 0, m); });
            e23 = e23 * sinv;
            e23 = e23 * rinv;
            divB = dB + e23;
        }
        if constexpr (DIVB == 2) {
            RBr = RBr - divB * vr;
            RBt = RBt - divB * vt;
            RBp = RBp - divB * vp;
        }
        if constexpr (DIVB == 1) {
            const T* P = static_cast<const T*>(psi.in) + (size_t)b * NCELL + (size_t)kp * PL + jj * NIP + ii;
            auto Q = [&](int di, int dj, int dk) -> T { return P[(size_t)dk * PL + dj * NIP + di]; };
            // ModSpherical_Grad_f (3_6/ModSpherical.f90:201-239)
            const T g1 = D(c1, [&](int m) { return Q(m, 0, 0); });
            T g2 = D(c2, [&](int m) { return Q(0, m, 0); });
            g2 = g2 * rinv;
            T g3 = D(c3, [&](int m) { return Q(0, 0, m); });
            g3 = g3 * rinv;
            g3 = g3 * sinv;
            RBr = RBr - g1;
            RBt = RBt - g2;
            RBp = RBp - g3;
            // ModWaveSpeed_Dynamo (3_6/ModWaveSpeed.f90:8-27) and h_LLL
            // (3_6/ModBlock.f90:416-425) at this cell, as the CFL pass forms them
            T w = gi[GI_CS * NIP + ii] +
                  sqrt(u0s[V_VR] * u0s[V_VR] + u0s[V_VT] * u0s[V_VT] + u0s[V_VP] * u0s[V_VP]);
            w = w + sqrt(u0s[V_BR] * u0s[V_BR] + u0s[V_BT] * u0s[V_BT] + u0s[V_BP] * u0s[V_BP]) / sqrt(rho0c);
            const T rcell = GR[ii];
            const T h = fmin(fmin(gs[GS_DXI], rcell * gs[GS_DXJ]), rcell * sin_c * gs[GS_DXK]);
            const T Rpsi = -(w * w * divB) - w / h * Q(0, 0, 0);
            const size_t pc = (size_t)b * NCELL + (size_t)kp * PL + jj * NIP + ii;
            const T pn = static_cast<const T*>(psi.un)[pc];
            T po;
            if constexpr (Pol<T>::exact) po = (T)((double)pn + over_divs(dt * (double)Rpsi));
            else po = fmaf((float)dtk, (float)Rpsi, (float)pn);
            static_cast<T*>(psi.out)[pc] = po;
        }

        // stage update
        const T R[NV] = {Rrho, Rvr, Rvt, Rvp, RBr, RBt, RBp, Rs};
        T o[NV];
        if constexpr (Pol<T>::exact) {
#pragma unroll
            for (int v = 0; v < NV; ++v) o[v] = (T)((double)u0s[v] + over_divs(dt * (double)R[v]));
        } else if (ulo != nullptr && stage == 4) {
            // u^{n+1} = u^n + dt*R with u^n and u^{n+1} compensated
            int8_t* ql = ulo + (size_t)b * NV * S::NINT + ((size_t)(kp - 2) * NJ + (jj - 2)) * NI + (ii - 2);
            int8_t q0[NV];
#pragma unroll
            for (int v = 0; v < NV; ++v) q0[v] = ql[(size_t)v * S::NINT];
#pragma unroll
            for (int v = 0; v < NV; v += 2) {   // pairs of variables: ff_add2 gives ff_add's bits
                int8_t qa, qb;
                const float2 ov = ff_add2(f2((float)u0s[v], (float)u0s[v + 1]), q0[v], q0[v + 1],
                                          __fmul2_rn(f2(dtk), f2((float)R[v], (float)R[v + 1])), qa, qb);
                o[v] = ov.x;
                o[v + 1] = ov.y;
                ql[(size_t)v * S::NINT] = qa;
                ql[(size_t)(v + 1) * S::NINT] = qb;
            }
        } else {
#pragma unroll
            for (int v = 0; v < NV; ++v) o[v] = fmaf((float)dtk, (float)R[v], (float)u0s[v]);
        }
#pragma unroll
        for (int v = 0; v < NV; ++v) out[base + (size_t)v * NCELL] = o[v];
        if constexpr (!Pol<T>::exact) {
            if (push.tgt != nullptr) push_faces<T, S>(out, pb, ii, jj, kp, o);
        }
    }
    if (__syncthreads_or(late)) {
        copy_wait_abort(sc, bars, nchunk - 1, nchunk - 1);
        return;
    }
    if (threadIdx.x == 0) {   // every copy has been waited for
        mbar_inval(&bars[0]);
        mbar_inval(&bars[1]);
    }
}
template <class T, int NI, int NJ, int NK, int KPAR, int DIVB>
__global__ void __launch_bounds__(NI* NJ* KPAR, (Shape<T, NI, NJ, NK, KPAR>::min_blocks))
k_stage(const T* in, const T* un, T* out, int8_t* ulo, PushTable push, DivBArgs psi, Geometry g, StepScalars* sc,
        int stage, int bc_writeback, int heat_on) {
    stage_body<T, NI, NJ, NK, KPAR, DIVB>(blockIdx.x, in, un, out, ulo, push, psi, g, sc, stage, bc_writeback, heat_on);
}

// ---------------------------------------------------------------------------
// Artificial diffusion with h=2 (3_6/ModDiffusion.f90:9-150) and the update
// u += 0.5*dt*R (3_6/ModAdvance.f90:101-108), in place.
//
// The reference evaluates, for every cell and direction, the limited fluxes
// through its two faces, so every face flux (and the minmod slopes under it)
// is formed twice. Here each face flux is formed once per chunk of KPAR
// planes into shared memory: i and j faces of the chunk's planes, and the k
// faces in a ring of KPAR+1 face planes (the last face of a chunk is the
// first of the next). A flux is the same function of the same four values as
// the reference's, so sharing it changes no bit. Then each cell sums
// (F_left - F_right)/den over the three directions, in the reference's order.
template <class T, int NI, int NJ, int NK, int KPAR>
struct DShape : Shape<T, NI, NJ, NK, KPAR> {
    using B = Shape<T, NI, NJ, NK, KPAR>;
    static constexpr int NCELLS = NI * NJ * KPAR;        // interior cells of a chunk
    // threads per cell in the sum (variables split): one in FP32, two for a
    // 256-cell FP64 chunk
    static constexpr int TPC = (NCELLS >= 512 || sizeof(T) == 4) ? 1 : 2;
    static constexpr int NT = NCELLS * TPC;
    static constexpr int VPT = NV / TPC;
    static constexpr int KS = KPAR + 1;                  // k-face ring slots
    // FP32, 16-wide rows: a warp takes rows j and j+4 of a plane (80 floats,
    // 16 banks apart) so that its two halves touch disjoint banks in every
    // tile access (rows j and j+1, 20 floats apart, share 4 banks). The i-face
    // rows get a pitch of 20 for the same reason, and the j- and k-face rows
    // are stored in the order rpos() that puts the two rows of a warp side by side.
    static constexpr bool R4 = sizeof(T) == 4 && NI == 16 && NJ % 8 == 0;
    static constexpr int FIP = R4 ? 20 : NI + 1;         // i-face row pitch
    __device__ static __forceinline__ void cell(int c, int& i, int& j, int& kq) {
        kq = c / (NI * NJ);
        const int cc = c % (NI * NJ);
        i = cc % NI;
        if constexpr (R4) {
            const int w = cc / 32;
            j = (w % 4) + 8 * (w / 4) + 4 * ((cc / 16) % 2);
        } else {
            j = cc / NI;
        }
    }
    __device__ static __forceinline__ int rpos(int j) {   // j in [0, NJ]; NJ maps to itself
        if constexpr (R4) return j >= NJ ? NJ : 2 * ((j % 4) + 4 * (j / 8)) + ((j / 4) % 2);
        else return j;
    }
    static constexpr int NFI = NV * KPAR * NJ * FIP;
    static constexpr int NFJ = NV * KPAR * (NJ + 1) * NI;
    static constexpr int NFK = KS * NV * NJ * NI;
    // shared memory: mbarriers | tile[NV][W][PL] | FI | FJ | FK | gi | gj | gs
    static constexpr size_t off_tile = 16;
    static constexpr size_t off_fi = off_tile + (size_t)NV * B::W * B::PL * sizeof(T);
    static constexpr size_t off_fj = off_fi + (size_t)NFI * sizeof(T);
    static constexpr size_t off_fk = off_fj + (size_t)NFJ * sizeof(T);
    static constexpr size_t off_gi = off_fk + (size_t)NFK * sizeof(T);
    static constexpr size_t off_gj = off_gi + (size_t)GI_COUNT * B::NIP * sizeof(T);
    static constexpr size_t off_gs = off_gj + (size_t)GJ_COUNT * B::NJP * sizeof(T);
    static constexpr size_t smem = off_gs + GS_COUNT * sizeof(T);
    static constexpr bool fits = smem <= 232448;         // 227 KB of opt-in shared memory per CTA
    static constexpr int by_smem = (int)(233472 / (smem + 1024));
    static constexpr int reg_cap = 2048 / NT;
    static constexpr int min_blocks =
        sizeof(T) != 4 || by_smem < 2 ? 1 : (by_smem < reg_cap ? by_smem : (reg_cap < 1 ? 1 : reg_cap));
};

// Limited flux through the face between cells L and R along one direction
// (3_6/ModDiffusion.f90:40-60 for one side): values at L-1, L, R, R+1 and
// the speeds |v_dir| + c_s at L and R.
// The limited slope of a cell from its two neighbours along one direction.
template <class T>
__device__ __forceinline__ T face_slope(T ul, T u, T ur) {
    if constexpr (Pol<T>::exact) return minmod(ul, u, ur);
    else return minmod_sel(ul, u, ur);   // the minmod selector as a compare
}
// The flux from the face's two cell values and their slopes.
template <class T>
__device__ __forceinline__ T face_flux_s(T fl, T fr, T dL, T dR, T cL, T cR) {
    if constexpr (Pol<T>::exact) {
        const T num = ((fr - dR * T(0.5)) - fl) - dL * T(0.5);
        const T phi = fmax(T(0), T(1) + T(2) * (Pol<T>::ratio(num, fr - fl) - T(1)));
        const T f = -(T(0.5) * phi * num);
        return f * (cR + cL) * T(0.5);
    } else {
        // the same limiter in fewer FP32 operations: 1 + 2(r - 1) as 2r - 1,
        // the two halves folded
        const float num = fmaf(-0.5f, dL, fmaf(-0.5f, dR, fr) - fl);
        const float phi = fmaxf(0.f, fmaf(2.f, __fdividef(num, fr - fl), -1.f));
        return (-0.25f * phi) * num * (cR + cL);
    }
}
template <class T>
__device__ __forceinline__ T face_flux(T fm, T fl, T fr, T fp, T cL, T cR) {
    return face_flux_s(fl, fr, face_slope(fm, fl, fr), face_slope(fl, fr, fp), cL, cR);
}

//
// In place (out == u), or out of place into `out` (mixed step): then the
// kernel also writes the regular ghost faces of its neighbours in `out`
// (push, as the stage kernel does) and copies the radial physical-boundary
// ghost columns (set by the boundary condition at stage 1) from u to out, so
// that with an exchange of the remaining ghost entries `out` holds the whole
// updated state.
//
// cfl_next (mixed): the outputs are the next step's u^n, so the kernel also
// forms the next step's CFL minimum and NaN flag from them (k_cfl's formula,
// cfl_ratio_f), and that step skips k_cfl.
template <class T, int NI, int NJ, int NK, int KPAR>
__global__ void __launch_bounds__(DShape<T, NI, NJ, NK, KPAR>::NT, (DShape<T, NI, NJ, NK, KPAR>::min_blocks))
k_diffusion(const T* u, T* out, int8_t* ulo, PushTable push, Geometry g, StepScalars* sc, int cfl_next) {
    using S = DShape<T, NI, NJ, NK, KPAR>;
    static_assert(S::fits, "diffusion shared memory above 227 KB");
    constexpr int NIP = S::NIP, PL = S::PL, W = S::W, NCELL = S::NCELL, KS = S::KS;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
    T* tile = reinterpret_cast<T*>(smem + S::off_tile);
    T* FI = reinterpret_cast<T*>(smem + S::off_fi);
    T* FJ = reinterpret_cast<T*>(smem + S::off_fj);
    T* FK = reinterpret_cast<T*>(smem + S::off_fk);
    T* gi = reinterpret_cast<T*>(smem + S::off_gi);
    T* gj = reinterpret_cast<T*>(smem + S::off_gj);
    T* gs = reinterpret_cast<T*>(smem + S::off_gs);
    const int b = blockIdx.x;
    const T* blk = u + (size_t)b * NV * NCELL;
    T* oblk = out + (size_t)b * NV * NCELL;
    const int flb = g.flags[b];
    const bool copy_bc = out != u && (flb & 6);
    __shared__ PushBlock pb;
    load_push_block(push, b, &pb);
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) issue_planes<T, S>(blk, tile, 0, KPAR + 4, &bars[0]);
    // the int8 corrections of u^n are read with plain loads: warm L2 with the
    // first chunk's planes, then one chunk ahead
    const int8_t* blk_lo = ulo != nullptr ? ulo + (size_t)b * NV * S::NINT : nullptr;
    auto prefetch_lo = [&](int kp_first) {
        if (threadIdx.x >= NV) return;
        if (blk_lo != nullptr) prefetch_l2(blk_lo + ((size_t)threadIdx.x * NK + (kp_first - 2)) * S::PLI, KPAR * S::PLI);
    };
    prefetch_lo(2);
    load_geometry<T, S>(g, b, gi, gj, gs, nullptr);
    __syncthreads();   // the geometry tables are read by every thread below
    const int tid = threadIdx.x;
    const T* GCS = gi + GI_CS * NIP;
    // the cell and variables this thread sums and updates
    const int c = tid % S::NCELLS, v0 = (tid / S::NCELLS) * S::VPT;
    int i, j, kq;
    S::cell(c, i, j, kq);
    const int ii = i + 2, jj = j + 2, jr = S::rpos(j), jr1 = S::rpos(j + 1);
    const T rc = gi[GI_R * NIP + ii];
    const T den[3] = {gs[GS_DXI], gs[GS_DXJ] * rc, gs[GS_DXK] * rc * gj[GJ_SIN * S::NJP + jj]};
    const T dinv[3] = {T(1) / den[0], T(1) / den[1], T(1) / den[2]};
    const double hdt = 0.5 * sc->dt;
    const float hdt_f = sc->dt_half_f;
    T sk[S::VPT];            // k slopes carried to the next chunk (one plane per chunk)
#pragma unroll
    for (int t = 0; t < S::VPT; ++t) sk[t] = T(0);
    float cmin = INFINITY;   // next step's CFL ratio minimum over this thread's cells
    int cnan = 0;
    __shared__ float sb2[S::TPC == 2 ? S::NCELLS : 1];   // |B|^2 from the thread holding B
    constexpr int nchunk = NK / KPAR;
    const int polls = sc->wait_polls;
    int late = 0;   // a wait of this thread for a chunk's planes ran out
    for (int ch = 0; ch < nchunk; ++ch) {
        const int k0 = 1 + ch * KPAR;
        const int hi = k0 + KPAR + 3;
        // ring slots and face arrays of the previous chunk are free; a wait of
        // chunk ch-1 that ran out ends the CTA here (chunks ch-1 and ch in flight)
        if (__syncthreads_or(late)) {
            copy_wait_abort(sc, bars, ch - 1, ch);
            return;
        }
        if (threadIdx.x == 0 && ch + 1 < nchunk) issue_planes<T, S>(blk, tile, hi, hi + KPAR, &bars[(ch + 1) & 1]);
        if (ch + 1 < nchunk) prefetch_lo(k0 + KPAR + 1);
        // this thread's int8 corrections, loaded now so that their latency
        // overlaps the copy wait and the face phase
        int8_t qlo[S::VPT];
        if constexpr (!Pol<T>::exact) {
            if (ulo != nullptr) {
                const int8_t* q = ulo + ((size_t)b * NV + v0) * S::NINT +
                                  ((size_t)(k0 - 1 + kq) * NJ + j) * NI + i;
#pragma unroll
                for (int t = 0; t < S::VPT; ++t) qlo[t] = q[(size_t)t * S::NINT];
            }
        }
        // as in the stage kernel: a wait that runs out finishes the chunk on
        // whatever the slots hold; the step is flagged and discarded
        late |= mbar_wait(&bars[ch & 1], (uint32_t)((ch >> 1) & 1), polls) ? 0 : 1;
        const int kp0 = k0 + 1;   // padded index of the chunk's first plane
        const int kp = kp0 + kq;
        if (copy_bc) {   // radial boundary ghost columns of the planes new to this chunk
            const int plo = ch == 0 ? 0 : k0 + 3, phi = k0 + KPAR + 3, fl = flb;
            const int total = (phi - plo) * S::NJP * NV * 4;
            for (int x = tid; x < total; x += S::NT) {
                const int c4 = x & 3, r = x >> 2;
                const int v = r % NV, r2 = r / NV;
                const int y = r2 % S::NJP, z = plo + r2 / S::NJP;
                if (!((c4 < 2) ? (fl & 4) : (fl & 2))) continue;
                const int xi = c4 < 2 ? c4 : NI + c4;   // 0, 1 (bottom) or NI+2, NI+3 (top)
                oblk[((size_t)v * S::NKP + z) * PL + y * NIP + xi] = tile[(v * W + z % W) * PL + y * NIP + xi];
            }
        }
        // ring offsets of planes kp-2 .. kp+2
        int so[5];
        so[0] = ((kp - 2) % W) * PL;
#pragma unroll
        for (int d = 1; d < 5; ++d) so[d] = so[d - 1] + PL >= W * PL ? so[d - 1] + PL - W * PL : so[d - 1] + PL;
        const T* t0 = tile + jj * NIP + ii;   // this cell's column in every plane
        // this cell's left i and j faces and right k face, for its variables
        {
            const T* tc = t0 + so[2];
            const T cLi = fabs(tc[V_VR * W * PL - 1]) + GCS[ii - 1], cRi = fabs(tc[V_VR * W * PL]) + GCS[ii];
            const T cs = GCS[ii];
            const T cLj = fabs(tc[V_VT * W * PL - NIP]) + cs, cRj = fabs(tc[V_VT * W * PL]) + cs;
            const T cLk = fabs(t0[V_VP * W * PL + so[2]]) + cs, cRk = fabs(t0[V_VP * W * PL + so[3]]) + cs;
            T* fkw = FK + ((size_t)((kp - 1) % KS) * NV) * NJ * NI + jr * NI + i;
#pragma unroll
            for (int t = 0; t < S::VPT; ++t) {
                const int v = v0 + t;
                const T* a = tc + v * W * PL;
                FI[((v * KPAR + kq) * NJ + j) * S::FIP + i] = face_flux(a[-2], a[-1], a[0], a[1], cLi, cRi);
                FJ[((v * KPAR + kq) * (NJ + 1) + jr) * NI + i] =
                    face_flux(a[-2 * NIP], a[-NIP], a[0], a[NIP], cLj, cRj);
                // the k face's slopes: with one plane per chunk the lower one
                // is the upper one of the previous chunk (same values, same bits)
                const T* ak = t0 + v * W * PL;
                const T dRk = face_slope(ak[so[2]], ak[so[3]], ak[so[4]]);
                T dLk;
                if constexpr (KPAR == 1) {
                    dLk = ch == 0 ? face_slope(ak[so[1]], ak[so[2]], ak[so[3]]) : sk[t];
                    sk[t] = dRk;
                } else {
                    dLk = face_slope(ak[so[1]], ak[so[2]], ak[so[3]]);
                }
                fkw[v * NJ * NI] = face_flux_s(ak[so[2]], ak[so[3]], dLk, dRk, cLk, cRk);
            }
        }
        // the right faces of the last cells of i rows and j columns
        constexpr int NXI = NV * KPAR * NJ, NXJ = NV * KPAR * NI;
        for (int x = tid; x < NXI + NXJ; x += S::NT) {
            if (x < NXI) {
                const int y = x % NJ + 2, q = (x / NJ) % KPAR, v = x / (NJ * KPAR);
                const T* a = tile + (v * W + (kp0 + q) % W) * PL + y * NIP + NI + 1;   // last interior cell
                const T* vr = tile + (V_VR * W + (kp0 + q) % W) * PL + y * NIP + NI + 1;
                const T cL = fabs(vr[0]) + GCS[NI + 1], cR = fabs(vr[1]) + GCS[NI + 2];
                FI[((v * KPAR + q) * NJ + (y - 2)) * S::FIP + NI] = face_flux(a[-1], a[0], a[1], a[2], cL, cR);
            } else {
                const int z = x - NXI;
                const int xx = z % NI + 2, q = (z / NI) % KPAR, v = z / (NI * KPAR);
                const T* a = tile + (v * W + (kp0 + q) % W) * PL + (NJ + 1) * NIP + xx;
                const T* vt = tile + (V_VT * W + (kp0 + q) % W) * PL + (NJ + 1) * NIP + xx;
                const T cs = GCS[xx];
                const T cL = fabs(vt[0]) + cs, cR = fabs(vt[NIP]) + cs;
                FJ[((v * KPAR + q) * (NJ + 1) + NJ) * NI + (xx - 2)] =
                    face_flux(a[-NIP], a[0], a[NIP], a[2 * NIP], cL, cR);
            }
        }
        // first chunk: the k faces below the first plane (between padded planes 1 and 2)
        if (ch == 0) {
            for (int x = tid; x < NV * NJ * NI; x += S::NT) {
                const int xx = x % NI + 2, y = (x / NI) % NJ + 2, v = x / (NI * NJ);
                const T* a = tile + (size_t)v * W * PL + y * NIP + xx;
                const T* vp = tile + (size_t)V_VP * W * PL + y * NIP + xx;
                const T cs = GCS[xx];
                const T cL = fabs(vp[PL]) + cs, cR = fabs(vp[2 * PL]) + cs;
                FK[((0 * NV + v) * NJ + S::rpos(y - 2)) * NI + (xx - 2)] =
                    face_flux(a[0], a[PL], a[2 * PL], a[3 * PL], cL, cR);
            }
        }
        __syncthreads();
        const size_t base = (size_t)kp * PL + jj * NIP + ii;
        const T* fk_l = FK + ((size_t)((kp - 2) % KS) * NV) * NJ * NI + jr * NI + i;
        const T* fk_r = FK + ((size_t)((kp - 1) % KS) * NV) * NJ * NI + jr * NI + i;
        T o[S::VPT];
#pragma unroll
        for (int t = 0; t < S::VPT; ++t) {
            const int v = v0 + t;
            const T* fi = FI + ((v * KPAR + kq) * NJ + j) * S::FIP + i;
            const T* fj = FJ + ((v * KPAR + kq) * (NJ + 1)) * NI + i;
            T R = T(0);
            R = R + Pol<T>::dv(fi[0] - fi[1], den[0], dinv[0]);
            R = R + Pol<T>::dv(fj[jr * NI] - fj[jr1 * NI], den[1], dinv[1]);
            R = R + Pol<T>::dv(fk_l[v * NJ * NI] - fk_r[v * NJ * NI], den[2], dinv[2]);
            const T u0 = t0[v * W * PL + so[2]];
            if constexpr (Pol<T>::exact) {
                o[t] = (T)((double)u0 + hdt * (double)R);
            } else if (ulo != nullptr) {
                int8_t q1;
                o[t] = ff_add((float)u0, qlo[t], __fmul_rn(hdt_f, (float)R), q1);
                ulo[((size_t)b * NV + v) * S::NINT + ((size_t)(kp - 2) * NJ + j) * NI + i] = q1;
            } else {
                o[t] = fmaf(hdt_f, (float)R, (float)u0);
            }
            oblk[(size_t)v * NCELL + base] = o[t];
        }
        if constexpr (!Pol<T>::exact) {
            if (push.tgt != nullptr) push_faces_part<T, S, S::VPT>(out, pb, ii, jj, kp, o, v0);
            if (cfl_next) {   // uniform over the CTA
#pragma unroll
                for (int t = 0; t < S::VPT; ++t) cnan |= (o[t] != o[t]);
                float v2 = 0.f, b2 = 0.f;
                if constexpr (S::TPC == 1) {
                    v2 = cfl_sq3(o[V_VR], o[V_VT], o[V_VP]);
                    b2 = cfl_sq3(o[V_BR], o[V_BT], o[V_BP]);
                } else {
                    if (v0 != 0) sb2[c] = cfl_sq3(o[V_BR - 4], o[V_BT - 4], o[V_BP - 4]);
                    __syncthreads();
                    if (v0 == 0) {
                        v2 = cfl_sq3(o[V_VR], o[V_VT], o[V_VP]);
                        b2 = sb2[c];
                    }
                }
                if (v0 == 0) {
                    float ratio = cfl_ratio_f(v2, b2, GCS[ii], gi[GI_RHO0 * NIP + ii], rc, gj[GJ_SIN * S::NJP + jj],
                                              gs[GS_DXI], gs[GS_DXJ], gs[GS_DXK]);
                    if (ratio != ratio) { cnan = 1; ratio = INFINITY; }
                    cmin = fminf(cmin, ratio);
                }
            }
        }
    }
    if (__syncthreads_or(late)) {
        copy_wait_abort(sc, bars, nchunk - 1, nchunk - 1);
        return;
    }
    if constexpr (!Pol<T>::exact) {
        if (cfl_next) cfl_commit(cmin, cnan, sc);
    }
}

// ---------------------------------------------------------------------------
// FP32 artificial diffusion of one 16^3 block as a march along k (the mixed
// step's diffusion pass; same arguments and results as k_diffusion).
//
// One thread per (i, j) column of the block (256 threads), marching k over the
// 16 interior planes. Along k everything stays in registers: the column's
// values at planes kp and kp+1, its k slope at kp and the flux through the
// face below kp; per plane the thread reads one new value per variable (plane
// kp+2, from the ring), forms one k slope and one k face. Across the plane,
// every i and j slope is formed once (phase A, into shared memory, ghost
// columns and rows by the same threads), then every i and j face flux once
// (phase B), then each cell sums its six faces and updates (phase C). Per
// cell and variable that is 3 slopes and 3 fluxes, the minimum; the face
// fluxes are the same functions of the same values as k_diffusion's, summed
// in the same order. The arithmetic runs on pairs of variables (packed FP32
// instructions, above), and the slope and face arrays hold the pairs side by
// side, so their shared-memory accesses are 64-bit.
//
// Planes arrive by bulk copy into a ring of 5 slots, one mbarrier each: the
// column window needs planes kp..kp+2, and the slot of plane kp is refilled
// with plane kp+5 once phase B of plane kp has passed its barrier (planes
// kp+3 and kp+4 are in flight meanwhile). A warp takes rows j and j+4
// (half-warps of 16 cells), so a half-warp holds one row, as the pushed
// radial faces need.
template <int NI, int NJ, int NK, int TPC>
struct MShape {
    static constexpr int NG = 2, NIP = NI + 4, NJP = NJ + 4, NKP = NK + 4;
    static constexpr int PL = NIP * NJP, NCELL = PL * NKP;
    static constexpr int NCOL = NI * NJ, NT = NCOL * TPC;   // columns; threads (TPC per column)
    static constexpr int W = 5;                          // plane ring slots
    static constexpr int PLI = NI * NJ, NINT = PLI * NK;
    static constexpr int NP = NV / 2, PPT = NP / TPC;    // variable pairs; pairs per thread
    static constexpr uint32_t PLB = PL * 4u;
    static constexpr int P = 20;                         // row pitch (pairs) of the slope and face arrays
    // per pair (float2): SI[NJ][P] slopes along i of cells i = -1..NI at i + 1;
    // SJ[NJ + 2][P] slopes along j of rows j = -1..NJ at row j + 1;
    // FI[NJ][P] fluxes through faces i - 1/2, i = 0..NI; FJ[NJ + 1][P] likewise along j
    static constexpr int NSI = NJ * P, NSJ = (NJ + 2) * P, NFI = NJ * P, NFJ = (NJ + 1) * P;
    // shared memory: mbarriers | tile[NV][W][PL] | SI | SJ | FI | FJ | gi | gj | gs
    static constexpr size_t off_tile = 64;
    static constexpr size_t off_si = off_tile + (size_t)NV * W * PL * 4;
    static constexpr size_t off_sj = off_si + (size_t)NP * NSI * 8;
    static constexpr size_t off_fi = off_sj + (size_t)NP * NSJ * 8;
    static constexpr size_t off_fj = off_fi + (size_t)NP * NFI * 8;
    static constexpr size_t off_gi = off_fj + (size_t)NP * NFJ * 8;
    static constexpr size_t off_gj = off_gi + (size_t)GI_COUNT * NIP * 4;
    static constexpr size_t off_gs = off_gj + (size_t)GJ_COUNT * NJP * 4;
    // two threads per column: |B|^2 of the second half, [plane parity][column]
    static constexpr size_t off_sb2 = off_gs + GS_COUNT * 4;
    static constexpr size_t smem = off_sb2 + (TPC == 2 ? 2 * NCOL * 4 : 0);
    static_assert(W * 8 <= (int)off_tile, "mbarriers");
    static_assert(off_si % 8 == 0, "float2 arrays");
    static_assert(TPC == 1 || TPC == 2, "one or two threads per column");
};

// TPC threads per column: with two, thread half h = tid / 256 takes the
// variable pairs 2h, 2h+1 (warps never mix halves), doubling the warps per SM
// at half the registers; the CFL ratio, which needs v (first half) and B
// (second half), takes |B|^2 through shared memory one plane later.
template <int NI, int NJ, int NK, int TPC>
__device__ __forceinline__ void march_body(int b, const float* u, float* out, int8_t* ulo, PushTable push, Geometry g,
                                           StepScalars* sc, int cfl_next) {
    using S = MShape<NI, NJ, NK, TPC>;
    static_assert(NI == 16 && NJ == 16, "rows of 16 cells: one half-warp per row");
    static_assert(2 * (S::smem + 1024) <= 233472, "two CTAs per SM");
    constexpr int NIP = S::NIP, PL = S::PL, W = S::W, NCELL = S::NCELL, P = S::P, PPT = S::PPT;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
    float* tile = reinterpret_cast<float*>(smem + S::off_tile);
    float2* SI = reinterpret_cast<float2*>(smem + S::off_si);
    float2* SJ = reinterpret_cast<float2*>(smem + S::off_sj);
    float2* FI = reinterpret_cast<float2*>(smem + S::off_fi);
    float2* FJ = reinterpret_cast<float2*>(smem + S::off_fj);
    float* gi = reinterpret_cast<float*>(smem + S::off_gi);
    float* gj = reinterpret_cast<float*>(smem + S::off_gj);
    float* gs = reinterpret_cast<float*>(smem + S::off_gs);
    float* sb2 = reinterpret_cast<float*>(smem + S::off_sb2);   // |B|^2 of the second half, by plane parity
    const int tid = threadIdx.x;
    const float* blk = u + (size_t)b * NV * NCELL;
    float* oblk = out + (size_t)b * NV * NCELL;
    const int flb = g.flags[b];
    const bool copy_bc = out != u && (flb & 6);
    __shared__ PushBlock pb;
    load_push_block(push, b, &pb);
    if (tid == 0) {
        for (int s = 0; s < W; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    int issued = 0;   // thread 0: planes [0, issued) have been requested
    if (tid == 0) {
        for (int p = 0; p < W; ++p) issue_planes<float, S>(blk, tile, p, p + 1, &bars[p]);
        issued = W;
    }
    const int8_t* blk_lo = ulo != nullptr ? ulo + (size_t)b * NV * S::NINT : nullptr;
    if (blk_lo != nullptr && tid < NV) prefetch_l2(blk_lo + (size_t)tid * S::NINT, 2 * S::PLI);
    load_geometry<float, S>(g, b, gi, gj, gs, nullptr);
    __syncthreads();   // the geometry tables are read by every thread below
    // this thread's column: warp w takes rows (w % 4) + 8 (w / 4) and that + 4;
    // its pairs p0 .. p0 + PPT - 1
    const int c = tid % S::NCOL, half = tid / S::NCOL, p0 = half * PPT, v0 = 2 * p0;
    const int wq = c >> 5, i = c & 15;
    const int j = (wq & 3) + 8 * (wq >> 2) + 4 * ((c >> 4) & 1);
    const int ii = i + 2, jj = j + 2;
    const float* GCS = gi + GI_CS * NIP;
    const float cs = GCS[ii];
    const float rc = gi[GI_R * NIP + ii];
    const float den[3] = {gs[GS_DXI], gs[GS_DXJ] * rc, gs[GS_DXK] * rc * gj[GJ_SIN * S::NJP + jj]};
    const float2 dinv0 = f2(1.f / den[0]), dinv1 = f2(1.f / den[1]), dinv2 = f2(1.f / den[2]);
    const float2 hdt2 = f2(sc->dt_half_f);
    const int polls = sc->wait_polls;
    int late = 0;   // a wait of this thread for a plane ran out
    auto abort_cta = [&]() {   // after a uniform decision: flag, drain the copies in flight
        if (tid != 0) return;
        atomicOr(&sc->nan_flag, 2);
        for (int p = issued - W < 0 ? 0 : issued - W; p < issued; ++p)
            mbar_wait(&bars[p % W], (uint32_t)((p / W) & 1), kWaitPolls);
        for (int q = 0; q < W; ++q) mbar_inval(&bars[q]);
    };
    // radial boundary ghost columns of planes [plo, phi), u -> out
    auto copy_cols = [&](int plo, int phi) {
        const int total = (phi - plo) * S::NJP * NV * 4;
        for (int x = tid; x < total; x += S::NT) {
            const int c4 = x & 3, r = x >> 2;
            const int v = r % NV, r2 = r / NV;
            const int y = r2 % S::NJP, z = plo + r2 / S::NJP;
            if (!((c4 < 2) ? (flb & 4) : (flb & 2))) continue;
            const int xi = c4 < 2 ? c4 : NI + c4;   // 0, 1 (bottom) or NI+2, NI+3 (top)
            oblk[((size_t)v * S::NKP + z) * PL + y * NIP + xi] = tile[(v * W + z % W) * PL + y * NIP + xi];
        }
    };
    // the pair (v, v+1) of a tile value, p = v / 2, at offset o from variable 0's
    auto tv = [&](const float* base, int p) { return f2(base[2 * p * W * PL], base[(2 * p + 1) * W * PL]); };
    // the column window from planes 0..3: u at kp = 2 and 3, the k slope at 2,
    // the flux through the face between planes 1 and 2
    for (int p = 0; p < 4; ++p) late |= mbar_wait(&bars[p], 0u, polls) ? 0 : 1;
    if (copy_bc) copy_cols(0, 4);
    const float* col = tile + jj * NIP + ii;
    const float* colvp = col + V_VP * W * PL;
    float2 u0[PPT], u1[PPT], dk0[PPT], fk0[PPT];
    {
        const float2 cc = f2(-0.25f * ((fabsf(colvp[2 * PL]) + cs) + (fabsf(colvp[PL]) + cs)));
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            const int p = p0 + q;
            const float2 a0 = tv(col, p), a1 = tv(col + PL, p), a2 = tv(col + 2 * PL, p), a3 = tv(col + 3 * PL, p);
            const float2 d1 = minmod_sel2(a0, a1, a2), d2 = minmod_sel2(a1, a2, a3);
            u0[q] = a2;
            u1[q] = a3;
            dk0[q] = d2;
            fk0[q] = face_flux2(a1, a2, d1, d2, cc);
        }
    }
    float cmin = INFINITY;   // next step's CFL ratio minimum over this column
    int cnan = 0;
    float v2_prev = 0.f;     // two threads per column: the first half's |v|^2 of the previous plane
    const float rho0c = gi[GI_RHO0 * NIP + ii], sin_c = gj[GJ_SIN * S::NJP + jj];
    auto cfl_point = [&](float v2, float b2) {
        float ratio = cfl_ratio_f(v2, b2, cs, rho0c, rc, sin_c, gs[GS_DXI], gs[GS_DXJ], gs[GS_DXK]);
        if (ratio != ratio) { cnan = 1; ratio = INFINITY; }
        cmin = fminf(cmin, ratio);
    };
    for (int kp = 2; kp < NK + 2; ++kp) {
        const int p2 = kp + 2;
        if (blk_lo != nullptr && tid < NV && kp < NK) prefetch_l2(blk_lo + (size_t)tid * S::NINT + (size_t)kp * S::PLI, S::PLI);
        // this cell's int8 corrections, loaded before the wait
        int8_t qlo[2 * PPT];
        if (ulo != nullptr) {
            const int8_t* q = blk_lo + (size_t)v0 * S::NINT + ((size_t)(kp - 2) * NJ + j) * NI + i;
#pragma unroll
            for (int v = 0; v < 2 * PPT; ++v) qlo[v] = q[(size_t)v * S::NINT];
        }
        // a wait that runs out finishes the plane on whatever the slot holds;
        // the step is flagged and discarded
        late |= mbar_wait(&bars[p2 % W], (uint32_t)((p2 / W) & 1), polls) ? 0 : 1;
        if (copy_bc) copy_cols(p2, p2 + 1);
        const int s0 = (kp % W) * PL, s1 = ((kp + 1) % W) * PL, s2 = (p2 % W) * PL;
        const float* tc = tile + s0 + jj * NIP + ii;   // this cell in plane kp (+ v W PL)
        // ---- phase A: k slope and k face from the window; i and j slopes
        float2 u2[PPT], dk1[PPT], fk1[PPT];
        {
            const float2 cc = f2(-0.25f * ((fabsf(colvp[s1]) + cs) + (fabsf(colvp[s0]) + cs)));
#pragma unroll
            for (int q = 0; q < PPT; ++q) {
                const int p = p0 + q;
                u2[q] = tv(col + s2, p);
                dk1[q] = minmod_sel2(u0[q], u1[q], u2[q]);
                fk1[q] = face_flux2(u0[q], u1[q], dk0[q], dk1[q], cc);
                SI[p * S::NSI + j * P + i + 1] = minmod_sel2(tv(tc - 1, p), u0[q], tv(tc + 1, p));
                SJ[p * S::NSJ + (j + 1) * P + i] = minmod_sel2(tv(tc - NIP, p), u0[q], tv(tc + NIP, p));
            }
        }
        // slopes of the ghost cells next to the block: i = -1, NI of every row
        // (items 0..255) and j = -1, NJ of every column (items 256..511)
#pragma unroll
        for (int x = tid; x < 512; x += S::NT) {
            const int side = x & 1, r = (x >> 1) & 15, v = (x >> 5) & 7;
            const float* a = tile + v * W * PL + s0;
            float* dst;
            float val;
            if (x < 256) {
                const float* q = a + (r + 2) * NIP + (side ? NI + 2 : 1);
                val = face_slope(q[-1], q[0], q[1]);
                dst = reinterpret_cast<float*>(SI + (v >> 1) * S::NSI + r * P + (side ? NI + 1 : 0));
            } else {
                const float* q = a + (side ? NJ + 2 : 1) * NIP + r + 2;
                val = face_slope(q[-NIP], q[0], q[NIP]);
                dst = reinterpret_cast<float*>(SJ + (v >> 1) * S::NSJ + (side ? NJ + 1 : 0) * P + r);
            }
            dst[v & 1] = val;
        }
        if (__syncthreads_or(late)) {
            abort_cta();
            return;
        }
        // ---- phase B: the faces i - 1/2 and j - 1/2 of this cell, and the
        // last faces of the rows (items 0..127) and columns (128..255)
        float2 fi0[PPT], fj0[PPT];
        {
            const float cLi = fabsf(tc[V_VR * W * PL - 1]) + GCS[ii - 1], cRi = fabsf(tc[V_VR * W * PL]) + cs;
            const float cLj = fabsf(tc[V_VT * W * PL - NIP]) + cs, cRj = fabsf(tc[V_VT * W * PL]) + cs;
            const float2 cci = f2(-0.25f * (cRi + cLi)), ccj = f2(-0.25f * (cRj + cLj));
#pragma unroll
            for (int q = 0; q < PPT; ++q) {
                const int p = p0 + q;
                const float2* si = SI + p * S::NSI + j * P + i;
                const float2* sj = SJ + p * S::NSJ + j * P + i;
                fi0[q] = face_flux2(tv(tc - 1, p), u0[q], si[0], si[1], cci);
                fj0[q] = face_flux2(tv(tc - NIP, p), u0[q], sj[0], sj[P], ccj);
                FI[p * S::NFI + j * P + i] = fi0[q];
                FJ[p * S::NFJ + j * P + i] = fj0[q];
            }
        }
        if (tid < 256) {
            const int x = tid, r = x & 15, v = (x >> 4) & 7;
            const float* sl = reinterpret_cast<const float*>(x < 128 ? SI + (v >> 1) * S::NSI + r * P + NI
                                                                     : SJ + (v >> 1) * S::NSJ + NJ * P + r);
            if (x < 128) {
                const float* a = tile + v * W * PL + s0 + (r + 2) * NIP + NI + 1;   // last interior cell of row r
                const float* vr = tile + V_VR * W * PL + s0 + (r + 2) * NIP + NI + 1;
                const float cL = fabsf(vr[0]) + GCS[NI + 1], cR = fabsf(vr[1]) + GCS[NI + 2];
                reinterpret_cast<float*>(FI + (v >> 1) * S::NFI + r * P + NI)[v & 1] =
                    face_flux_s(a[0], a[1], sl[v & 1], sl[2 + (v & 1)], cL, cR);
            } else {
                const float* a = tile + v * W * PL + s0 + (NJ + 1) * NIP + r + 2;   // last interior row, column r
                const float* vt = tile + V_VT * W * PL + s0 + (NJ + 1) * NIP + r + 2;
                const float c2 = GCS[r + 2];
                const float cL = fabsf(vt[0]) + c2, cR = fabsf(vt[NIP]) + c2;
                reinterpret_cast<float*>(FJ + (v >> 1) * S::NFJ + NJ * P + r)[v & 1] =
                    face_flux_s(a[0], a[NIP], sl[v & 1], sl[2 * P + (v & 1)], cL, cR);
            }
        }
        __syncthreads();
        // planes below kp + 1 are done with: refill their slots, up to plane
        // kp + W (at kp = 2 that is planes 5, 6, 7; then one plane a step)
        if (tid == 0) {
            for (; issued < S::NKP && issued <= kp + W; ++issued)
                issue_planes<float, S>(blk, tile, issued, issued + 1, &bars[issued % W]);
        }
        // ---- phase C: sum the six faces in the reference's order, update
        const size_t base = (size_t)kp * PL + jj * NIP + ii;
        float o[2 * PPT];
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            const int p = p0 + q;
            float2 R = __fmul2_rn(sub2(fi0[q], FI[p * S::NFI + j * P + i + 1]), dinv0);
            R = __ffma2_rn(sub2(fj0[q], FJ[p * S::NFJ + (j + 1) * P + i]), dinv1, R);
            R = __ffma2_rn(sub2(fk0[q], fk1[q]), dinv2, R);
            float2 ov;
            if (ulo != nullptr) {
                int8_t q0, q1;
                ov = ff_add2(u0[q], qlo[2 * q], qlo[2 * q + 1], __fmul2_rn(hdt2, R), q0, q1);
                int8_t* qo = ulo + ((size_t)b * NV + 2 * p) * S::NINT + ((size_t)(kp - 2) * NJ + j) * NI + i;
                qo[0] = q0;
                qo[S::NINT] = q1;
            } else {
                ov = __ffma2_rn(hdt2, R, u0[q]);
            }
            o[2 * q] = ov.x;
            o[2 * q + 1] = ov.y;
            oblk[(size_t)(2 * p) * NCELL + base] = ov.x;
            oblk[(size_t)(2 * p + 1) * NCELL + base] = ov.y;
        }
        if (push.tgt != nullptr) push_faces_part<float, S, 2 * PPT>(out, pb, ii, jj, kp, o, v0);
        if (cfl_next) {   // uniform over the CTA
#pragma unroll
            for (int v = 0; v < 2 * PPT; ++v) cnan |= (o[v] != o[v]);
            if constexpr (TPC == 1) {
                cfl_point(cfl_sq3(o[V_VR], o[V_VT], o[V_VP]), cfl_sq3(o[V_BR], o[V_BT], o[V_BP]));
            } else if (half == 0) {
                if (kp > 2) cfl_point(v2_prev, sb2[((kp - 1) & 1) * S::NCOL + c]);
                v2_prev = cfl_sq3(o[V_VR], o[V_VT], o[V_VP]);
            } else {
                sb2[(kp & 1) * S::NCOL + c] = cfl_sq3(o[V_BR - 4], o[V_BT - 4], o[V_BP - 4]);
            }
        }
        // the window moves up one plane
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            u0[q] = u1[q];
            u1[q] = u2[q];
            dk0[q] = dk1[q];
            fk0[q] = fk1[q];
        }
    }
    if (__syncthreads_or(late)) {
        abort_cta();
        return;
    }
    if constexpr (TPC == 2) {
        if (cfl_next && half == 0) cfl_point(v2_prev, sb2[((NK + 1) & 1) * S::NCOL + c]);
    }
    if (tid == 0)   // every copy has been waited for
        for (int q = 0; q < W; ++q) mbar_inval(&bars[q]);
    if (cfl_next) cfl_commit(cmin, cnan, sc);
}
template <int NI, int NJ, int NK, int TPC>
__global__ void __launch_bounds__(NI * NJ * TPC, 2)
k_diffusion_march(const float* u, float* out, int8_t* ulo, PushTable push, Geometry g, StepScalars* sc, int cfl_next) {
    march_body<NI, NJ, NK, TPC>(blockIdx.x, u, out, ulo, push, g, sc, cfl_next);
}

// ---------------------------------------------------------------------------
// Every cell outside the core of each block and variable set to 0 (the k ghost
// planes and, in the interior planes, the j ghost rows: per block and
// variable, (NJP-4)*NIP-wide gaps between the core runs). A core upload clears
// them before its exchange refills the listed ones: the mixed interpolations
// read some ghost cells of their source blocks with weight 0, which is
// harmless for finite values only, and the buffer may hold an earlier state
// with NaNs there. Cleared, the uploaded state's ghost cells are the same
// whatever the buffer held (a new context starts with zeros too).
template <class T>
__global__ void __launch_bounds__(256) k_clear_outside_core(T* u, int64_t nbv, StepDims d) {
    const int pl = d.nip * d.njp, lead = 2 * pl + 2 * d.nip, gap = 4 * d.nip;
    const int per = 2 * lead + (d.nkp - 5) * gap;   // non-core cells per block and variable
    for (int64_t bv = blockIdx.x; bv < nbv; bv += gridDim.x) {
        T* base = u + bv * d.ncell;
        for (int x = threadIdx.x; x < per; x += blockDim.x) {
            int c;
            if (x < lead) {
                c = x;                                   // planes 0, 1 and rows 0, 1 of plane 2
            } else if (x < per - lead) {
                const int q = (x - lead) / gap, r = (x - lead) - q * gap;
                c = (2 + q) * pl + (d.njp - 2) * d.nip + r;   // rows NJP-2, NJP-1 of plane 2+q, rows 0, 1 of the next
            } else {
                c = d.ncell - lead + (x - (per - lead));   // rows NJP-2, NJP-1 of the last interior plane, 2 ghost planes
            }
            base[c] = T(0);
        }
    }
}

// ---------------------------------------------------------------------------
// After the core of a mixed state has been replaced from the host (the core
// upload), what the diffusion pass closing a mixed step leaves besides
// u^{n+1} itself: the regular faces pushed into the neighbours' ghost layers
// (the face entries left to the final exchange follow as a separate launch),
// and the next step's CFL minimum with the NaN scan, each cell's ratio the
// one k_cfl forms. One CTA per block and a thread per (i, j) column marching
// k; a row of NI cells lies in consecutive lanes, as the pushed radial faces
// need.
template <int NI, int NJ, int NK>
__global__ void __launch_bounds__(NI * NJ) k_push_state(float* u, PushTable push, Geometry g, StepScalars* sc) {
    using S = MShape<NI, NJ, NK, 1>;
    constexpr int NIP = S::NIP, NJP = S::NJP;
    static_assert((NI * NJ) % 32 == 0 && 32 % NI == 0, "whole rows in every warp");
    __shared__ PushBlock pb;
    const int b = blockIdx.x, tid = threadIdx.x;
    load_push_block(push, b, &pb);
    __syncthreads();
    const int ii = tid % NI + 2, jj = tid / NI + 2;
    const float* Gi = gi_ptr<float>(g) + (size_t)b * GI_COUNT * NIP;
    const float* Gj = gj_ptr<float>(g) + (size_t)b * GJ_COUNT * NJP;
    const float* Gs = gs_ptr<float>(g) + (size_t)b * GS_COUNT;
    const float cs = Gi[GI_CS * NIP + ii], rho0 = Gi[GI_RHO0 * NIP + ii], r = Gi[GI_R * NIP + ii];
    const float sin_t = Gj[GJ_SIN * NJP + jj], dxi = Gs[GS_DXI], dxj = Gs[GS_DXJ], dxk = Gs[GS_DXK];
    const float* blk = u + (size_t)b * NV * S::NCELL;
    float cmin = INFINITY;
    int cnan = 0;
    constexpr int G = 4;   // planes whose loads are all issued before the first push
    static_assert(NK % G == 0, "whole plane groups");
    for (int k0 = 2; k0 < NK + 2; k0 += G) {
        float o[G][NV];
#pragma unroll
        for (int q = 0; q < G; ++q) {
            const size_t base = ((size_t)(k0 + q) * NJP + jj) * NIP + ii;
#pragma unroll
            for (int v = 0; v < NV; ++v) o[q][v] = blk[(size_t)v * S::NCELL + base];
        }
#pragma unroll
        for (int q = 0; q < G; ++q) {
            if (push.tgt != nullptr) push_faces_part<float, S, NV>(u, pb, ii, jj, k0 + q, o[q], 0);
#pragma unroll
            for (int v = 0; v < NV; ++v) cnan |= (o[q][v] != o[q][v]);
            float ratio = cfl_ratio_f(cfl_sq3(o[q][V_VR], o[q][V_VT], o[q][V_VP]),
                                      cfl_sq3(o[q][V_BR], o[q][V_BT], o[q][V_BP]), cs, rho0, r, sin_t, dxi, dxj, dxk);
            if (ratio != ratio) { cnan = 1; ratio = INFINITY; }
            cmin = fminf(cmin, ratio);
        }
    }
    cfl_commit(cmin, cnan, sc);
}

// ---------------------------------------------------------------------------
// FP64 artificial diffusion (3_6/ModDiffusion.f90:9-150) of one block as a k
// march, in place (the exact path: no pushes, no fused CFL minimum, no u^n
// correction). One thread per (cell column, variable): NI*NJ*NV threads. The
// k window, slope and face of the thread's column and variable stay in
// registers; across each plane every i and j slope is formed once, then every
// i and j face flux, then each cell sums its six faces. The fluxes are the
// chunked kernel's functions of the same four values and the sum runs in the
// reference's order (i, j, k, each as a division by its denominator), so the
// result is the same bit for bit, with 3 minmod slopes per cell and variable
// where the chunked kernel forms 5 or 6.
template <int NI, int NJ, int NK>
struct M64Shape {
    static constexpr int NG = 2, NIP = NI + 4, NJP = NJ + 4, NKP = NK + 4;
    static constexpr int PL = NIP * NJP, NCELL = PL * NKP;
    static constexpr int NCOL = NI * NJ, NT = NCOL * NV;
    static constexpr int W = 5;                          // plane ring slots
    static constexpr uint32_t PLB = PL * 8u;
    static constexpr int P = NI + 2;                     // row pitch of the slope and face arrays
    // per variable: SI[NJ][P] (cells i = -1..NI at i + 1), SJ[NJ + 2][P]
    // (rows j = -1..NJ at j + 1), FI[NJ][P] (faces i - 1/2, i = 0..NI), FJ[NJ + 1][P]
    static constexpr int NSI = NJ * P, NSJ = (NJ + 2) * P, NFI = NJ * P, NFJ = (NJ + 1) * P;
    // shared memory: mbarriers | tile[NV][W][PL] | SI | SJ | FI | FJ | gi | gj | gs
    static constexpr size_t off_tile = 64;
    static constexpr size_t off_si = off_tile + (size_t)NV * W * PL * 8;
    static constexpr size_t off_sj = off_si + (size_t)NV * NSI * 8;
    static constexpr size_t off_fi = off_sj + (size_t)NV * NSJ * 8;
    static constexpr size_t off_fj = off_fi + (size_t)NV * NFI * 8;
    static constexpr size_t off_gi = off_fj + (size_t)NV * NFJ * 8;
    static constexpr size_t off_gj = off_gi + (size_t)GI_COUNT * NIP * 8;
    static constexpr size_t off_gs = off_gj + (size_t)GJ_COUNT * NJP * 8;
    static constexpr size_t smem = off_gs + GS_COUNT * 8;
    static_assert(NT <= 1024, "one thread per column and variable");
};

template <int NI, int NJ, int NK>
__global__ void __launch_bounds__(NI * NJ * NV)
k_diffusion_march64(double* u, Geometry g, StepScalars* sc) {
    using S = M64Shape<NI, NJ, NK>;
    constexpr int NIP = S::NIP, PL = S::PL, W = S::W, NCELL = S::NCELL, P = S::P;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
    double* tile = reinterpret_cast<double*>(smem + S::off_tile);
    double* SI = reinterpret_cast<double*>(smem + S::off_si);
    double* SJ = reinterpret_cast<double*>(smem + S::off_sj);
    double* FI = reinterpret_cast<double*>(smem + S::off_fi);
    double* FJ = reinterpret_cast<double*>(smem + S::off_fj);
    double* gi = reinterpret_cast<double*>(smem + S::off_gi);
    double* gj = reinterpret_cast<double*>(smem + S::off_gj);
    double* gs = reinterpret_cast<double*>(smem + S::off_gs);
    const int b = blockIdx.x, tid = threadIdx.x;
    double* blk = u + (size_t)b * NV * NCELL;
    if (tid == 0) {
        for (int q = 0; q < W; ++q) mbar_init(&bars[q], 1);
        fence_mbar_init();
    }
    __syncthreads();
    int issued = 0;   // thread 0: planes [0, issued) have been requested
    if (tid == 0) {
        for (int p = 0; p < W; ++p) issue_planes<double, S>(blk, tile, p, p + 1, &bars[p]);
        issued = W;
    }
    load_geometry<double, S>(g, b, gi, gj, gs, nullptr);
    __syncthreads();
    const int c = tid % S::NCOL, v = tid / S::NCOL;
    const int i = c % NI, j = c / NI, ii = i + 2, jj = j + 2;
    const double* GCS = gi + GI_CS * NIP;
    const double cs = GCS[ii];
    const double rc = gi[GI_R * NIP + ii];
    const double den[3] = {gs[GS_DXI], gs[GS_DXJ] * rc, gs[GS_DXK] * rc * gj[GJ_SIN * S::NJP + jj]};
    const double hdt = 0.5 * sc->dt;
    const int polls = sc->wait_polls;
    int late = 0;
    auto abort_cta = [&]() {
        if (tid != 0) return;
        atomicOr(&sc->nan_flag, 2);
        for (int p = issued - W < 0 ? 0 : issued - W; p < issued; ++p)
            mbar_wait(&bars[p % W], (uint32_t)((p / W) & 1), kWaitPolls);
        for (int q = 0; q < W; ++q) mbar_inval(&bars[q]);
    };
    double* SIv = SI + v * S::NSI;
    double* SJv = SJ + v * S::NSJ;
    double* FIv = FI + v * S::NFI;
    double* FJv = FJ + v * S::NFJ;
    const double* col = tile + (size_t)v * W * PL + jj * NIP + ii;         // this column, this variable
    const double* colvp = tile + (size_t)V_VP * W * PL + jj * NIP + ii;    // this column's v_phi
    for (int p = 0; p < 4; ++p) late |= mbar_wait(&bars[p], 0u, polls) ? 0 : 1;
    double u0, u1, dk0, fk0;
    {
        const double a0 = col[0], a1 = col[PL], a2 = col[2 * PL], a3 = col[3 * PL];
        const double d1 = face_slope(a0, a1, a2), d2 = face_slope(a1, a2, a3);
        u0 = a2;
        u1 = a3;
        dk0 = d2;
        fk0 = face_flux_s(a1, a2, d1, d2, fabs(colvp[PL]) + cs, fabs(colvp[2 * PL]) + cs);
    }
    for (int kp = 2; kp < NK + 2; ++kp) {
        const int p2 = kp + 2;
        late |= mbar_wait(&bars[p2 % W], (uint32_t)((p2 / W) & 1), polls) ? 0 : 1;
        const int s0 = (kp % W) * PL, s1 = ((kp + 1) % W) * PL, s2 = (p2 % W) * PL;
        const double* tc = col + s0;   // this cell in plane kp
        // ---- phase A: k slope and face from the window; i and j slopes
        const double u2 = col[s2];
        const double dk1 = face_slope(u0, u1, u2);
        const double fk1 = face_flux_s(u0, u1, dk0, dk1, fabs(colvp[s0]) + cs, fabs(colvp[s1]) + cs);
        SIv[j * P + i + 1] = face_slope(tc[-1], u0, tc[1]);
        SJv[(j + 1) * P + i] = face_slope(tc[-NIP], u0, tc[NIP]);
        // ghost-cell slopes: i = -1, NI of every row, j = -1, NJ of every column
        constexpr int NEI = 2 * NJ * NV, NEJ = 2 * NI * NV;
        for (int x = tid; x < NEI + NEJ; x += S::NT) {
            if (x < NEI) {
                const int side = x & 1, r = (x >> 1) % NJ, w = (x >> 1) / NJ;
                const double* q = tile + (size_t)w * W * PL + s0 + (r + 2) * NIP + (side ? NI + 2 : 1);
                SI[w * S::NSI + r * P + (side ? NI + 1 : 0)] = face_slope(q[-1], q[0], q[1]);
            } else {
                const int y = x - NEI, side = y & 1, r = (y >> 1) % NI, w = (y >> 1) / NI;
                const double* q = tile + (size_t)w * W * PL + s0 + (side ? NJ + 2 : 1) * NIP + r + 2;
                SJ[w * S::NSJ + (side ? NJ + 1 : 0) * P + r] = face_slope(q[-NIP], q[0], q[NIP]);
            }
        }
        if (__syncthreads_or(late)) {
            abort_cta();
            return;
        }
        // ---- phase B: this cell's faces i - 1/2 and j - 1/2; the last faces
        // of the rows and columns
        const double* vr = tile + (size_t)V_VR * W * PL + s0 + jj * NIP + ii;
        const double* vt = tile + (size_t)V_VT * W * PL + s0 + jj * NIP + ii;
        const double fi0 = face_flux_s(tc[-1], u0, SIv[j * P + i], SIv[j * P + i + 1], fabs(vr[-1]) + GCS[ii - 1],
                                       fabs(vr[0]) + cs);
        const double fj0 =
            face_flux_s(tc[-NIP], u0, SJv[j * P + i], SJv[(j + 1) * P + i], fabs(vt[-NIP]) + cs, fabs(vt[0]) + cs);
        FIv[j * P + i] = fi0;
        FJv[j * P + i] = fj0;
        constexpr int NFE = NJ * NV + NI * NV;
        for (int x = tid; x < NFE; x += S::NT) {
            if (x < NJ * NV) {
                const int r = x % NJ, w = x / NJ;
                const double* a = tile + (size_t)w * W * PL + s0 + (r + 2) * NIP + NI + 1;   // last interior cell of row r
                const double* vrr = tile + (size_t)V_VR * W * PL + s0 + (r + 2) * NIP + NI + 1;
                FI[w * S::NFI + r * P + NI] =
                    face_flux_s(a[0], a[1], SI[w * S::NSI + r * P + NI], SI[w * S::NSI + r * P + NI + 1],
                                fabs(vrr[0]) + GCS[NI + 1], fabs(vrr[1]) + GCS[NI + 2]);
            } else {
                const int y = x - NJ * NV, r = y % NI, w = y / NI;
                const double* a = tile + (size_t)w * W * PL + s0 + (NJ + 1) * NIP + r + 2;   // last interior row, column r
                const double* vtt = tile + (size_t)V_VT * W * PL + s0 + (NJ + 1) * NIP + r + 2;
                const double c2 = GCS[r + 2];
                FJ[w * S::NFJ + NJ * P + r] =
                    face_flux_s(a[0], a[NIP], SJ[w * S::NSJ + NJ * P + r], SJ[w * S::NSJ + (NJ + 1) * P + r],
                                fabs(vtt[0]) + c2, fabs(vtt[NIP]) + c2);
            }
        }
        __syncthreads();
        if (tid == 0) {
            for (; issued < S::NKP && issued <= kp + W; ++issued)
                issue_planes<double, S>(blk, tile, issued, issued + 1, &bars[issued % W]);
        }
        // ---- phase C: the six faces in the reference's order, the update in place
        double R = 0.0;
        R = R + Pol<double>::dv(fi0 - FIv[j * P + i + 1], den[0], 0.0);
        R = R + Pol<double>::dv(fj0 - FJv[(j + 1) * P + i], den[1], 0.0);
        R = R + Pol<double>::dv(fk0 - fk1, den[2], 0.0);
        blk[(size_t)v * NCELL + (size_t)kp * PL + jj * NIP + ii] = u0 + hdt * R;
        u0 = u1;
        u1 = u2;
        dk0 = dk1;
        fk0 = fk1;
    }
    if (__syncthreads_or(late)) {
        abort_cta();
        return;
    }
    if (tid == 0)
        for (int q = 0; q < W; ++q) mbar_inval(&bars[q]);
}

// ---------------------------------------------------------------------------
// dt = min(1.e20, CFL*min(h/v_wave)) (3_6/ModTimeStep.f90:20-29); also the
// per-stage FP32 factors of the mixed path and the reset of the accumulator.
// One thread (k_finalize_dt, or the first phase of the persistent step).
__device__ __forceinline__ void finalize_dt_body(StepScalars* sc) {
    const double m = __longlong_as_double((long long)sc->min_ratio_bits);
    const double dt = fmin((double)1.e20f, sc->cfl * m);
    sc->dt = dt;
    for (int s = 1; s <= 4; ++s) sc->dt_stage_f[s - 1] = (float)(dt / (double)(5.0f - (float)s));
    sc->dt_half_f = (float)(0.5 * dt);
    sc->min_ratio_bits = 0x7FF0000000000000ull;   // +inf for the next step
    if (sc->nan_flag && sc->nan_step < 0) sc->nan_step = sc->step_counter;
    sc->step_counter += 1;
}

// ---------------------------------------------------------------------------
// Wave speed (3_6/ModWaveSpeed.f90:8-27), h/v_wave min-reduction
// (3_6/ModTimeStep.f90:10-30) and the NaN scan of 3_6/ModCheck.f90:12-71.
template <class T>
__global__ void __launch_bounds__(256) k_cfl(const T* u, Geometry g, StepScalars* sc, StepDims d) {
    // R: the type the ratio and its block minimum are formed in (FP64 on the
    // exact path, FP32 on the mixed path); the cross-block minimum is FP64.
    using R = T;
    const int nint = d.ni * d.nj * d.nk;
    const int b = blockIdx.y;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    R ratio = R(INFINITY);
    int nan = 0;
    if (q < nint) {
        const int i = q % d.ni + 2, j = (q / d.ni) % d.nj + 2, k = q / (d.ni * d.nj) + 2;
        const T* blk = u + (size_t)b * NV * d.ncell + ((size_t)k * d.njp + j) * d.nip + i;
        T x[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            x[v] = blk[(size_t)v * d.ncell];
            nan |= (x[v] != x[v]);
        }
        const T* Gi = gi_ptr<T>(g) + (size_t)b * GI_COUNT * d.nip;
        const T* Gj = gj_ptr<T>(g) + (size_t)b * GJ_COUNT * d.njp;
        const T* Gs = gs_ptr<T>(g) + (size_t)b * GS_COUNT;
        // h_LLL = min(dxi, r*dxj, r*sin(theta)*dxk) (3_6/ModBlock.f90:416-425)
        const T r = Gi[GI_R * d.nip + i];
        if constexpr (Pol<T>::exact) {
            const T h = fmin(fmin(Gs[GS_DXI], r * Gs[GS_DXJ]), r * Gj[GJ_SIN * d.njp + j] * Gs[GS_DXK]);
            T w = Gi[GI_CS * d.nip + i] + sqrt(x[V_VR] * x[V_VR] + x[V_VT] * x[V_VT] + x[V_VP] * x[V_VP]);
            w = w + sqrt(x[V_BR] * x[V_BR] + x[V_BT] * x[V_BT] + x[V_BP] * x[V_BP]) / sqrt(Gi[GI_RHO0 * d.nip + i]);
            ratio = h / w;                 // the reference's h_LLL/v_wave
        } else {
            ratio = cfl_ratio_f(cfl_sq3(x[V_VR], x[V_VT], x[V_VP]), cfl_sq3(x[V_BR], x[V_BT], x[V_BP]),
                                Gi[GI_CS * d.nip + i], Gi[GI_RHO0 * d.nip + i], r, Gj[GJ_SIN * d.njp + j],
                                Gs[GS_DXI], Gs[GS_DXJ], Gs[GS_DXK]);
        }
        if (ratio != ratio) { nan = 1; ratio = R(INFINITY); }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ratio = fmin(ratio, __shfl_xor_sync(0xffffffffu, ratio, o));
        nan |= __shfl_xor_sync(0xffffffffu, nan, o);
    }
    __shared__ R wmin[8];
    __shared__ int wnan[8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { wmin[wid] = ratio; wnan[wid] = nan; }
    __syncthreads();
    if (threadIdx.x == 0) {
        R m = wmin[0];
        int n = wnan[0];
        for (int w2 = 1; w2 < (int)(blockDim.x >> 5); ++w2) { m = fmin(m, wmin[w2]); n |= wnan[w2]; }
        // positive doubles order like their bit patterns
        atomicMin(&sc->min_ratio_bits, (unsigned long long)__double_as_longlong((double)m));
        if (n) atomicOr(&sc->nan_flag, 1);
    }
}

// ---------------------------------------------------------------------------
// Ghost fill: the single-GPU form of ModCommunication_SendRecvGC_new
// (3_6/ModCommunication.f90:655-795). Exact copies first, then trilinear
// entries (3_6/ModMath.f90:283-291) with the Yin-Yang vector rotation
// (3_6/ModYinYang.f90:58-60).
// Source values are read with ld (CG false) or, in the persistent step,
// with ld.global.cg (L2 only): there another SM wrote them in the phase
// before, after this SM may have cached the same lines in its L1.
template <bool CG, class T>
__device__ __forceinline__ T ldsrc(const T* p) {
    if constexpr (CG) return __ldcg(p);
    else return *p;
}
template <class T, bool CG = false>
__device__ __forceinline__ void ghost_copy_one(T* u, const GhostCopyList& L, int ncell, int64_t e) {
    const size_t d = (size_t)L.dst[e], s = (size_t)L.src[e];
    T v[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = ldsrc<CG>(u + s + (size_t)q * ncell);
#pragma unroll
    for (int q = 0; q < NV; ++q) u[d + (size_t)q * ncell] = v[q];
}

// one-dimensional linear interpolation (radial neighbours of different
// spacing: the other two weights snapped to exactly 0), mixed path only
template <class T, bool CG = false>
__device__ __forceinline__ void ghost_lin_one(T* u, const GhostLinList& L, int ncell, int64_t e) {
    const size_t d = (size_t)L.dst[e], s = (size_t)L.src[e], st = (size_t)L.stride[e];
    const T w = (T)L.w[e], uw = T(1) - w;
    T v[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        const T* f = u + s + (size_t)q * ncell;
        v[q] = blend(ldsrc<CG>(f), ldsrc<CG>(f + st), uw, w);
    }
#pragma unroll
    for (int q = 0; q < NV; ++q) u[d + (size_t)q * ncell] = v[q];
}

// The values of one interpolated/rotated ghost entry (into val); the FP64
// path is the reference's trilinear form and operand order.
template <class T, bool CG = false>
__device__ __forceinline__ void ghost_interp_vals(const T* u, const GhostInterpList& L, int ncell, int nip, int pl,
                                                  int64_t e, T* val);

template <class T, bool CG = false>
__device__ __forceinline__ void ghost_interp_one(T* u, const GhostInterpList& L, int ncell, int nip, int pl, int64_t e) {
    T val[NV];
    ghost_interp_vals<T, CG>(u, L, ncell, nip, pl, e, val);
    const size_t dd = (size_t)L.dst[e];
#pragma unroll
    for (int v = 0; v < NV; ++v) u[dd + (size_t)v * ncell] = val[v];
}

template <class T, bool CG>
__device__ __forceinline__ void ghost_interp_vals(const T* u, const GhostInterpList& L, int ncell, int nip, int pl,
                                                  int64_t e, T* val) {
    const int kind = L.kind[e];
    const size_t s = (size_t)L.src[e];
    if constexpr (!Pol<T>::exact) {
        // FP32 weights; the Yin-Yang seam is aligned in r (wi == 0 after
        // snapping), so most entries are bilinear in (j, k): 4 source points
        const float wi = L.wf[3 * e], wj = L.wf[3 * e + 1], wk = L.wf[3 * e + 2];
        const float ui = 1.f - wi, uj = 1.f - wj, uk = 1.f - wk;
        if (!(kind & 1)) {
#pragma unroll
            for (int v = 0; v < NV; ++v) val[v] = ldsrc<CG>(u + s + (size_t)v * ncell);
        } else if (wi == 0.f) {
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                const T* f = u + s + (size_t)v * ncell;
                val[v] = ldsrc<CG>(f + (0)) * uj * uk + ldsrc<CG>(f + (nip)) * wj * uk + ldsrc<CG>(f + (pl)) * uj * wk + ldsrc<CG>(f + (nip + pl)) * wj * wk;
            }
        } else {
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                const T* f = u + s + (size_t)v * ncell;
                val[v] = ldsrc<CG>(f + (0)) * ui * uj * uk + ldsrc<CG>(f + (1)) * wi * uj * uk + ldsrc<CG>(f + (nip)) * ui * wj * uk + ldsrc<CG>(f + (pl)) * ui * uj * wk +
                         ldsrc<CG>(f + (1 + nip)) * wi * wj * uk + ldsrc<CG>(f + (nip + pl)) * ui * wj * wk + ldsrc<CG>(f + (1 + pl)) * wi * uj * wk +
                         ldsrc<CG>(f + (1 + nip + pl)) * wi * wj * wk;
            }
        }
        if (kind & 2) {
            const float a = L.rotf[2 * e], c = L.rotf[2 * e + 1];
            T x2 = val[V_BT], x3 = val[V_BP];
            val[V_BT] = -(a * x2) - c * x3;
            val[V_BP] = -(a * x3) + c * x2;
            x2 = val[V_VT]; x3 = val[V_VP];
            val[V_VT] = -(a * x2) - c * x3;
            val[V_VP] = -(a * x3) + c * x2;
        }
        return;
    }
    if (kind & 1) {
        const T wi = (T)L.w[3 * e], wj = (T)L.w[3 * e + 1], wk = (T)L.w[3 * e + 2];
        const T ui = T(1) - wi, uj = T(1) - wj, uk = T(1) - wk;
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            const T* f = u + s + (size_t)v * ncell;
            val[v] = ldsrc<CG>(f + (0)) * ui * uj * uk + ldsrc<CG>(f + (1)) * wi * uj * uk + ldsrc<CG>(f + (nip)) * ui * wj * uk + ldsrc<CG>(f + (pl)) * ui * uj * wk +
                     ldsrc<CG>(f + (1 + nip)) * wi * wj * uk + ldsrc<CG>(f + (nip + pl)) * ui * wj * wk + ldsrc<CG>(f + (1 + pl)) * wi * uj * wk +
                     ldsrc<CG>(f + (1 + nip + pl)) * wi * wj * wk;
        }
    } else {
#pragma unroll
        for (int v = 0; v < NV; ++v) val[v] = ldsrc<CG>(u + s + (size_t)v * ncell);
    }
    if (kind & 2) {
        const T a = (T)L.rot[2 * e], c = (T)L.rot[2 * e + 1];
        T x2 = val[V_BT], x3 = val[V_BP];
        val[V_BT] = -(a * x2) - c * x3;
        val[V_BP] = -(a * x3) + c * x2;
        x2 = val[V_VT]; x3 = val[V_VP];
        val[V_VT] = -(a * x2) - c * x3;
        val[V_VP] = -(a * x3) + c * x2;
    }
}

// ---------------------------------------------------------------------------
// A barrier over every CTA of a cooperative launch (all co-resident). Thread
// 0 of each CTA reads the generation, arrives on the counter; the last one
// resets the counter and advances the generation, the others poll it, at most
// `polls` times (a poll that runs out flags the step: bit 1 of nan_flag, the
// host returns FALCON_ERR_TIMEOUT, and the CTA goes on). Fences on both sides
// make every CTA's writes before the barrier visible to every CTA after it.
struct GridBarrier {
    unsigned int* count;   // 0 between barriers
    unsigned int* gen;
    unsigned int* ticket;  // [5]: the next block of each block phase (4 stages, diffusion), 0 at launch
};
__device__ __forceinline__ void grid_sync(const GridBarrier& gb, StepScalars* sc, int polls) {
    // the next phase reads this one's global writes also through bulk copies
    // (the async proxy): order them across the proxies on both sides
    asm volatile("fence.proxy.async.global;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int g0 = *(volatile unsigned int*)gb.gen;
        __threadfence();
        if (atomicAdd(gb.count, 1u) == gridDim.x - 1) {
            atomicExch(gb.count, 0u);
            __threadfence();
            atomicAdd(gb.gen, 1u);
        } else {
            int it = 0;
            while (*(volatile unsigned int*)gb.gen == g0) {
                if (++it > polls) {
                    atomicOr(&sc->nan_flag, 2);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    asm volatile("fence.proxy.async.global;" ::: "memory");
}

// The pointers of one mixed step: u^n in U, the stage buffer RK, the second
// state buffer R2 (u^{n+1} is written there, then the host swaps U and R2).
struct StepBuffers {
    float* U;
    float* RK;
    float* R2;
    int8_t* ulo;
};

// One mixed RK4 step of 16^3 blocks in one persistent launch: the CTAs take
// the blocks (and, in the exchanges, the ghost entries) in turn and meet at a
// grid barrier between the phases the graph runs as separate launches:
// dt, then per stage s the stage kernel's body into seq[s] (pushing the
// regular ghost faces) and the exchange of the rest (face lists), then the
// diffusion body into R2 (pushes, next step's CFL minimum) and the exchange
// of the remaining entries. The bodies are the separate kernels' own
// (KPAR 2 for the stages, two threads per column for the diffusion: 512
// threads each, and every variant computes the same bits), so the step
// equals the graph's bit for bit.
template <int N>
__global__ void __launch_bounds__(512, 2)
k_step_persistent(StepBuffers sb, PushTable push, Geometry g, StepScalars* sc, GhostLists gl_stage,
                  GhostLists gl_final, StepDims d, GridBarrier gb) {
    static_assert(N == 16, "16^3 blocks");
    const int polls = sc->wait_polls;
    if (blockIdx.x == 0 && threadIdx.x == 0) finalize_dt_body(sc);
    grid_sync(gb, sc, polls);
    const int64_t tstride = (int64_t)gridDim.x * blockDim.x;
    const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    auto exchange = [&](const GhostLists& G, float* u) {
        for (int64_t e = t0; e < G.ip.n; e += tstride)
            ghost_interp_one<float, true>(u, G.ip, d.ncell, d.nip, d.nip * d.njp, e);
        for (int64_t e = t0; e < G.ln.n; e += tstride) ghost_lin_one<float, true>(u, G.ln, d.ncell, e);
        for (int64_t e = t0; e < G.cp.n; e += tstride) ghost_copy_one<float, true>(u, G.cp, d.ncell, e);
    };
    // between two bodies in one CTA: the generic writes of the one before
    // are ordered before the bulk copies of the next into the same memory
    auto next_body = [&]() {
        fence_proxy_async();
        __syncthreads();
    };
    // blocks are handed out one at a time from a ticket counter per phase, as
    // the hardware scheduler hands CTAs to SMs: a CTA that finishes early
    // takes the next block instead of waiting at the barrier
    __shared__ int next_b;
    auto take = [&](int phase) -> int {
        if (threadIdx.x == 0) next_b = (int)atomicAdd(&gb.ticket[phase], 1u);
        __syncthreads();
        return next_b;   // read before the next take's write: a body or next_body() barrier lies between
    };
    for (int s = 1; s <= 4; ++s) {
        float* in = s == 1 ? sb.U : (s == 3 ? sb.R2 : sb.RK);
        float* out = s == 4 ? sb.U : (s == 2 ? sb.R2 : sb.RK);   // U -> RK -> R2 -> RK -> U
        for (int b = take(s - 1); b < d.nblocks; b = take(s - 1)) {
            stage_body<float, 16, 16, 16, 2, 0>(b, in, sb.U, out, sb.ulo, push, DivBArgs{nullptr, nullptr, nullptr, 0},
                                                g, sc, s, 1, 1);
            next_body();
        }
        grid_sync(gb, sc, polls);
        exchange(gl_stage, out);
        grid_sync(gb, sc, polls);
    }
    for (int b = take(4); b < d.nblocks; b = take(4)) {
        march_body<16, 16, 16, 2>(b, sb.U, sb.R2, sb.ulo, push, g, sc, 1);
        next_body();
    }
    grid_sync(gb, sc, polls);
    exchange(gl_final, sb.R2);
}

// ---- block sharding: the entries that cross ranks ---------------------------
// The sender evaluates each outgoing ghost entry from its own blocks (the
// same values as the single-GPU ghost fill) into a pack buffer pack[e][NV];
// the receiver writes pack[e] into its ghost cells (dst[e], the entries in
// the same order), as the reference's per-peer send/receive buffers
// (3_6/ModCommunication.f90:725-765).
template <class T>
__global__ void __launch_bounds__(128) k_shard_pack(const T* u, GhostInterpList L, int ncell, int nip, int pl, T* pack) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= L.n) return;
    T val[NV];
    ghost_interp_vals(u, L, ncell, nip, pl, e, val);
#pragma unroll
    for (int v = 0; v < NV; ++v) pack[e * NV + v] = val[v];
}
template <class T>
__global__ void __launch_bounds__(128) k_shard_unpack(T* u, const int32_t* dst, int64_t n, int ncell, const T* pack) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const size_t d = (size_t)dst[e];
#pragma unroll
    for (int v = 0; v < NV; ++v) u[d + (size_t)v * ncell] = pack[e * NV + v];
}

template <class T>
__global__ void __launch_bounds__(256) k_ghost_copy(T* u, GhostCopyList L, int ncell) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < L.n) ghost_copy_one(u, L, ncell, e);
}
template <class T>
__global__ void __launch_bounds__(256) k_ghost_lin(T* u, GhostLinList L, int ncell) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < L.n) ghost_lin_one(u, L, ncell, e);
}
template <class T>
__global__ void __launch_bounds__(128) k_ghost_interp(T* u, GhostInterpList L, int ncell, int nip, int pl) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < L.n) ghost_interp_one(u, L, ncell, nip, pl, e);
}
// The three lists of one exchange in one launch: every entry reads interior
// cells and writes a ghost cell that no other entry writes, so the lists are
// independent. The interpolated entries (the longest) take the first CTAs.
template <class T>
__global__ void __launch_bounds__(128) k_ghost_all(T* u, GhostLists G, int ncell, int nip, int pl, int nb_ip, int nb_ln) {
    const int bx = blockIdx.x;
    if (bx < nb_ip) {
        const int64_t e = (int64_t)bx * 128 + threadIdx.x;
        if (e < G.ip.n) ghost_interp_one(u, G.ip, ncell, nip, pl, e);
    } else if (bx < nb_ip + nb_ln) {
        const int64_t e = (int64_t)(bx - nb_ip) * 128 + threadIdx.x;
        if (e < G.ln.n) ghost_lin_one(u, G.ln, ncell, e);
    } else {
        const int64_t e = (int64_t)(bx - nb_ip - nb_ln) * 128 + threadIdx.x;
        if (e < G.cp.n) ghost_copy_one(u, G.cp, ncell, e);
    }
}

// ---------------------------------------------------------------------------
// GLM psi: artificial diffusion (3_6/ModDiffusion.f90:9-150 applies to every
// variable, psi included) into psi_out = psi + dt/2 R_psi, the same formulas
// as k_diffusion with psi read from global memory; wave speeds from u.
template <class T>
__global__ void __launch_bounds__(256) k_psi_diffusion(const T* u, const T* psi, T* psi_out, Geometry g,
                                                       StepScalars* sc, StepDims d) {
    const int nint = d.ni * d.nj * d.nk;
    const int b = blockIdx.y;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nint) return;
    const int ii = q % d.ni + 2, jj = (q / d.ni) % d.nj + 2, kp = q / (d.ni * d.nj) + 2;
    const size_t pl = (size_t)d.nip * d.njp;
    const size_t c0 = (size_t)b * d.ncell + (size_t)kp * pl + (size_t)jj * d.nip + ii;
    const T* Gi = gi_ptr<T>(g) + (size_t)b * GI_COUNT * d.nip;
    const T* Gj = gj_ptr<T>(g) + (size_t)b * GJ_COUNT * d.njp;
    const T* Gs = gs_ptr<T>(g) + (size_t)b * GS_COUNT;
    const T* GCS = Gi + GI_CS * d.nip;
    const T rc = Gi[GI_R * d.nip + ii];
    const T den[3] = {Gs[GS_DXI], Gs[GS_DXJ] * rc, Gs[GS_DXK] * rc * Gj[GJ_SIN * d.njp + jj]};
    const size_t strides[3] = {1, (size_t)d.nip, pl};
    T R = T(0);
#pragma unroll
    for (int dir = 0; dir < 3; ++dir) {
        const size_t s = strides[dir];
        const T* vd = u + (size_t)b * NV * d.ncell + (size_t)(V_VR + dir) * d.ncell + (c0 - (size_t)b * d.ncell);
        auto at = [&](int m) -> T { return psi[(ptrdiff_t)c0 + (ptrdiff_t)m * (ptrdiff_t)s]; };
        const T csm = dir == 0 ? GCS[ii - 1] : GCS[ii];
        const T cs0 = GCS[ii];
        const T csp = dir == 0 ? GCS[ii + 1] : GCS[ii];
        const T cm = fabs(vd[-(ptrdiff_t)s]) + csm, cz = fabs(vd[0]) + cs0, cp = fabs(vd[s]) + csp;
        const T fm2 = at(-2), fm1 = at(-1), f0 = at(0), fp1 = at(1), fp2 = at(2);
        const T dm1 = minmod(fm2, fm1, f0);
        const T d0 = minmod(fm1, f0, fp1);
        const T dp1 = minmod(f0, fp1, fp2);
        T num = ((f0 - d0 * T(0.5)) - fm1) - dm1 * T(0.5);
        T phi = fmax(T(0), T(1) + T(2) * (Pol<T>::ratio(num, f0 - fm1) - T(1)));
        T fL = -(T(0.5) * phi * num);
        fL = fL * (cz + cm) * T(0.5);
        num = ((fp1 - dp1 * T(0.5)) - f0) - d0 * T(0.5);
        phi = fmax(T(0), T(1) + T(2) * (Pol<T>::ratio(num, fp1 - f0) - T(1)));
        T fR = -(T(0.5) * phi * num);
        fR = fR * (cp + cz) * T(0.5);
        R = R + (fL - fR) / den[dir];
    }
    const T p0 = psi[c0];
    T o;
    if constexpr (Pol<T>::exact) o = (T)((double)p0 + (0.5 * sc->dt) * (double)R);
    else o = fmaf(sc->dt_half_f, (float)R, (float)p0);
    psi_out[c0] = o;
}

// GLM psi ghost fill with the state's ghost lists (psi is a scalar: no
// rotation). List offsets address var 0 of the [b][NV][cell] state; psi's
// array is [b][cell].
__device__ __forceinline__ size_t psi_off(size_t off, int ncell) {
    const size_t b = off / ((size_t)NV * ncell);
    return off - b * (size_t)(NV - 1) * ncell;
}
template <class T>
__global__ void __launch_bounds__(256) k_psi_ghost(T* psi, GhostLists L, int ncell, int nip, int pl) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t ncp = L.cp.n, nln = L.ln.n, nip_ = L.ip.n;
    if (e < ncp) {
        psi[psi_off(L.cp.dst[e], ncell)] = psi[psi_off(L.cp.src[e], ncell)];
    } else if (e < ncp + nln) {
        const int64_t q = e - ncp;
        const T* f = psi + psi_off(L.ln.src[q], ncell);
        const T w = (T)L.ln.w[q];
        psi[psi_off(L.ln.dst[q], ncell)] = blend(f[0], f[L.ln.stride[q]], T(1) - w, w);
    } else if (e < ncp + nln + nip_) {
        const int64_t q = e - ncp - nln;
        const T* f = psi + psi_off(L.ip.src[q], ncell);
        T val;
        if (!(L.ip.kind[q] & 1)) {
            val = f[0];
        } else {
            T wi, wj, wk;
            if constexpr (Pol<T>::exact) { wi = L.ip.w[3 * q]; wj = L.ip.w[3 * q + 1]; wk = L.ip.w[3 * q + 2]; }
            else { wi = L.ip.wf[3 * q]; wj = L.ip.wf[3 * q + 1]; wk = L.ip.wf[3 * q + 2]; }
            const T ui = T(1) - wi, uj = T(1) - wj, uk = T(1) - wk;
            val = f[0] * ui * uj * uk + f[1] * wi * uj * uk + f[nip] * ui * wj * uk + f[pl] * ui * uj * wk +
                  f[1 + nip] * wi * wj * uk + f[nip + pl] * ui * wj * wk + f[1 + pl] * wi * uj * wk +
                  f[1 + nip + pl] * wi * wj * wk;
        }
        psi[psi_off(L.ip.dst[q], ncell)] = val;
    }
}

}  // namespace impl
}  // namespace falcon
