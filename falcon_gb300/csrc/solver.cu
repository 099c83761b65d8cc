// solver.cu -- GPU multigrid-preconditioned flexible CG on the Yin-Yang grid.
//
// Reference algorithm: ModLinearSolver_Multigrid_CG / _V_cycle / _JCB_CG
// (3_5/ModLinearSolver.f90:86-427) with the 7-point face-coefficient operator
// (:15-84) and the 1-layer face-ghost halo (3_5/ModCommunication.f90:1497-1639).
// GB300 form:
//   - FP64 iterative refinement outside: the true residual r = b - A x, its
//     norms and the update x += d are FP64, and convergence is judged only on
//     the FP64 ||b - A x|| / ||b||;
//   - inside, flexible CG in float-float (FP32 pairs, about 48 bits; GB300's
//     FP64 pipe is too slow for the per-cell work of every iteration) on the
//     correction equation scaled by per-problem powers of two, per-problem
//     dot products reduced into FP64; y = A x of falcon_solver_apply and the
//     coarse training solve stay FP64;
//   - V-cycle preconditioner in FP32: red-black Gauss-Seidel smoothing,
//     restriction R = P^T (sum of 8 children), injection prolongation,
//     Galerkin coarse operators;
//   - every problem of a batch is advanced by the same launches: kernels index
//     block -> problem, scalars are per problem, converged problems freeze.
// Kernels are launched with one CTA per block (grid.x = block) looping over the
// block's cells, so a CTA never mixes problems and its reductions go to one
// per-problem slot with one atomic.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <map>
#include <vector>

#include "../../include/falcon_gb300.h"
#include "lcc.h"
#include "solver.h"

namespace falcon {
namespace sv {

struct LevelDims {
    int m0, m1, m2;        // interior
    int p0, p1, p2;        // padded (m+2)
    int nint, npad;
    int chunk;             // cells per CTA (a multiple of m0; the solver's tuned tile)
    int tpb;               // threads per CTA (<= 1024, a multiple of 32)
};

struct HaloList {
    int64_t n;
    const int32_t* dst;    // padded global offset
    const int32_t* src;    // padded global offset of the base source cell
    const uint8_t* code;   // bit d set: the weight of direction d is not 0
    const double* w;       // [n][3] (FP64 fills)
    const float* wf;       // [n][3] (FP32 fills: the V-cycle)
    int32_t sj, sk;        // padded strides of j and k
};

struct Ops64 { const double *Aii, *Ai, *Aj, *Ak; };
struct Ops32 { const float *Aii, *Ai, *Aj, *Ak; };

// Launch geometry of the cell kernels: CTAs take chunks of d.chunk cells,
// block-major (consecutive CTAs stream consecutive memory); a chunk never
// spans two blocks, so a CTA's reductions go to one problem. The chunk and
// the CTA size are the solver's tile shape, picked by its autotuner.
__device__ __forceinline__ int cell_chunks(const LevelDims& d) { return (d.nint + d.chunk - 1) / d.chunk; }
__device__ __forceinline__ int cell_block(const LevelDims& d) { return (int)(blockIdx.x / (unsigned)cell_chunks(d)); }
__device__ __forceinline__ int cell_first(const LevelDims& d) {
    return (int)(blockIdx.x % (unsigned)cell_chunks(d)) * d.chunk;
}
__device__ __forceinline__ int cell_end(const LevelDims& d) { return min(cell_first(d) + d.chunk, d.nint); }

__device__ __forceinline__ void cell_ijk(const LevelDims& d, int c, int& i, int& j, int& k) {
    i = c % d.m0 + 1;
    j = (c / d.m0) % d.m1 + 1;
    k = c / (d.m0 * d.m1) + 1;
}
__device__ __forceinline__ size_t pidx(const LevelDims& d, int b, int i, int j, int k) {
    return (size_t)b * d.npad + ((size_t)k * d.p1 + j) * d.p0 + i;
}

// y = A x over the interior, reference operand order (3_5/ModLinearSolver.f90:43-50)
template <class T, class O>
__device__ __forceinline__ T apply_A(const O& A, const LevelDims& d, const T* x, int b, int c, int i, int j, int k) {
    const size_t P = pidx(d, b, i, j, k);
    const size_t sj = d.p0, sk = (size_t)d.p0 * d.p1;
    const size_t fi = ((size_t)b * d.m2 * d.m1 + (size_t)(k - 1) * d.m1 + (j - 1)) * (d.m0 + 1) + (i - 1);
    const size_t fj = ((size_t)b * d.m2 * (d.m1 + 1) + (size_t)(k - 1) * (d.m1 + 1) + (j - 1)) * d.m0 + (i - 1);
    const size_t fk = ((size_t)b * (d.m2 + 1) * d.m1 + (size_t)(k - 1) * d.m1 + (j - 1)) * d.m0 + (i - 1);
    return A.Aii[(size_t)b * d.nint + c] * x[P] + A.Ai[fi] * x[P - 1] + A.Ai[fi + 1] * x[P + 1] + A.Aj[fj] * x[P - sj] +
           A.Aj[fj + d.m0] * x[P + sj] + A.Ak[fk] * x[P - sk] + A.Ak[fk + (size_t)d.m0 * d.m1] * x[P + sk];
}

template <class T>
__device__ __forceinline__ void block_sum_atomic(T v, double* slot) {
    double s = (double)v;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ double ws[32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ws[w];
        atomicAdd(slot, t);
    }
    __syncthreads();
}

// ---- halo fill (trilinear from the source interior) ------------------------
// entries whose three weights are exactly zero are plain copies of the base
// cell (a separate index list, no weights)
// one launch for both lists: entries [0, nc) are the copies, the rest the
// interpolated entries of H
template <class T>
__global__ void k_halo(T* v, HaloList H, const int32_t* cdst, const int32_t* csrc, int64_t nc) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < nc) {
        v[cdst[e]] = v[csrc[e]];
        return;
    }
    e -= nc;
    if (e >= H.n) return;
    const size_t s = (size_t)H.src[e];
    const int cd = H.code[e];
    const int a = (cd & 1) ? 1 : 0, bq = (cd & 2) ? H.sj : 0, c = (cd & 4) ? H.sk : 0;
    T wi, wj, wk;
    if constexpr (sizeof(T) == 4) {
        wi = H.wf[3 * e]; wj = H.wf[3 * e + 1]; wk = H.wf[3 * e + 2];
    } else {
        wi = H.w[3 * e]; wj = H.w[3 * e + 1]; wk = H.w[3 * e + 2];
    }
    const T ui = T(1) - wi, uj = T(1) - wj, uk = T(1) - wk;
    const T* f = v + s;
    v[H.dst[e]] = f[0] * ui * uj * uk + f[a] * wi * uj * uk + f[bq] * ui * wj * uk + f[c] * ui * uj * wk +
                  f[a + bq] * wi * wj * uk + f[bq + c] * ui * wj * wk + f[a + c] * wi * uj * wk + f[a + bq + c] * wi * wj * wk;
}

// ---- FP64 outer iteration ----------------------------------------------------
struct Dots {
    double *pAp, *pr, *zAp, *rr, *bb, *ab;   // ab: sum of (|b| + sum_j |A_ij x_j|)^2
    const int32_t* active;
    const int32_t* bprob;
};

// Ap = A p; pAp += p.Ap; pr += p.r (per problem)
__global__ void k_spmv_dots(Ops64 A, LevelDims d, const double* p, double* Ap, const double* r, Dots D) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    double pa = 0, pr = 0;
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        const double y = apply_A<double>(A, d, p, b, c, i, j, k);
        const size_t q = (size_t)b * d.nint + c;
        Ap[q] = y;
        const double pv = p[pidx(d, b, i, j, k)];
        pa += pv * y;
        pr += pv * r[q];
    }
    const int pb = D.bprob[b];
    block_sum_atomic(pa, &D.pAp[pb]);
    block_sum_atomic(pr, &D.pr[pb]);
}

// alpha = p.r / p.Ap; x += alpha p; r -= alpha Ap; rr += r.r; rf = (float)r
__global__ void k_update_xr(LevelDims d, double* x, const double* p, double* r, const double* Ap, float* rf, Dots D) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    const int pb = D.bprob[b];
    // a problem whose direction vanished (p.Ap == 0) takes no step instead of 0/0
    const double alpha = (D.active[pb] && D.pAp[pb] != 0.0) ? D.pr[pb] / D.pAp[pb] : 0.0;
    double rr = 0;
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        const size_t P = pidx(d, b, i, j, k), q = (size_t)b * d.nint + c;
        x[P] = x[P] + alpha * p[P];
        const double rv = r[q] - alpha * Ap[q];
        r[q] = rv;
        rf[q] = (float)rv;
        rr += rv * rv;
    }
    block_sum_atomic(rr, &D.rr[pb]);
}

// sum_j |A_ij x_j| of one row: the scale of the rounding error of b - A x
__device__ __forceinline__ double abs_row(const Ops64& A, const LevelDims& d, const double* x, int b, int c, int i,
                                          int j, int k) {
    const size_t P = pidx(d, b, i, j, k);
    const size_t sj = d.p0, sk = (size_t)d.p0 * d.p1;
    const size_t fi = ((size_t)b * d.m2 * d.m1 + (size_t)(k - 1) * d.m1 + (j - 1)) * (d.m0 + 1) + (i - 1);
    const size_t fj = ((size_t)b * d.m2 * (d.m1 + 1) + (size_t)(k - 1) * (d.m1 + 1) + (j - 1)) * d.m0 + (i - 1);
    const size_t fk = ((size_t)b * (d.m2 + 1) * d.m1 + (size_t)(k - 1) * d.m1 + (j - 1)) * d.m0 + (i - 1);
    return fabs(A.Aii[(size_t)b * d.nint + c] * x[P]) + fabs(A.Ai[fi] * x[P - 1]) + fabs(A.Ai[fi + 1] * x[P + 1]) +
           fabs(A.Aj[fj] * x[P - sj]) + fabs(A.Aj[fj + d.m0] * x[P + sj]) + fabs(A.Ak[fk] * x[P - sk]) +
           fabs(A.Ak[fk + (size_t)d.m0 * d.m1] * x[P + sk]);
}

// r = b - A x (FP64 true residual); rr += r.r; ab += (|b| + sum|A x|)^2; rf = (float)r
__global__ void k_residual64(Ops64 A, LevelDims d, const double* x, const double* bvec, double* r, float* rf, Dots D,
                             int want_bb) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    double rr = 0, bb = 0, ab = 0;
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        const size_t q = (size_t)b * d.nint + c;
        const double rv = bvec[q] - apply_A<double>(A, d, x, b, c, i, j, k);
        r[q] = rv;
        rf[q] = (float)rv;
        rr += rv * rv;
        bb += bvec[q] * bvec[q];
        const double s = fabs(bvec[q]) + abs_row(A, d, x, b, c, i, j, k);
        ab += s * s;
    }
    const int pb = D.bprob[b];
    block_sum_atomic(rr, &D.rr[pb]);
    block_sum_atomic(ab, &D.ab[pb]);
    if (want_bb) block_sum_atomic(bb, &D.bb[pb]);
}

// z (FP64, interior) from the preconditioner (FP32 padded z or the residual);
// zAp += z.Ap
__global__ void k_take_z(LevelDims d, const float* zf, const double* r, int use_r, double* z, const double* Ap, Dots D,
                         int want_zAp) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    double za = 0;
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        const size_t q = (size_t)b * d.nint + c;
        const double zv = use_r ? r[q] : (double)zf[pidx(d, b, i, j, k)];
        z[q] = zv;
        if (want_zAp) za += zv * Ap[q];
    }
    if (want_zAp) block_sum_atomic(za, &D.zAp[D.bprob[b]]);
}

// p = z + beta p, beta = -z.Ap / p.Ap (flexible CG, one-term A-orthogonalisation);
// restart (beta = 0) when `restart`
__global__ void k_update_p(LevelDims d, double* p, const double* z, Dots D, int restart) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        const int pb = D.bprob[b];
        if (!D.active[pb]) continue;
        const double beta = (restart || D.pAp[pb] == 0.0) ? 0.0 : -D.zAp[pb] / D.pAp[pb];
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        const size_t P = pidx(d, b, i, j, k);
        p[P] = z[(size_t)b * d.nint + c] + beta * p[P];
    }
}

// ---- float-float inner iteration -------------------------------------------------
// GB300 runs FP64 at a small fraction of its FP32 rate, and FP64 kernels run
// every iteration are bound by the FP64 pipe. The inner solve of each
// refinement pass therefore runs the flexible CG in float-float: every value
// an FP32 pair (hi, lo), hi + lo with |lo| <= ulp(hi)/2, about 48 significant
// bits, formed with error-free FP32 transformations (this file is compiled
// without FMA contraction; the FMAs below are explicit). FP32's exponent range
// is too narrow for the raw system (b.b reaches 1e54 for conduction), so the
// inner solve works on A' = A / sA, r' = r / sr, d' = d sA / sr per problem
// with sA, sr powers of two (exact): every vector and dot product is O(1).
struct Ops2 { const float2 *Aii, *Ai, *Aj, *Ak; };

__device__ __forceinline__ float2 ff_quick(float s, float e) {
    const float h = s + e;
    return make_float2(h, e - (h - s));
}
__device__ __forceinline__ float2 ff_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return make_float2(s, (a - (s - bb)) + (b - bb));
}
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
    float2 s = ff_two_sum(a.x, b.x);
    const float2 t = ff_two_sum(a.y, b.y);
    s.y += t.x;
    s = ff_quick(s.x, s.y);
    s.y += t.y;
    return ff_quick(s.x, s.y);
}
__device__ __forceinline__ float2 ff_mul(float2 a, float2 b) {
    const float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    return ff_quick(p, e);
}
__device__ __forceinline__ float2 ff_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 ff_from(double v) {   // a few FP64 operations: per thread, not per cell
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
}
__device__ __forceinline__ double ff_to(float2 a) { return (double)a.x + (double)a.y; }

// per-problem FF sums -> one FP64 atomic per CTA (FP64 work once per warp)
__device__ __forceinline__ void block_sum_atomic_ff(float2 v, double* slot) {
    for (int o = 16; o > 0; o >>= 1)
        v = ff_add(v, make_float2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o)));
    __shared__ double ws[32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = ff_to(v);
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ws[w];
        atomicAdd(slot, t);
    }
    __syncthreads();
}

// y = A' x over the interior, the reference's operand order
__device__ __forceinline__ float2 apply_A_ff(const Ops2& A, const LevelDims& d, const float2* x, int b, int c, int i,
                                             int j, int k, float* absrow) {
    const size_t P = pidx(d, b, i, j, k);
    const size_t sj = d.p0, sk = (size_t)d.p0 * d.p1;
    const size_t fi = ((size_t)b * d.m2 * d.m1 + (size_t)(k - 1) * d.m1 + (j - 1)) * (d.m0 + 1) + (i - 1);
    const size_t fj = ((size_t)b * d.m2 * (d.m1 + 1) + (size_t)(k - 1) * (d.m1 + 1) + (j - 1)) * d.m0 + (i - 1);
    const size_t fk = ((size_t)b * (d.m2 + 1) * d.m1 + (size_t)(k - 1) * d.m1 + (j - 1)) * d.m0 + (i - 1);
    const float2 c7[7] = {A.Aii[(size_t)b * d.nint + c], A.Ai[fi], A.Ai[fi + 1], A.Aj[fj], A.Aj[fj + d.m0], A.Ak[fk],
                          A.Ak[fk + (size_t)d.m0 * d.m1]};
    const float2 x7[7] = {x[P], x[P - 1], x[P + 1], x[P - sj], x[P + sj], x[P - sk], x[P + sk]};
    float2 y = ff_mul(c7[0], x7[0]);
    float ar = fabsf(c7[0].x * x7[0].x);
#pragma unroll
    for (int t = 1; t < 7; ++t) {
        y = ff_add(y, ff_mul(c7[t], x7[t]));
        ar += fabsf(c7[t].x * x7[t].x);
    }
    if (absrow) *absrow = ar;
    return y;
}

// Ap = A' p; pAp += p.Ap; pr += p.r
__global__ void k_spmv_dots_ff(Ops2 A, LevelDims d, const float2* p, float2* Ap, const float2* r, Dots D) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    float2 pa = make_float2(0.f, 0.f), pr = make_float2(0.f, 0.f);
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        const float2 y = apply_A_ff(A, d, p, b, c, i, j, k, nullptr);
        const size_t q = (size_t)b * d.nint + c;
        Ap[q] = y;
        const float2 pv = p[pidx(d, b, i, j, k)];
        pa = ff_add(pa, ff_mul(pv, y));
        pr = ff_add(pr, ff_mul(pv, r[q]));
    }
    const int pb = D.bprob[b];
    block_sum_atomic_ff(pa, &D.pAp[pb]);
    block_sum_atomic_ff(pr, &D.pr[pb]);
}

// alpha = p.r / p.Ap; x += alpha p; r -= alpha Ap; rr += r.r; rf = hi(r) (the V-cycle's input)
__global__ void k_update_xr_ff(LevelDims d, float2* x, const float2* p, float2* r, const float2* Ap, float* rf, Dots D) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    const int pb = D.bprob[b];
    const double alpha = (D.active[pb] && D.pAp[pb] != 0.0) ? D.pr[pb] / D.pAp[pb] : 0.0;
    const float2 al = ff_from(alpha), nal = ff_neg(al);
    float2 rr = make_float2(0.f, 0.f);
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        const size_t P = pidx(d, b, i, j, k), q = (size_t)b * d.nint + c;
        x[P] = ff_add(x[P], ff_mul(al, p[P]));
        const float2 rv = ff_add(r[q], ff_mul(nal, Ap[q]));
        r[q] = rv;
        rf[q] = rv.x;
        rr = ff_add(rr, ff_mul(rv, rv));
    }
    block_sum_atomic_ff(rr, &D.rr[pb]);
}

// z = the preconditioner's FP32 output scaled by sA (it inverts the unscaled
// FP32 operator), or r; zAp += z.Ap
__global__ void k_take_z_ff(LevelDims d, const float* zf, const float* sA, const float2* r, int use_r, float2* z,
                            const float2* Ap, Dots D, int want_zAp) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    const float s = sA[D.bprob[b]];
    float2 za = make_float2(0.f, 0.f);
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        const size_t q = (size_t)b * d.nint + c;
        const float2 zv = use_r ? r[q] : make_float2(zf[pidx(d, b, i, j, k)] * s, 0.f);
        z[q] = zv;
        if (want_zAp) za = ff_add(za, ff_mul(zv, Ap[q]));
    }
    if (want_zAp) block_sum_atomic_ff(za, &D.zAp[D.bprob[b]]);
}

// p = z + beta p, beta = -z.Ap / p.Ap; restart (beta = 0) when `restart`
__global__ void k_update_p_ff(LevelDims d, float2* p, const float2* z, Dots D, int restart) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    const int pb = D.bprob[b];
    if (!D.active[pb]) return;
    const double beta = (restart || D.pAp[pb] == 0.0) ? 0.0 : -D.zAp[pb] / D.pAp[pb];
    const float2 be = ff_from(beta);
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        const size_t P = pidx(d, b, i, j, k);
        p[P] = ff_add(z[(size_t)b * d.nint + c], ff_mul(be, p[P]));
    }
}

// halo of an FF vector: the trilinear sum with the 8 corner weights
// precomputed in FP64 on the host and stored as FF pairs
struct HaloListFF {
    int64_t n;
    const int32_t* dst;
    const int32_t* src;
    const uint8_t* code;   // as HaloList
    const float2* w8;      // [n][8] corner weights
    int32_t sj, sk;
};
__global__ void k_halo_ff(float2* v, HaloListFF H, const int32_t* cdst, const int32_t* csrc, int64_t nc) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < nc) {
        v[cdst[e]] = v[csrc[e]];
        return;
    }
    e -= nc;
    if (e >= H.n) return;
    const int cd = H.code[e];
    const int a = (cd & 1) ? 1 : 0, bq = (cd & 2) ? H.sj : 0, c = (cd & 4) ? H.sk : 0;
    const int off[8] = {0, a, bq, c, a + bq, bq + c, a + c, a + bq + c};
    const float2* f = v + H.src[e];
    const float2* w = H.w8 + 8 * e;
    float2 s = ff_mul(w[0], f[0]);
#pragma unroll
    for (int t = 1; t < 8; ++t) s = ff_add(s, ff_mul(w[t], f[off[t]]));
    v[H.dst[e]] = s;
}

// ---- the inner solve's loop control on the device -----------------------------
// One inner solve (an FCG on the correction equation) runs as one graph launch:
// a first iteration, then a WHILE node whose body is one more iteration; the
// last kernel of every iteration decides, on the device, whether the loop goes
// on. The loop is bounded: it counts its iterations and stops at max_it.
struct InnerCtl {
    int32_t it;        // iterations done by this inner solve
    int32_t max_it;    // its iteration limit (<= kInnerCap)
    int32_t stalled;   // the largest relative residual fell by < 5% over 8 iterations
    int32_t nan;       // a non-finite residual
    int32_t cont;      // the loop condition written by the last check
    int32_t pad_;
    double hist[16];   // ring of the largest relative residual per iteration
};
constexpr int32_t kInnerCap = 100000;

// After an iteration's x/r update: each problem's relative recursive residual
// h = sqrt(r.r / r0.r0); a problem at or below its eta leaves the iteration
// (active = 0: no further update). One CTA of 256 threads, problem per thread
// (nproblems <= 256). With `set_cond`, sets the WHILE node's condition.
__global__ void __launch_bounds__(256) k_inner_check(int np, const double* rr, const double* rr0, const double* eta,
                                                     int32_t* active, InnerCtl* ctl, cudaGraphConditionalHandle h,
                                                     int set_cond) {
    __shared__ double smax[256];
    __shared__ int sany[256], snan[256];
    const int q = threadIdx.x;
    double hq = 0.0;
    int still = 0, bad = 0;
    if (q < np && active[q]) {
        hq = sqrt(rr[q] / rr0[q]);
        if (!(hq == hq) || hq > 1e300) {
            bad = 1;
        } else if (hq <= eta[q]) {
            active[q] = 0;
        } else {
            still = 1;
        }
    }
    smax[q] = hq;
    sany[q] = still;
    snan[q] = bad;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (q < o) {
            smax[q] = fmax(smax[q], smax[q + o]);
            sany[q] |= sany[q + o];
            snan[q] |= snan[q + o];
        }
        __syncthreads();
    }
    if (q == 0) {
        const int it = ctl->it + 1;
        ctl->it = it;
        if (snan[0]) ctl->nan = 1;
        int stalled = ctl->stalled;
        if (sany[0]) {
            ctl->hist[it & 15] = smax[0];
            if (it > 10 && smax[0] > 0.95 * ctl->hist[(it - 8) & 15]) stalled = 1;
        }
        ctl->stalled = stalled;
        const int cap = ctl->max_it < kInnerCap ? ctl->max_it : kInnerCap;
        const int cont = (sany[0] && !stalled && !snan[0] && it < cap) ? 1 : 0;
        ctl->cont = cont;
        if (set_cond) cudaGraphSetConditional(h, (unsigned)cont);
    }
}

// ---- FP64 iterative refinement around the float-float solve ------------------
// r' = r / sr per problem as FF pairs (sr a power of two at or above ||r||_2:
// exact, and |r'| <= 1), its FP32 part for the V-cycle, and rr += r'.r'
__global__ void k_ir_start(LevelDims d, const double* r, const double* inv_sr, float2* r2, float* rf, Dots D) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    const int pb = D.bprob[b];
    const double s = inv_sr[pb];
    float2 rr = make_float2(0.f, 0.f);
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        const size_t q = (size_t)b * d.nint + c;
        const double v = r[q] * s;
        const float h = (float)v;
        const float2 x = make_float2(h, (float)(v - (double)h));
        r2[q] = x;
        rf[q] = h;
        rr = ff_add(rr, ff_mul(x, x));
    }
    block_sum_atomic_ff(rr, &D.rr[pb]);
}

// x += d' * fac per problem (FP64): d' the float-float correction of the
// scaled system, fac = sr / sA (a power of two, so the scaling is exact)
__global__ void k_ir_accum(LevelDims d, const float2* x2, const double* fac, const int32_t* bprob, double* x) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    const double f = fac[bprob[b]];
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        const size_t P = pidx(d, b, i, j, k);
        x[P] = x[P] + ff_to(x2[P]) * f;
    }
}

// ---- FP32 V-cycle ------------------------------------------------------------
__global__ void k_zero_f(float* v, size_t n) {
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (size_t)gridDim.x * blockDim.x) v[x] = 0.f;
}

// red-black Gauss-Seidel half sweep: z = (r - sum_nb A z_nb) / Aii on cells of one colour
// (The smoother's rounding is free -- the outer CG is flexible -- so it uses
// explicit FMAs and a fast division; this file is otherwise compiled without
// contraction.) With an even row length that divides the chunk a thread takes
// only cells of the colour: m0/2 cells of each colour per row.
__device__ __forceinline__ void rbgs_cell(const Ops32& A, const LevelDims& d, const float* r, float* z, int b, int c,
                                          int i, int j, int k) {
    const size_t P = pidx(d, b, i, j, k);
    const size_t sj = d.p0, sk = (size_t)d.p0 * d.p1;
    const size_t fi = ((size_t)b * d.m2 * d.m1 + (size_t)(k - 1) * d.m1 + (j - 1)) * (d.m0 + 1) + (i - 1);
    const size_t fj = ((size_t)b * d.m2 * (d.m1 + 1) + (size_t)(k - 1) * (d.m1 + 1) + (j - 1)) * d.m0 + (i - 1);
    const size_t fk = ((size_t)b * (d.m2 + 1) * d.m1 + (size_t)(k - 1) * d.m1 + (j - 1)) * d.m0 + (i - 1);
    float off = A.Ai[fi] * z[P - 1];
    off = fmaf(A.Ai[fi + 1], z[P + 1], off);
    off = fmaf(A.Aj[fj], z[P - sj], off);
    off = fmaf(A.Aj[fj + d.m0], z[P + sj], off);
    off = fmaf(A.Ak[fk], z[P - sk], off);
    off = fmaf(A.Ak[fk + (size_t)d.m0 * d.m1], z[P + sk], off);
    z[P] = __fdividef(r[(size_t)b * d.nint + c] - off, A.Aii[(size_t)b * d.nint + c]);
}

__global__ void k_rbgs(Ops32 A, LevelDims d, const float* r, float* z, int colour) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    if ((d.m0 & 1) == 0 && d.chunk % d.m0 == 0) {   // rows whole within a chunk
        const int half = d.m0 >> 1;
        for (int h = (c0 >> 1) + threadIdx.x; h < (c1 >> 1); h += blockDim.x) {
            const int row = h / half, ih = h - row * half;
            const int j = row % d.m1 + 1, k = row / d.m1 + 1;
            const int i = (((colour - j - k) & 1) ? 1 : 2) + 2 * ih;
            rbgs_cell(A, d, r, z, b, row * d.m0 + (i - 1), i, j, k);
        }
        return;
    }
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        if (((i + j + k) & 1) != colour) continue;
        const size_t P = pidx(d, b, i, j, k);
        const size_t sj = d.p0, sk = (size_t)d.p0 * d.p1;
        const size_t fi = ((size_t)b * d.m2 * d.m1 + (size_t)(k - 1) * d.m1 + (j - 1)) * (d.m0 + 1) + (i - 1);
        const size_t fj = ((size_t)b * d.m2 * (d.m1 + 1) + (size_t)(k - 1) * (d.m1 + 1) + (j - 1)) * d.m0 + (i - 1);
        const size_t fk = ((size_t)b * (d.m2 + 1) * d.m1 + (size_t)(k - 1) * d.m1 + (j - 1)) * d.m0 + (i - 1);
        const float off = A.Ai[fi] * z[P - 1] + A.Ai[fi + 1] * z[P + 1] + A.Aj[fj] * z[P - sj] + A.Aj[fj + d.m0] * z[P + sj] +
                          A.Ak[fk] * z[P - sk] + A.Ak[fk + (size_t)d.m0 * d.m1] * z[P + sk];
        z[P] = (r[(size_t)b * d.nint + c] - off) / A.Aii[(size_t)b * d.nint + c];
    }
}

// res = r - A z
__global__ void k_resid32(Ops32 A, LevelDims d, const float* r, const float* z, float* res) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        const size_t q = (size_t)b * d.nint + c;
        res[q] = r[q] - apply_A<float>(A, d, z, b, c, i, j, k);
    }
}

// r_coarse(I) = sum of the 8 children of res_fine (R = P^T)
__global__ void k_restrict(LevelDims f, LevelDims cd, const float* res, float* rc) {
    const int b = cell_block(cd), c0 = cell_first(cd), c1 = cell_end(cd);
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        const int I = c % cd.m0, J = (c / cd.m0) % cd.m1, K = c / (cd.m0 * cd.m1);
        const float* R = res + (size_t)b * f.nint;
        float s = 0.f;
    #pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int i = 2 * I + (q & 1), j = 2 * J + ((q >> 1) & 1), k = 2 * K + (q >> 2);
            s += R[((size_t)k * f.m1 + j) * f.m0 + i];
        }
        rc[(size_t)b * cd.nint + c] = s;
    }
}

// z_fine(child) += z_coarse(I) (injection)
__global__ void k_prolong_add(LevelDims f, LevelDims cd, const float* zc, float* zf) {
    const int b = cell_block(f), c0 = cell_first(f), c1 = cell_end(f);
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(f, c, i, j, k);
        const int I = (i - 1) / 2 + 1, J = (j - 1) / 2 + 1, K = (k - 1) / 2 + 1;
        zf[pidx(f, b, i, j, k)] += zc[pidx(cd, b, I, J, K)];
    }
}

// ---- learned coarse correction: coarsest level <-> dense panel grids ---------
// gmap[b][c]: panel-grid voxel of coarse cell c of block b

// static input channels 1..7: the six face couplings / diag, (diag + sum)/diag
__global__ void k_lcc_static(Ops64 A, LevelDims d, const int32_t* gmap, float* feat) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        const size_t fi = ((size_t)b * d.m2 * d.m1 + (size_t)(k - 1) * d.m1 + (j - 1)) * (d.m0 + 1) + (i - 1);
        const size_t fj = ((size_t)b * d.m2 * (d.m1 + 1) + (size_t)(k - 1) * (d.m1 + 1) + (j - 1)) * d.m0 + (i - 1);
        const size_t fk = ((size_t)b * (d.m2 + 1) * d.m1 + (size_t)(k - 1) * d.m1 + (j - 1)) * d.m0 + (i - 1);
        const double dg = A.Aii[(size_t)b * d.nint + c];
        const double cpl[6] = {A.Ai[fi], A.Ai[fi + 1], A.Aj[fj], A.Aj[fj + d.m0], A.Ak[fk], A.Ak[fk + (size_t)d.m0 * d.m1]};
        float* f = feat + (size_t)gmap[(size_t)b * d.nint + c] * 8;
        double sum = dg;
        for (int q = 0; q < 6; ++q) { f[1 + q] = (float)(cpl[q] / dg); sum += cpl[q]; }
        f[7] = (float)(sum / dg);
    }
}

// sum over coarse cells of (r/diag)^2
__global__ void k_lcc_sumsq(LevelDims d, const float* r, const float* Aii, double* sum) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    double v = 0.0;
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        const size_t q = (size_t)b * d.nint + c;
        const double x = (double)r[q] / (double)Aii[q];
        v += x * x;
    }
    block_sum_atomic(v, sum);
}

__device__ __forceinline__ double lcc_scale(const double* sum, int64_t n) {
    const double s = sqrt(*sum / (double)n);
    return s > 0.0 ? s : 1.0;
}

// input channel 0: (r/diag)/s, s = RMS of r/diag
__global__ void k_lcc_feat(LevelDims d, const float* r, const float* Aii, const int32_t* gmap, const double* sum,
                           int64_t n, float* feat) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        const size_t q = (size_t)b * d.nint + c;
        feat[(size_t)gmap[q] * 8] = (float)((double)r[q] / (double)Aii[q] / lcc_scale(sum, n));
    }
}

// coarse correction z = s * y (padded coarse layout)
__global__ void k_lcc_scatter(LevelDims d, const float* y, const int32_t* gmap, const double* sum, int64_t n, float* z) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        z[pidx(d, b, i, j, k)] = (float)(lcc_scale(sum, n) * (double)y[gmap[(size_t)b * d.nint + c]]);
    }
}

// training target: t = e/s (e: padded FP64 coarse solution)
__global__ void k_lcc_target(LevelDims d, const double* e, const int32_t* gmap, const double* sum, int64_t n, float* t) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        t[gmap[(size_t)b * d.nint + c]] = (float)(e[pidx(d, b, i, j, k)] / lcc_scale(sum, n));
    }
}

// ---- Jacobi-preconditioned CG on one level (FP64): exact coarse errors -------
// dots: [0] r.z  [1] p.Ap  [2] r.r (current); nd: the same for the next iterate
__global__ void k_ccg_init(Ops64 A, LevelDims d, const float* rc, double* r, double* z, double* p, double* dots) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    double rz = 0, rr = 0;
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        const size_t q = (size_t)b * d.nint + c;
        const double rv = (double)rc[q], zv = rv / A.Aii[q];
        r[q] = rv;
        z[q] = zv;
        p[pidx(d, b, i, j, k)] = zv;
        rz += rv * zv;
        rr += rv * rv;
    }
    block_sum_atomic(rz, &dots[0]);
    block_sum_atomic(rr, &dots[2]);
}

__global__ void k_ccg_spmv(Ops64 A, LevelDims d, const double* p, double* Ap, double* dots) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    double pa = 0;
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        const double y = apply_A<double>(A, d, p, b, c, i, j, k);
        Ap[(size_t)b * d.nint + c] = y;
        pa += p[pidx(d, b, i, j, k)] * y;
    }
    block_sum_atomic(pa, &dots[1]);
}

__global__ void k_ccg_update(Ops64 A, LevelDims d, double* x, const double* p, double* r, const double* Ap, double* z,
                             const double* dots, double* nd) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    const double alpha = dots[0] / dots[1];
    double rz = 0, rr = 0;
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        const size_t P = pidx(d, b, i, j, k), q = (size_t)b * d.nint + c;
        x[P] += alpha * p[P];
        const double rv = r[q] - alpha * Ap[q], zv = rv / A.Aii[q];
        r[q] = rv;
        z[q] = zv;
        rz += rv * zv;
        rr += rv * rv;
    }
    block_sum_atomic(rz, &nd[0]);
    block_sum_atomic(rr, &nd[2]);
}

__global__ void k_ccg_p(LevelDims d, double* p, const double* z, const double* dots, const double* nd) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        const size_t P = pidx(d, b, i, j, k);
        p[P] = z[(size_t)b * d.nint + c] + (nd[0] / dots[0]) * p[P];
    }
}

}  // namespace sv
}  // namespace falcon

using namespace falcon;
using namespace falcon::sv;

struct SvLevel {
    LevelDims d{};
    double *Aii = nullptr, *Ai = nullptr, *Aj = nullptr, *Ak = nullptr;
    float *fAii = nullptr, *fAi = nullptr, *fAj = nullptr, *fAk = nullptr;
    int32_t *hdst = nullptr, *hsrc = nullptr;
    uint8_t* hcode = nullptr;
    float* hwf = nullptr;
    double* hw = nullptr;
    int64_t nh = 0;
    int32_t *hcdst = nullptr, *hcsrc = nullptr;   // halo entries that are plain copies
    int64_t nhc = 0;
    // the copies in three runs: ghost and source both of parity 0 (nhc0), of
    // differing parities (nhcm), both of parity 1 (the rest); parity of i+j+k
    int64_t nhc0 = 0, nhcm = 0;
    float *z = nullptr, *r = nullptr, *res = nullptr;
    // level 0: the scaled operator A / sA and the halo's corner weights as FF pairs
    float2 *Aii2 = nullptr, *Ai2 = nullptr, *Aj2 = nullptr, *Ak2 = nullptr, *hw8 = nullptr;
    HaloList halo() const { return HaloList{nh, hdst, hsrc, hcode, hw, hwf, d.p0, d.p0 * d.p1}; }
    HaloListFF halo_ff() const { return HaloListFF{nh, hdst, hsrc, hcode, hw8, d.p0, d.p0 * d.p1}; }
    Ops2 ops2() const { return Ops2{Aii2, Ai2, Aj2, Ak2}; }
    Ops64 ops64() const { return Ops64{Aii, Ai, Aj, Ak}; }
    Ops32 ops32() const { return Ops32{fAii, fAi, fAj, fAk}; }
};

struct falcon_solver {
    SolverProblemSet S;
    std::string err;
    int device = 0;
    cudaStream_t st = nullptr;
    std::vector<SvLevel> lv;
    double *x = nullptr, *p = nullptr, *r = nullptr, *Ap = nullptr, *z = nullptr, *bvec = nullptr;
    // the float-float inner solve (scaled system, see Ops2): padded x2, p2; interior r2, Ap2, z2
    float2 *x2 = nullptr, *p2 = nullptr, *r2 = nullptr, *Ap2 = nullptr, *z2 = nullptr;
    std::vector<double> sA;               // per-problem powers of two (the operator's scale)
    float* dsA = nullptr;                 // sA on the device (FP32: powers of two are exact)
    double* dots = nullptr;       // [6][nproblems]: pAp, pr, zAp, rr, bb, ab
    double* ir_par = nullptr;     // [2][nproblems]: 1/sr and sr/sA of the refinement pass
    int32_t *active = nullptr, *bprob = nullptr;
    std::vector<void*> allocs;
    int nu_pre = 2, nu_post = 2, nu_coarse = 16;
    double dt_conduction = 0;
    uint64_t seed = 0;                    // the spec's seed (problem q: seed + q)
    double r_surface = 0;                 // PFSS: lower boundary radius (cm) of the synthetic magnetogram
    // learned coarse correction
    falcon_lcc* net = nullptr;
    int net_sweeps = 2;
    bool use_net = false;                 // set per V-cycle by the solve
    bool cmap_ok = false;
    int cD = 0, cH = 0, cW = 0;           // dense panel grid of the coarsest level
    int32_t* gmap = nullptr;              // [b][nint_c] -> panel-grid voxel
    float *feat = nullptr, *yout = nullptr;
    double* csum = nullptr;
    double* cdots = nullptr;              // [6] scalars of the coarse CG
    // recording of coarsest-level residuals (falcon_solver_record)
    float* rec = nullptr;
    int rec_max = 0, rec_n = 0;
    // one instantiated CUDA graph per V-cycle shape (smoothing sweeps, network on/off)
    std::map<int64_t, cudaGraphExec_t> vgraphs;
    // one instantiated graph per inner-solve shape: a first iteration and a
    // device-controlled WHILE loop of iterations (the V-cycle inside it)
    std::map<int64_t, cudaGraphExec_t> igraphs;
    bool capturing = false;               // enqueueing into a graph: the V-cycle's kernels inline
    InnerCtl* ictl = nullptr;             // device loop control
    double *rr0 = nullptr, *eta = nullptr;   // device, per problem
    // tile shape of the cell kernels (cells per CTA, threads per CTA), tuned at the first solve
    int tile_chunk = 1024, tile_tpb = 256;
    bool tuned = false;
    double tuned_ms = 0;                  // time of one timed iteration with the chosen tile
    void clear_graphs() {
        for (auto& kv : vgraphs) cudaGraphExecDestroy(kv.second);
        vgraphs.clear();
        for (auto& kv : igraphs) cudaGraphExecDestroy(kv.second);
        igraphs.clear();
    }
    int fail(int c, const std::string& m) { err = m; return c; }
    // zero-filled; the fill completes before returning: the uploads that follow
    // an allocation are plain cudaMemcpy calls, which nothing orders after
    // work on the solver's non-blocking stream
    template <class P> cudaError_t alloc(P** ptr, size_t bytes) {
        cudaError_t e = cudaMalloc((void**)ptr, bytes ? bytes : 16);
        if (e == cudaSuccess) {
            allocs.push_back(*ptr);
            e = cudaMemsetAsync(*ptr, 0, bytes ? bytes : 16, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        }
        return e;
    }
    Dots D() const {
        const int n = S.nproblems;
        return Dots{dots, dots + n, dots + 2 * n, dots + 3 * n, dots + 4 * n, dots + 5 * n, active, bprob};
    }
};

#define SCK(call, where)                                                                    \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) return sv->fail(FALCON_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e_)); \
    } while (0)

namespace {

// CTAs over (block, chunk of d.chunk cells), block-major: consecutive CTAs
// stream consecutive memory, and each per-problem reduction takes one atomic
// per chunk.
dim3 grid_cells(const LevelDims& d, int nblocks) {
    return dim3((unsigned)nblocks * (unsigned)((d.nint + d.chunk - 1) / d.chunk));
}
unsigned tpb(const LevelDims& d) { return (unsigned)std::min(d.tpb, (std::min(d.nint, d.chunk) + 31) / 32 * 32); }

template <class T> cudaError_t halo_fill(falcon_solver* sv, int l, T* v) {
    const SvLevel& L = sv->lv[l];
    const int64_t n = L.nhc + L.nh;
    if (n > 0) k_halo<T><<<(unsigned)((n + 255) / 256), 256, 0, sv->st>>>(v, L.halo(), L.hcdst, L.hcsrc, L.nhc);
    return cudaGetLastError();
}

// Before a red-black half sweep of `colour`: only the ghosts of the other
// parity are read. Copies whose ghost and source share a parity go stale only
// when that parity's cells change, so the fill refreshes the copies of the
// other parity, the copies whose parities differ and every interpolated
// entry; the copies of `colour`'s parity were refreshed after that colour's
// last sweep (the sweeps alternate).
template <class T> cudaError_t halo_fill_part(falcon_solver* sv, int l, T* v, int colour) {
    const SvLevel& L = sv->lv[l];
    const int p = 1 - colour;
    const int64_t off = p == 0 ? 0 : L.nhc0;
    const int64_t nc = p == 0 ? L.nhc0 + L.nhcm : L.nhc - L.nhc0;
    const int64_t n = nc + L.nh;
    if (n > 0) k_halo<T><<<(unsigned)((n + 255) / 256), 256, 0, sv->st>>>(v, L.halo(), L.hcdst + off, L.hcsrc + off, nc);
    return cudaGetLastError();
}

cudaError_t halo_fill_ff(falcon_solver* sv, float2* v) {
    const SvLevel& L = sv->lv[0];
    const int64_t n = L.nhc + L.nh;
    if (n > 0) k_halo_ff<<<(unsigned)((n + 255) / 256), 256, 0, sv->st>>>(v, L.halo_ff(), L.hcdst, L.hcsrc, L.nhc);
    return cudaGetLastError();
}

// power of two at or above max |v| over each problem's blocks (1 if all zero)
std::vector<double> problem_scale(const SolverProblemSet& S, const std::vector<double>& v, size_t per_block) {
    std::vector<double> m(S.nproblems, 0.0);
    for (int b = 0; b < S.nblocks; ++b) {
        double& q = m[S.block_problem[b]];
        for (size_t c = 0; c < per_block; ++c) q = std::max(q, std::fabs(v[(size_t)b * per_block + c]));
    }
    for (double& q : m) {
        if (!(q > 0) || !std::isfinite(q)) { q = 1.0; continue; }
        int e;
        std::frexp(q, &e);
        q = std::ldexp(1.0, e);
    }
    return m;
}
std::vector<float2> to_ff(const std::vector<double>& v, const std::vector<double>& scale_of_elem) {
    std::vector<float2> o(v.size());
    for (size_t q = 0; q < v.size(); ++q) {
        const double x = v[q] / scale_of_elem[q];
        const float h = (float)x;
        o[q] = make_float2(h, (float)(x - (double)h));
    }
    return o;
}

// z_0 = M r_0: one V-cycle on the FP32 residual stored in lv[0].r
cudaError_t vcycle_body(falcon_solver* sv) {
    const int nl = (int)sv->lv.size(), nb = sv->S.nblocks;
    cudaError_t e = cudaSuccess;
    // smooth(): `zero` when z (ghosts included) was just zeroed, so the first
    // sweep needs no fill; otherwise z changed everywhere and the first fill is
    // whole. Returns the colour of the last half sweep (-1 if none).
    auto smooth = [&](int l, int sweeps, bool reverse, bool zero) -> int {
        SvLevel& L = sv->lv[l];
        int last = -1;
        for (int s = 0; s < sweeps && e == cudaSuccess; ++s)
            for (int h = 0; h < 2 && e == cudaSuccess; ++h) {
                const int colour = reverse ? 1 - h : h;
                if (last >= 0) e = halo_fill_part<float>(sv, l, L.z, colour);
                else if (!zero) e = halo_fill<float>(sv, l, L.z);
                if (e != cudaSuccess) break;
                k_rbgs<<<grid_cells(L.d, nb), tpb(L.d), 0, sv->st>>>(L.ops32(), L.d, L.r, L.z, colour);
                e = cudaGetLastError();
                last = colour;
            }
        return last;
    };
    int last = -1;
    for (int l = 0; l < nl && e == cudaSuccess; ++l) {
        SvLevel& L = sv->lv[l];
        k_zero_f<<<1216, 256, 0, sv->st>>>(L.z, (size_t)nb * L.d.npad);
        e = cudaGetLastError();
        const bool coarsest = l == nl - 1 && nl > 1;
        if (coarsest && sv->rec && sv->rec_n < sv->rec_max && e == cudaSuccess)
            e = cudaMemcpyAsync(sv->rec + (size_t)sv->rec_n++ * nb * L.d.nint, L.r, (size_t)nb * L.d.nint * 4,
                                cudaMemcpyDeviceToDevice, sv->st);
        if (coarsest && sv->use_net && e == cudaSuccess) {
            // z_c = s * net(r_c / diag / s, operator) then a few sweeps
            const int64_t N = (int64_t)nb * L.d.nint;
            e = cudaMemsetAsync(sv->csum, 0, 8, sv->st);
            if (e == cudaSuccess) {
                k_lcc_sumsq<<<grid_cells(L.d, nb), tpb(L.d), 0, sv->st>>>(L.d, L.r, L.fAii, sv->csum);
                k_lcc_feat<<<grid_cells(L.d, nb), tpb(L.d), 0, sv->st>>>(L.d, L.r, L.fAii, sv->gmap, sv->csum, N, sv->feat);
                e = lcc::forward_device(sv->net, sv->feat, 2, sv->cD, sv->cH, sv->cW, sv->yout, sv->st);
            }
            if (e == cudaSuccess) {
                k_lcc_scatter<<<grid_cells(L.d, nb), tpb(L.d), 0, sv->st>>>(L.d, sv->yout, sv->gmap, sv->csum, N, L.z);
                e = cudaGetLastError();
            }
            last = smooth(l, sv->net_sweeps, false, false);
        } else {
            last = smooth(l, l == nl - 1 ? sv->nu_coarse : sv->nu_pre, false, true);
        }
        if (l + 1 < nl && e == cudaSuccess) {
            // the residual reads every ghost: refresh those of the last sweep's parity
            e = last >= 0 ? halo_fill_part<float>(sv, l, L.z, 1 - last) : halo_fill<float>(sv, l, L.z);
            if (e != cudaSuccess) break;
            k_resid32<<<grid_cells(L.d, nb), tpb(L.d), 0, sv->st>>>(L.ops32(), L.d, L.r, L.z, L.res);
            SvLevel& C = sv->lv[l + 1];
            k_restrict<<<grid_cells(C.d, nb), tpb(C.d), 0, sv->st>>>(L.d, C.d, L.res, C.r);
            e = cudaGetLastError();
        }
    }
    for (int l = nl - 2; l >= 0 && e == cudaSuccess; --l) {
        SvLevel& L = sv->lv[l];
        SvLevel& C = sv->lv[l + 1];
        k_prolong_add<<<grid_cells(L.d, nb), tpb(L.d), 0, sv->st>>>(L.d, C.d, C.z, L.z);
        e = cudaGetLastError();
        smooth(l, sv->nu_post, true, false);
    }
    return e;
}

// z_0 = M r_0 as one CUDA graph launch: the V-cycle's ~100 launches are
// captured once per shape and replayed (recording calls run eagerly: their
// destination changes from call to call)
cudaError_t vcycle(falcon_solver* sv) {
    if (sv->rec || sv->capturing) return vcycle_body(sv);
    const int64_t key = (int64_t)(sv->use_net ? 1 : 0) | ((int64_t)sv->nu_pre << 1) | ((int64_t)sv->nu_post << 8) |
                        ((int64_t)sv->nu_coarse << 15) | ((int64_t)sv->net_sweeps << 28);
    auto it = sv->vgraphs.find(key);
    if (it == sv->vgraphs.end()) {
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(sv->st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        const cudaError_t eb = vcycle_body(sv);
        e = cudaStreamEndCapture(sv->st, &g);
        if (eb != cudaSuccess) { if (g) cudaGraphDestroy(g); return eb; }
        if (e != cudaSuccess) return e;
        cudaGraphExec_t x = nullptr;
        e = cudaGraphInstantiate(&x, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return e;
        it = sv->vgraphs.emplace(key, x).first;
    }
    return cudaGraphLaunch(it->second, sv->st);
}

int setup(falcon_solver* sv) {
    SolverProblemSet& S = sv->S;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return sv->fail(FALCON_ERR_NO_DEVICE, "no CUDA device");
    SCK(cudaSetDevice(sv->device), "cudaSetDevice");
    SCK(cudaStreamCreateWithFlags(&sv->st, cudaStreamNonBlocking), "stream");
    const int nb = S.nblocks;
    sv->lv.resize(S.nlevels);
    for (int l = 0; l < S.nlevels; ++l) {
        const SolverLevel& H = S.L[l];
        SvLevel& L = sv->lv[l];
        L.d.m0 = H.m[0]; L.d.m1 = H.m[1]; L.d.m2 = H.m[2];
        L.d.p0 = H.m[0] + 2; L.d.p1 = H.m[1] + 2; L.d.p2 = H.m[2] + 2;
        L.d.nint = H.nint();
        L.d.npad = L.d.p0 * L.d.p1 * L.d.p2;
        L.d.chunk = sv->tile_chunk;
        L.d.tpb = sv->tile_tpb;
        auto up64 = [&](double** d, const std::vector<double>& h) -> cudaError_t {
            cudaError_t e = sv->alloc(d, h.size() * 8);
            if (e == cudaSuccess) e = cudaMemcpy(*d, h.data(), h.size() * 8, cudaMemcpyHostToDevice);
            return e;
        };
        auto up32 = [&](float** d, const std::vector<double>& h) -> cudaError_t {
            std::vector<float> f(h.begin(), h.end());
            cudaError_t e = sv->alloc(d, f.size() * 4);
            if (e == cudaSuccess) e = cudaMemcpy(*d, f.data(), f.size() * 4, cudaMemcpyHostToDevice);
            return e;
        };
        SCK(up64(&L.Aii, H.Aii), "operator");
        SCK(up64(&L.Ai, H.Ai), "operator");
        SCK(up64(&L.Aj, H.Aj), "operator");
        SCK(up64(&L.Ak, H.Ak), "operator");
        SCK(up32(&L.fAii, H.Aii), "operator");
        SCK(up32(&L.fAi, H.Ai), "operator");
        SCK(up32(&L.fAj, H.Aj), "operator");
        SCK(up32(&L.fAk, H.Ak), "operator");
        // halo entries -> padded offsets and strides
        // halo entries -> padded offsets; entries with all weights zero are
        // plain copies (a separate list: 8 bytes of index per entry)
        std::vector<int32_t> dst, src, stv, cdst, csrc;
        std::vector<double> w;
        const int32_t strides[3] = {1, L.d.p0, L.d.p0 * L.d.p1};
        for (const HaloEntry& h : H.halo) {
            const int32_t t = (int32_t)(h.tb * (int64_t)L.d.npad + ((int64_t)h.tk * L.d.p1 + h.tj) * L.d.p0 + h.ti);
            const int32_t f = (int32_t)(h.sb * (int64_t)L.d.npad + ((int64_t)h.k0 * L.d.p1 + h.j0) * L.d.p0 + h.i0);
            if (h.w[0] == 0.0 && h.w[1] == 0.0 && h.w[2] == 0.0) {
                cdst.push_back(t);
                csrc.push_back(f);
                continue;
            }
            dst.push_back(t);
            src.push_back(f);
            for (int dd = 0; dd < 3; ++dd) {
                w.push_back(h.w[dd]);
                stv.push_back(h.w[dd] != 0.0 ? strides[dd] : 0);
            }
        }
        {   // target order: a warp's stores write neighbouring ghost cells
            // (measured faster than source order, most for the PFSS batch)
            std::vector<size_t> ord(dst.size());
            for (size_t q = 0; q < ord.size(); ++q) ord[q] = q;
            std::stable_sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return dst[a] < dst[b]; });
            std::vector<int32_t> d2(ord.size()), s2(ord.size()), st2(3 * ord.size());
            std::vector<double> w2(3 * ord.size());
            for (size_t q = 0; q < ord.size(); ++q) {
                d2[q] = dst[ord[q]];
                s2[q] = src[ord[q]];
                for (int t = 0; t < 3; ++t) {
                    st2[3 * q + t] = stv[3 * ord[q] + t];
                    w2[3 * q + t] = w[3 * ord[q] + t];
                }
            }
            dst.swap(d2);
            src.swap(s2);
            stv.swap(st2);
            w.swap(w2);
            std::vector<size_t> oc(cdst.size());
            for (size_t q = 0; q < oc.size(); ++q) oc[q] = q;
            std::stable_sort(oc.begin(), oc.end(), [&](size_t a, size_t b) { return cdst[a] < cdst[b]; });
            // runs by parity (each run keeps the target order), see SvLevel
            auto par = [&](int32_t o) {
                const int64_t r = (int64_t)o % L.d.npad;
                return (int)((r % L.d.p0 + (r / L.d.p0) % L.d.p1 + r / ((int64_t)L.d.p0 * L.d.p1)) & 1);
            };
            auto run = [&](size_t q) {
                const int a = par(cdst[q]), b2 = par(csrc[q]);
                return a != b2 ? 1 : (a == 0 ? 0 : 2);
            };
            std::stable_sort(oc.begin(), oc.end(), [&](size_t a, size_t b) { return run(a) < run(b); });
            std::vector<int32_t> cd2(oc.size()), cs2(oc.size());
            int64_t n0 = 0, nm = 0;
            for (size_t q = 0; q < oc.size(); ++q) {
                cd2[q] = cdst[oc[q]];
                cs2[q] = csrc[oc[q]];
                const int rq = run(oc[q]);
                n0 += rq == 0;
                nm += rq == 1;
            }
            cdst.swap(cd2);
            csrc.swap(cs2);
            L.nhc0 = n0;
            L.nhcm = nm;
        }
        const size_t n = dst.size(), nc = cdst.size();
        L.nh = (int64_t)n;
        L.nhc = (int64_t)nc;
        SCK(sv->alloc(&L.hdst, n * 4), "halo");
        SCK(sv->alloc(&L.hsrc, n * 4), "halo");
        std::vector<uint8_t> code(n);
        std::vector<float> wf(3 * n);
        for (size_t q = 0; q < n; ++q) {
            code[q] = (uint8_t)((stv[3 * q] ? 1 : 0) | (stv[3 * q + 1] ? 2 : 0) | (stv[3 * q + 2] ? 4 : 0));
            for (int t = 0; t < 3; ++t) wf[3 * q + t] = (float)w[3 * q + t];
        }
        SCK(sv->alloc(&L.hcode, n), "halo");
        SCK(sv->alloc(&L.hwf, 3 * n * 4), "halo");
        SCK(sv->alloc(&L.hw, 3 * n * 8), "halo");
        SCK(sv->alloc(&L.hcdst, nc * 4), "halo");
        SCK(sv->alloc(&L.hcsrc, nc * 4), "halo");
        if (n) {
            SCK(cudaMemcpy(L.hdst, dst.data(), n * 4, cudaMemcpyHostToDevice), "halo");
            SCK(cudaMemcpy(L.hsrc, src.data(), n * 4, cudaMemcpyHostToDevice), "halo");
            SCK(cudaMemcpy(L.hcode, code.data(), n, cudaMemcpyHostToDevice), "halo");
            SCK(cudaMemcpy(L.hwf, wf.data(), 3 * n * 4, cudaMemcpyHostToDevice), "halo");
            SCK(cudaMemcpy(L.hw, w.data(), 3 * n * 8, cudaMemcpyHostToDevice), "halo");
        }
        if (nc) {
            SCK(cudaMemcpy(L.hcdst, cdst.data(), nc * 4, cudaMemcpyHostToDevice), "halo");
            SCK(cudaMemcpy(L.hcsrc, csrc.data(), nc * 4, cudaMemcpyHostToDevice), "halo");
        }
        if (l == 0) {   // the 8 corner weights of each interpolated halo entry, FF pairs
            std::vector<float2> w8(8 * n);
            for (size_t q = 0; q < n; ++q) {
                const double wi = w[3 * q], wj = w[3 * q + 1], wk = w[3 * q + 2];
                const double ui = 1.0 - wi, uj = 1.0 - wj, uk = 1.0 - wk;
                const double c8[8] = {ui * uj * uk, wi * uj * uk, ui * wj * uk, ui * uj * wk,
                                      wi * wj * uk, ui * wj * wk, wi * uj * wk, wi * wj * wk};
                for (int t = 0; t < 8; ++t) {
                    const float h = (float)c8[t];
                    w8[8 * q + t] = make_float2(h, (float)(c8[t] - (double)h));
                }
            }
            SCK(sv->alloc(&L.hw8, w8.size() * sizeof(float2)), "halo");
            if (n) SCK(cudaMemcpy(L.hw8, w8.data(), w8.size() * sizeof(float2), cudaMemcpyHostToDevice), "halo");
        }
        SCK(sv->alloc(&L.z, (size_t)nb * L.d.npad * 4), "vectors");
        SCK(sv->alloc(&L.r, (size_t)nb * L.d.nint * 4), "vectors");
        SCK(sv->alloc(&L.res, (size_t)nb * L.d.nint * 4), "vectors");
    }
    const LevelDims& d0 = sv->lv[0].d;
    SCK(sv->alloc(&sv->x, (size_t)nb * d0.npad * 8), "vectors");
    SCK(sv->alloc(&sv->p, (size_t)nb * d0.npad * 8), "vectors");
    SCK(sv->alloc(&sv->r, (size_t)nb * d0.nint * 8), "vectors");
    SCK(sv->alloc(&sv->Ap, (size_t)nb * d0.nint * 8), "vectors");
    SCK(sv->alloc(&sv->z, (size_t)nb * d0.nint * 8), "vectors");
    SCK(sv->alloc(&sv->bvec, (size_t)nb * d0.nint * 8), "vectors");
    SCK(sv->alloc(&sv->dots, (size_t)6 * S.nproblems * 8), "scalars");
    SCK(sv->alloc(&sv->ir_par, (size_t)2 * S.nproblems * 8), "scalars");
    SCK(sv->alloc(&sv->rr0, (size_t)S.nproblems * 8), "scalars");
    SCK(sv->alloc(&sv->eta, (size_t)S.nproblems * 8), "scalars");
    SCK(sv->alloc(&sv->ictl, sizeof(InnerCtl)), "scalars");
    SCK(sv->alloc(&sv->active, (size_t)S.nproblems * 4), "scalars");
    SCK(sv->alloc(&sv->bprob, (size_t)nb * 4), "scalars");
    SCK(cudaMemcpy(sv->bvec, S.b.data(), S.b.size() * 8, cudaMemcpyHostToDevice), "rhs");
    SCK(cudaMemcpy(sv->bprob, S.block_problem.data(), (size_t)nb * 4, cudaMemcpyHostToDevice), "scalars");
    // the float-float solve: A' = A / sA per problem (sA from the diagonal)
    {
        const SolverLevel& H = S.L[0];
        const size_t nint = (size_t)d0.nint;
        sv->sA = problem_scale(S, H.Aii, nint);
        auto upff = [&](float2** dptr, const std::vector<double>& h) -> cudaError_t {
            const size_t per = h.size() / (size_t)nb;   // entries per block
            std::vector<double> sc(h.size());
            for (int b = 0; b < nb; ++b)
                for (size_t c = 0; c < per; ++c) sc[(size_t)b * per + c] = sv->sA[S.block_problem[b]];
            const std::vector<float2> f = to_ff(h, sc);
            cudaError_t e = sv->alloc(dptr, f.size() * sizeof(float2));
            if (e == cudaSuccess) e = cudaMemcpy(*dptr, f.data(), f.size() * sizeof(float2), cudaMemcpyHostToDevice);
            return e;
        };
        SvLevel& L0 = sv->lv[0];
        SCK(upff(&L0.Aii2, H.Aii), "operator");
        SCK(upff(&L0.Ai2, H.Ai), "operator");
        SCK(upff(&L0.Aj2, H.Aj), "operator");
        SCK(upff(&L0.Ak2, H.Ak), "operator");
        for (float2** v : {&sv->x2, &sv->p2}) SCK(sv->alloc(v, (size_t)nb * d0.npad * sizeof(float2)), "vectors");
        for (float2** v : {&sv->r2, &sv->Ap2, &sv->z2})
            SCK(sv->alloc(v, (size_t)nb * d0.nint * sizeof(float2)), "vectors");
        std::vector<float> fa(sv->sA.begin(), sv->sA.end());
        SCK(sv->alloc(&sv->dsA, fa.size() * 4), "scalars");
        SCK(cudaMemcpy(sv->dsA, fa.data(), fa.size() * 4, cudaMemcpyHostToDevice), "scalars");
    }
    SCK(cudaStreamSynchronize(sv->st), "setup");
    return FALCON_OK;
}

// scatter an interior [b][nint] vector into the padded x
template <class T>
__global__ void k_scatter_pad(LevelDims d, const T* v, T* x) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        x[pidx(d, b, i, j, k)] = v[(size_t)b * d.nint + c];
    }
}
template <class T>
__global__ void k_gather_pad(LevelDims d, const T* x, T* v) {
    const int b = cell_block(d), c0 = cell_first(d), c1 = cell_end(d);
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        int i, j, k;
        cell_ijk(d, c, i, j, k);
        v[(size_t)b * d.nint + c] = x[pidx(d, b, i, j, k)];
    }
}

// Map the coarsest level onto one dense grid per panel (single problem,
// whole uniform blocks); builds gmap and the static input channels.
int ensure_coarse_map(falcon_solver* sv) {
    if (sv->cmap_ok) return FALCON_OK;
    const SolverProblemSet& S = sv->S;
    if (!sv->st) return sv->fail(FALCON_ERR_NO_DEVICE, "solver created without a device");
    if (S.nproblems != 1) return sv->fail(FALCON_ERR_INVALID_ARG, "learned coarse correction: single-problem solvers only");
    if (S.nlevels < 2) return sv->fail(FALCON_ERR_INVALID_ARG, "learned coarse correction: needs at least 2 levels");
    const int lc = S.nlevels - 1, nb = S.nblocks;
    const SolverLevel& C = S.L[lc];
    const Grid& g = S.grids[0];
    int tiles[2][3] = {{0, 0, 0}, {0, 0, 0}};
    std::vector<int32_t> bt((size_t)nb * 3), bpan(nb);
    for (int pnl = 0; pnl < 2; ++pnl) {
        int count = 0;
        for (int ax = 0; ax < 3; ++ax) {
            std::vector<double> starts;
            for (int b = 0; b < nb; ++b)
                if (((S.block_flags[b] & 1) != 0) == (pnl == 0)) starts.push_back(g.ranges[(size_t)b * 6 + ax * 2]);
            std::sort(starts.begin(), starts.end());
            std::vector<double> uniq;
            for (double v : starts)
                if (uniq.empty() || std::fabs(v - uniq.back()) > 1e-12 * std::max(1.0, std::fabs(v))) uniq.push_back(v);
            tiles[pnl][ax] = (int)uniq.size();
            for (int b = 0; b < nb; ++b) {
                if (((S.block_flags[b] & 1) != 0) != (pnl == 0)) continue;
                const double v = g.ranges[(size_t)b * 6 + ax * 2];
                int idx = 0;
                while (idx + 1 < (int)uniq.size() && v > uniq[idx] + 1e-12 * std::max(1.0, std::fabs(v))) ++idx;
                bt[(size_t)b * 3 + ax] = idx;
                bpan[b] = pnl;
            }
        }
        for (int b = 0; b < nb; ++b) count += ((S.block_flags[b] & 1) != 0) == (pnl == 0);
        if (count != tiles[pnl][0] * tiles[pnl][1] * tiles[pnl][2])
            return sv->fail(FALCON_ERR_INVALID_ARG, "learned coarse correction: blocks do not tile the panels uniformly");
    }
    for (int ax = 0; ax < 3; ++ax)
        if (tiles[0][ax] != tiles[1][ax]) return sv->fail(FALCON_ERR_INVALID_ARG, "learned coarse correction: panels differ");
    const int D = tiles[0][0] * C.m[0], H = tiles[0][1] * C.m[1], W = tiles[0][2] * C.m[2];
    if (D % 8 || H % 8 || W % 8)
        return sv->fail(FALCON_ERR_INVALID_ARG, "learned coarse correction: coarse panel grid " + std::to_string(D) + "x" +
                                                    std::to_string(H) + "x" + std::to_string(W) + " is not a multiple of 8");
    const int nint = C.nint();
    std::vector<int32_t> gm((size_t)nb * nint);
    for (int b = 0; b < nb; ++b)
        for (int c = 0; c < nint; ++c) {
            const int i = c % C.m[0], j = (c / C.m[0]) % C.m[1], k = c / (C.m[0] * C.m[1]);
            const int64_t vox = (int64_t)bpan[b] * D * H * W +
                                ((int64_t)(bt[(size_t)b * 3] * C.m[0] + i) * H + bt[(size_t)b * 3 + 1] * C.m[1] + j) * W +
                                bt[(size_t)b * 3 + 2] * C.m[2] + k;
            gm[(size_t)b * nint + c] = (int32_t)vox;
        }
    // every coarse cell lands on its own voxel of the two panel grids
    {
        std::vector<uint8_t> seen((size_t)2 * D * H * W, 0);
        for (int32_t v : gm) {
            if (v < 0 || (size_t)v >= seen.size() || seen[v])
                return sv->fail(FALCON_ERR_INVALID_ARG, "learned coarse correction: block tiling is not a bijection");
            seen[v] = 1;
        }
    }
    SCK(sv->alloc(&sv->gmap, gm.size() * 4), "coarse map");
    SCK(cudaMemcpy(sv->gmap, gm.data(), gm.size() * 4, cudaMemcpyHostToDevice), "coarse map");
    SCK(sv->alloc(&sv->feat, (size_t)2 * D * H * W * 8 * 4), "coarse features");
    SCK(sv->alloc(&sv->yout, (size_t)2 * D * H * W * 4), "coarse features");
    SCK(sv->alloc(&sv->csum, 8), "coarse features");
    SCK(sv->alloc(&sv->cdots, 6 * 8), "coarse features");
    SvLevel& L = sv->lv[lc];
    k_lcc_static<<<grid_cells(L.d, nb), tpb(L.d), 0, sv->st>>>(L.ops64(), L.d, sv->gmap, sv->feat);
    SCK(cudaGetLastError(), "coarse features");
    SCK(cudaStreamSynchronize(sv->st), "coarse features");
    sv->cD = D; sv->cH = H; sv->cW = W;
    sv->cmap_ok = true;
    return FALCON_OK;
}

// e = A_c^{-1} r_c on the coarsest level (r_c: FP32 [b][nint]) by Jacobi-PCG
// to ||r|| <= 1e-6 ||r_c|| (a training target needs no more: the network's
// own error is near 1e-2); the solution stays in sv->x (padded FP64)
int coarse_solve(falcon_solver* sv, const float* rc) {
    const int lc = sv->S.nlevels - 1, nb = sv->S.nblocks;
    SvLevel& L = sv->lv[lc];
    const dim3 g = grid_cells(L.d, nb);
    double* dots = sv->cdots;      // [0..2] current, [3..5] next
    SCK(cudaMemsetAsync(sv->x, 0, (size_t)nb * L.d.npad * 8, sv->st), "coarse cg");
    SCK(cudaMemsetAsync(sv->p, 0, (size_t)nb * L.d.npad * 8, sv->st), "coarse cg");
    SCK(cudaMemsetAsync(dots, 0, 6 * 8, sv->st), "coarse cg");
    k_ccg_init<<<g, tpb(L.d), 0, sv->st>>>(L.ops64(), L.d, rc, sv->r, sv->z, sv->p, dots);
    double h[6];
    SCK(cudaMemcpyAsync(h, dots, 6 * 8, cudaMemcpyDeviceToHost, sv->st), "coarse cg");
    SCK(cudaStreamSynchronize(sv->st), "coarse cg");
    const double rr0 = h[2];
    if (!(rr0 > 0)) return FALCON_OK;
    for (int it = 0; it < 50000; ++it) {
        SCK(halo_fill<double>(sv, lc, sv->p), "coarse cg");
        SCK(cudaMemsetAsync(dots + 1, 0, 8, sv->st), "coarse cg");
        SCK(cudaMemsetAsync(dots + 3, 0, 3 * 8, sv->st), "coarse cg");
        k_ccg_spmv<<<g, tpb(L.d), 0, sv->st>>>(L.ops64(), L.d, sv->p, sv->Ap, dots);
        k_ccg_update<<<g, tpb(L.d), 0, sv->st>>>(L.ops64(), L.d, sv->x, sv->p, sv->r, sv->Ap, sv->z, dots, dots + 3);
        k_ccg_p<<<g, tpb(L.d), 0, sv->st>>>(L.d, sv->p, sv->z, dots, dots + 3);
        SCK(cudaGetLastError(), "coarse cg");
        SCK(cudaMemcpyAsync(dots, dots + 3, 3 * 8, cudaMemcpyDeviceToDevice, sv->st), "coarse cg");
        SCK(cudaMemcpyAsync(h, dots + 3, 3 * 8, cudaMemcpyDeviceToHost, sv->st), "coarse cg");
        SCK(cudaStreamSynchronize(sv->st), "coarse cg");
        if (h[2] <= 1e-12 * rr0) return FALCON_OK;
    }
    return sv->fail(FALCON_ERR_NOT_CONVERGED, "coarse solve did not reach 1e-6");
}

// The operators of every level on the device again, after the level-0
// operator changed on the host (falcon_solver_set_operator): FP64 and FP32
// copies of each level, the scaled float-float level 0 with its new sA, and
// the learned stage's static input channels. Same sizes, same buffers: the
// captured V-cycle graphs stay valid.
int reupload_operators(falcon_solver* sv) {
    const SolverProblemSet& S = sv->S;
    const int nb = S.nblocks;
    SCK(cudaStreamSynchronize(sv->st), "operator");
    for (int l = 0; l < S.nlevels; ++l) {
        const SolverLevel& H = S.L[l];
        SvLevel& L = sv->lv[l];
        const std::vector<double>* src[4] = {&H.Aii, &H.Ai, &H.Aj, &H.Ak};
        double* d64[4] = {L.Aii, L.Ai, L.Aj, L.Ak};
        float* d32[4] = {L.fAii, L.fAi, L.fAj, L.fAk};
        for (int a = 0; a < 4; ++a) {
            const std::vector<double>& h = *src[a];
            std::vector<float> f(h.begin(), h.end());
            SCK(cudaMemcpy(d64[a], h.data(), h.size() * 8, cudaMemcpyHostToDevice), "operator");
            SCK(cudaMemcpy(d32[a], f.data(), f.size() * 4, cudaMemcpyHostToDevice), "operator");
        }
    }
    const SolverLevel& H = S.L[0];
    const size_t nint = (size_t)sv->lv[0].d.nint;
    sv->sA = problem_scale(S, H.Aii, nint);
    SvLevel& L0 = sv->lv[0];
    const std::vector<double>* src[4] = {&H.Aii, &H.Ai, &H.Aj, &H.Ak};
    float2* dff[4] = {L0.Aii2, L0.Ai2, L0.Aj2, L0.Ak2};
    for (int a = 0; a < 4; ++a) {
        const std::vector<double>& h = *src[a];
        const size_t per = h.size() / (size_t)nb;
        std::vector<double> sc(h.size());
        for (int b = 0; b < nb; ++b)
            for (size_t c = 0; c < per; ++c) sc[(size_t)b * per + c] = sv->sA[S.block_problem[b]];
        const std::vector<float2> f = to_ff(h, sc);
        SCK(cudaMemcpy(dff[a], f.data(), f.size() * sizeof(float2), cudaMemcpyHostToDevice), "operator");
    }
    std::vector<float> fa(sv->sA.begin(), sv->sA.end());
    SCK(cudaMemcpy(sv->dsA, fa.data(), fa.size() * 4, cudaMemcpyHostToDevice), "operator");
    if (sv->cmap_ok) {
        SvLevel& Lc = sv->lv[S.nlevels - 1];
        k_lcc_static<<<grid_cells(Lc.d, nb), tpb(Lc.d), 0, sv->st>>>(Lc.ops64(), Lc.d, sv->gmap, sv->feat);
        SCK(cudaGetLastError(), "coarse features");
    }
    SCK(cudaStreamSynchronize(sv->st), "operator");
    return FALCON_OK;
}

bool all_finite(const double* v, size_t n) {
    for (size_t q = 0; q < n; ++q)
        if (!std::isfinite(v[q])) return false;
    return true;
}

// ---- the inner solve: one FCG iteration, as a graph or eagerly ----------------
// One iteration unit on the stream. `first`: z = M r, p = z (restart); else
// z = M r, beta = -z.Ap / p.Ap, p = z + beta p. Then the halo of p, q = A p
// with p.q and p.r, alpha, x += alpha p, r -= alpha q with r.r, and the
// device-side check (k_inner_check), which sets the WHILE condition when
// `set_cond`. Inactive problems take no step.
cudaError_t enqueue_iteration(falcon_solver* sv, int pc, bool first, cudaGraphConditionalHandle h, int set_cond) {
    const int nb = sv->S.nblocks, np = sv->S.nproblems;
    const LevelDims& d = sv->lv[0].d;
    const dim3 g = grid_cells(d, nb);
    cudaError_t e = cudaSuccess;
    if (pc != FALCON_PRECOND_NONE) {
        sv->use_net = pc == FALCON_PRECOND_MG_LCC;
        e = vcycle(sv);
        sv->use_net = false;
        if (e != cudaSuccess) return e;
    }
    k_take_z_ff<<<g, tpb(d), 0, sv->st>>>(d, sv->lv[0].z, sv->dsA, sv->r2, pc == FALCON_PRECOND_NONE, sv->z2, sv->Ap2,
                                          sv->D(), first ? 0 : 1);
    k_update_p_ff<<<g, tpb(d), 0, sv->st>>>(d, sv->p2, sv->z2, sv->D(), first ? 1 : 0);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = halo_fill_ff(sv, sv->p2);
    if (e == cudaSuccess) e = cudaMemsetAsync(sv->dots, 0, (size_t)4 * np * 8, sv->st);
    if (e != cudaSuccess) return e;
    k_spmv_dots_ff<<<g, tpb(d), 0, sv->st>>>(sv->lv[0].ops2(), d, sv->p2, sv->Ap2, sv->r2, sv->D());
    k_update_xr_ff<<<g, tpb(d), 0, sv->st>>>(d, sv->x2, sv->p2, sv->r2, sv->Ap2, sv->lv[0].r, sv->D());
    k_inner_check<<<1, 256, 0, sv->st>>>(np, sv->dots + 3 * np, sv->rr0, sv->eta, sv->active, sv->ictl, h, set_cond);
    return cudaGetLastError();
}

// The inner solve as one graph: the first iteration, then a WHILE node whose
// body is a continuing iteration; the loop runs on the device until every
// problem reached its eta, the residual stalls, or max_it (k_inner_check).
cudaError_t build_inner_graph(falcon_solver* sv, int pc, cudaGraphExec_t* out) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e != cudaSuccess) return e;
    cudaGraphConditionalHandle h;
    e = cudaGraphConditionalHandleCreate(&h, g, 0, 0);
    sv->capturing = true;
    if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(sv->st, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        const cudaError_t eb = enqueue_iteration(sv, pc, true, h, 1);
        e = cudaStreamEndCapture(sv->st, &g);
        if (eb != cudaSuccess) e = eb;
    }
    // the captured chain's last node is the check; the WHILE node follows it
    std::vector<cudaGraphNode_t> leaves;
    if (e == cudaSuccess) {
        size_t nn = 0, ne = 0;
        e = cudaGraphGetNodes(g, nullptr, &nn);
        std::vector<cudaGraphNode_t> nodes(nn);
        if (e == cudaSuccess) e = cudaGraphGetNodes(g, nodes.data(), &nn);
        if (e == cudaSuccess) e = cudaGraphGetEdges(g, nullptr, nullptr, nullptr, &ne);
        std::vector<cudaGraphNode_t> from(ne), to(ne);
        if (e == cudaSuccess && ne) e = cudaGraphGetEdges(g, from.data(), to.data(), nullptr, &ne);
        for (cudaGraphNode_t n : nodes)
            if (std::find(from.begin(), from.end(), n) == from.end()) leaves.push_back(n);
    }
    if (e == cudaSuccess) {
        cudaGraphNodeParams p = {};
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = h;
        p.conditional.type = cudaGraphCondTypeWhile;
        p.conditional.size = 1;
        cudaGraphNode_t wn;
        e = cudaGraphAddNode(&wn, g, leaves.data(), nullptr, leaves.size(), &p);
        if (e == cudaSuccess) {
            cudaGraph_t body = p.conditional.phGraph_out[0];
            e = cudaStreamBeginCaptureToGraph(sv->st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                const cudaError_t eb = enqueue_iteration(sv, pc, false, h, 1);
                e = cudaStreamEndCapture(sv->st, &body);
                if (eb != cudaSuccess) e = eb;
            }
        }
    }
    sv->capturing = false;
    if (e == cudaSuccess) e = cudaGraphInstantiate(out, g, 0);
    if (g) cudaGraphDestroy(g);
    return e;
}

// One inner solve from the current r2 (x2 = 0): the graph when the solve is
// not recording coarse residuals, else the same iterations eagerly with the
// host reading the loop control after each. Fills ctl (host copy).
cudaError_t run_inner(falcon_solver* sv, int pc, int max_it, InnerCtl* ctl) {
    InnerCtl c0;
    std::memset(&c0, 0, sizeof c0);
    c0.max_it = std::max(1, std::min(max_it, kInnerCap));
    cudaError_t e = cudaMemcpyAsync(sv->ictl, &c0, sizeof c0, cudaMemcpyHostToDevice, sv->st);
    if (e != cudaSuccess) return e;
    if (!sv->rec) {
        const int64_t key = (int64_t)pc | ((int64_t)sv->nu_pre << 4) | ((int64_t)sv->nu_post << 12) |
                            ((int64_t)sv->nu_coarse << 20) | ((int64_t)sv->net_sweeps << 34);
        auto it = sv->igraphs.find(key);
        if (it == sv->igraphs.end()) {
            cudaGraphExec_t x = nullptr;
            e = build_inner_graph(sv, pc, &x);
            if (e != cudaSuccess) return e;
            it = sv->igraphs.emplace(key, x).first;
        }
        e = cudaGraphLaunch(it->second, sv->st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(ctl, sv->ictl, sizeof *ctl, cudaMemcpyDeviceToHost, sv->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(sv->st);
        return e;
    }
    for (bool first = true;; first = false) {
        e = enqueue_iteration(sv, pc, first, 0, 0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(ctl, sv->ictl, sizeof *ctl, cudaMemcpyDeviceToHost, sv->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(sv->st);
        if (e != cudaSuccess || !ctl->cont) return e;
    }
}

// The tile shape of every cell kernel (all levels); launch shapes are baked
// into the captured graphs, so they go.
void apply_tile(falcon_solver* sv, int chunk, int tpb_) {
    sv->tile_chunk = chunk;
    sv->tile_tpb = tpb_;
    for (SvLevel& L : sv->lv) {
        L.d.chunk = chunk;
        L.d.tpb = tpb_;
    }
    sv->clear_graphs();
}

// The solver's autotuner: times one eager FCG iteration (V-cycle with the
// solver's smoothing, the float-float kernels, halo fills) for each candidate
// tile -- cells per CTA in {512, 1024, 2048, 4096} (a multiple of the row
// length, so the red-black sweep's colour-only form applies) x threads per
// CTA in {128, 256, 512} -- on this solver's own grid, and keeps the fastest.
// Runs once, at the first solve, on scratch vectors that the solve
// initialises afterwards.
int autotune_tile(falcon_solver* sv) {
    if (sv->tuned) return FALCON_OK;
    const int np = sv->S.nproblems;
    const int m0 = sv->lv[0].d.m0;
    std::vector<int32_t> act(np, 1);
    std::vector<double> ones(np, 1.0), zeros(np, 0.0);
    SCK(cudaMemcpyAsync(sv->active, act.data(), np * 4, cudaMemcpyHostToDevice, sv->st), "tune");
    SCK(cudaMemcpyAsync(sv->rr0, ones.data(), np * 8, cudaMemcpyHostToDevice, sv->st), "tune");
    SCK(cudaMemcpyAsync(sv->eta, zeros.data(), np * 8, cudaMemcpyHostToDevice, sv->st), "tune");
    SCK(cudaStreamSynchronize(sv->st), "tune");
    const int pc = sv->S.nlevels > 1 ? FALCON_PRECOND_MG : FALCON_PRECOND_NONE;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float best = 1e30f;
    int bc = sv->tile_chunk, bt = sv->tile_tpb;
    for (int chunk : {512, 1024, 2048, 4096}) {
        if (chunk % m0) continue;
        for (int t : {128, 256, 512}) {
            apply_tile(sv, chunk, t);
            InnerCtl c0;
            std::memset(&c0, 0, sizeof c0);
            c0.max_it = kInnerCap;
            SCK(cudaMemcpyAsync(sv->ictl, &c0, sizeof c0, cudaMemcpyHostToDevice, sv->st), "tune");
            SCK(enqueue_iteration(sv, pc, false, 0, 0), "tune");   // warm-up
            cudaEventRecord(a, sv->st);
            for (int r = 0; r < 2; ++r) SCK(enqueue_iteration(sv, pc, false, 0, 0), "tune");
            cudaEventRecord(b, sv->st);
            SCK(cudaEventSynchronize(b), "tune");
            float ms = 0;
            cudaEventElapsedTime(&ms, a, b);
            if (ms < best) { best = ms; bc = chunk; bt = t; }
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    apply_tile(sv, bc, bt);
    sv->tuned = true;
    sv->tuned_ms = best / 2.0;
    return FALCON_OK;
}

}  // namespace

extern "C" {

int falcon_solver_set_operator(falcon_solver* sv, const double* Aii, const double* Ai, const double* Aj, const double* Ak) {
    if (!sv || !Aii || !Ai || !Aj || !Ak) return FALCON_ERR_INVALID_ARG;
    SolverProblemSet& S = sv->S;
    SolverLevel& L = S.L[0];
    const double* in[4] = {Aii, Ai, Aj, Ak};
    std::vector<double>* dst[4] = {&L.Aii, &L.Ai, &L.Aj, &L.Ak};
    for (int a = 0; a < 4; ++a)
        if (!all_finite(in[a], dst[a]->size())) return sv->fail(FALCON_ERR_INVALID_ARG, "falcon_solver_set_operator: non-finite coefficient");
    for (size_t q = 0; q < L.Aii.size(); ++q)
        if (!(Aii[q] > 0.0)) return sv->fail(FALCON_ERR_INVALID_ARG, "falcon_solver_set_operator: the diagonal Aii must be positive");
    for (int a = 0; a < 4; ++a) std::memcpy(dst[a]->data(), in[a], dst[a]->size() * 8);
    galerkin_coarsen(S);
    if (!sv->st) return FALCON_OK;
    cudaSetDevice(sv->device);
    return reupload_operators(sv);
}

int falcon_solver_set_magnetogram(falcon_solver* sv, const double* br) {
    if (!sv || !br) return FALCON_ERR_INVALID_ARG;
    SolverProblemSet& S = sv->S;
    if (S.br.empty()) return sv->fail(FALCON_ERR_INVALID_ARG, "falcon_solver_set_magnetogram: not a PFSS solver");
    if (!all_finite(br, S.br.size())) return sv->fail(FALCON_ERR_INVALID_ARG, "falcon_solver_set_magnetogram: non-finite Br");
    std::vector<double> b(br, br + S.br.size());
    for (int gb = 0; gb < S.nblocks; ++gb)   // only bottom blocks carry a magnetogram
        if (!(S.block_flags[gb] & 4)) std::fill(b.begin() + (size_t)gb * (S.br.size() / S.nblocks),
                                                b.begin() + (size_t)(gb + 1) * (S.br.size() / S.nblocks), 0.0);
    pfss_rhs(S, b);
    if (!sv->st) return FALCON_OK;
    cudaSetDevice(sv->device);
    SCK(cudaStreamSynchronize(sv->st), "rhs");
    SCK(cudaMemcpy(sv->bvec, S.b.data(), S.b.size() * 8, cudaMemcpyHostToDevice), "rhs");
    return FALCON_OK;
}

int falcon_solver_magnetogram(const falcon_solver* sv, double* br) {
    if (!sv || !br) return FALCON_ERR_INVALID_ARG;
    if (sv->S.br.empty()) return FALCON_ERR_INVALID_ARG;
    std::memcpy(br, sv->S.br.data(), sv->S.br.size() * 8);
    return FALCON_OK;
}

int falcon_solver_vcycle_op(falcon_solver* sv, int32_t op, int32_t level, const float* in0, const float* in1,
                            float* out) {
    if (!sv || !in0 || !out) return FALCON_ERR_INVALID_ARG;
    if (!sv->st) return sv->fail(FALCON_ERR_NO_DEVICE, "solver created without a device");
    const int nl = sv->S.nlevels, nb = sv->S.nblocks;
    const bool needs_coarse = op == FALCON_VCYCLE_RESTRICT || op == FALCON_VCYCLE_PROLONG_ADD;
    if (op < FALCON_VCYCLE_RESTRICT || op > FALCON_VCYCLE_RESIDUAL || level < 0 || level >= nl ||
        (needs_coarse && level + 1 >= nl) || (op != FALCON_VCYCLE_RESTRICT && !in1))
        return sv->fail(FALCON_ERR_INVALID_ARG, "falcon_solver_vcycle_op: bad operation, level or input");
    cudaSetDevice(sv->device);
    SvLevel& L = sv->lv[level];
    const size_t nf = (size_t)nb * L.d.nint;
    const dim3 gf = grid_cells(L.d, nb);
    SCK(cudaStreamSynchronize(sv->st), "vcycle op");
    if (op == FALCON_VCYCLE_RESTRICT) {
        SvLevel& Cl = sv->lv[level + 1];
        SCK(cudaMemcpyAsync(L.res, in0, nf * 4, cudaMemcpyHostToDevice, sv->st), "vcycle op");
        k_restrict<<<grid_cells(Cl.d, nb), tpb(Cl.d), 0, sv->st>>>(L.d, Cl.d, L.res, Cl.r);
        SCK(cudaGetLastError(), "vcycle op");
        SCK(cudaMemcpyAsync(out, Cl.r, (size_t)nb * Cl.d.nint * 4, cudaMemcpyDeviceToHost, sv->st), "vcycle op");
    } else if (op == FALCON_VCYCLE_PROLONG_ADD) {
        SvLevel& Cl = sv->lv[level + 1];
        const size_t nc = (size_t)nb * Cl.d.nint;
        SCK(cudaMemsetAsync(Cl.z, 0, (size_t)nb * Cl.d.npad * 4, sv->st), "vcycle op");
        SCK(cudaMemsetAsync(L.z, 0, (size_t)nb * L.d.npad * 4, sv->st), "vcycle op");
        SCK(cudaMemcpyAsync(Cl.r, in0, nc * 4, cudaMemcpyHostToDevice, sv->st), "vcycle op");
        SCK(cudaMemcpyAsync(L.res, in1, nf * 4, cudaMemcpyHostToDevice, sv->st), "vcycle op");
        k_scatter_pad<float><<<grid_cells(Cl.d, nb), tpb(Cl.d), 0, sv->st>>>(Cl.d, Cl.r, Cl.z);
        k_scatter_pad<float><<<gf, tpb(L.d), 0, sv->st>>>(L.d, L.res, L.z);
        k_prolong_add<<<gf, tpb(L.d), 0, sv->st>>>(L.d, Cl.d, Cl.z, L.z);
        k_gather_pad<float><<<gf, tpb(L.d), 0, sv->st>>>(L.d, L.z, L.res);
        SCK(cudaGetLastError(), "vcycle op");
        SCK(cudaMemcpyAsync(out, L.res, nf * 4, cudaMemcpyDeviceToHost, sv->st), "vcycle op");
    } else {
        // z (interior) into the padded z, its halo filled, then one red-black
        // half sweep of a colour or the residual r - A z
        SCK(cudaMemsetAsync(L.z, 0, (size_t)nb * L.d.npad * 4, sv->st), "vcycle op");
        SCK(cudaMemcpyAsync(L.r, in0, nf * 4, cudaMemcpyHostToDevice, sv->st), "vcycle op");
        SCK(cudaMemcpyAsync(L.res, in1, nf * 4, cudaMemcpyHostToDevice, sv->st), "vcycle op");
        k_scatter_pad<float><<<gf, tpb(L.d), 0, sv->st>>>(L.d, L.res, L.z);
        SCK(halo_fill<float>(sv, level, L.z), "vcycle op");
        if (op == FALCON_VCYCLE_RESIDUAL) {
            k_resid32<<<gf, tpb(L.d), 0, sv->st>>>(L.ops32(), L.d, L.r, L.z, L.res);
        } else {
            k_rbgs<<<gf, tpb(L.d), 0, sv->st>>>(L.ops32(), L.d, L.r, L.z, op == FALCON_VCYCLE_SMOOTH_RED ? 0 : 1);
            k_gather_pad<float><<<gf, tpb(L.d), 0, sv->st>>>(L.d, L.z, L.res);
        }
        SCK(cudaGetLastError(), "vcycle op");
        SCK(cudaMemcpyAsync(out, L.res, nf * 4, cudaMemcpyDeviceToHost, sv->st), "vcycle op");
    }
    SCK(cudaStreamSynchronize(sv->st), "vcycle op");
    return FALCON_OK;
}

int falcon_solver_tuning(const falcon_solver* sv, int32_t* tile, double* ms_per_iteration) {
    if (!sv || !tile) return FALCON_ERR_INVALID_ARG;
    tile[0] = sv->tile_chunk;
    tile[1] = sv->tile_tpb;
    tile[2] = sv->tuned ? 1 : 0;
    if (ms_per_iteration) *ms_per_iteration = sv->tuned_ms;
    return FALCON_OK;
}

int falcon_solver_set_tile(falcon_solver* sv, int32_t cells_per_cta, int32_t threads_per_cta) {
    if (!sv) return FALCON_ERR_INVALID_ARG;
    if (cells_per_cta < 32 || cells_per_cta > (1 << 16) || (cells_per_cta & 31) || threads_per_cta < 32 ||
        threads_per_cta > 1024 || (threads_per_cta & 31))
        return sv->fail(FALCON_ERR_INVALID_ARG,
                        "falcon_solver_set_tile: cells per CTA in [32, 65536] and threads per CTA in [32, 1024], "
                        "both multiples of 32");
    if (sv->st) {
        cudaSetDevice(sv->device);
        SCK(cudaStreamSynchronize(sv->st), "tile");
    }
    apply_tile(sv, cells_per_cta, threads_per_cta);
    sv->tuned = true;   // the caller's shape: no autotuning
    sv->tuned_ms = 0;
    return FALCON_OK;
}

int falcon_solver_block_ranges(const falcon_solver* sv, double* ranges) {
    if (!sv || !ranges) return FALCON_ERR_INVALID_ARG;
    const SolverProblemSet& S = sv->S;
    for (int gb = 0; gb < S.nblocks; ++gb) {
        const int p = S.block_problem[gb];
        const int b = gb - S.problem_first_block[p];
        std::memcpy(ranges + (size_t)gb * 6, &S.grids[p].ranges[(size_t)b * 6], 6 * sizeof(double));
    }
    return FALCON_OK;
}

int falcon_solver_block_flags(const falcon_solver* sv, int32_t* flags) {
    if (!sv || !flags) return FALCON_ERR_INVALID_ARG;
    std::memcpy(flags, sv->S.block_flags.data(), sv->S.block_flags.size() * sizeof(int32_t));
    return FALCON_OK;
}

int falcon_solver_magnetogram_sources(const falcon_solver* sv, int32_t problem, double* xyzq, int32_t cap,
                                      int32_t* n) {
    if (!sv || !n || problem < 0 || problem >= sv->S.nproblems) return FALCON_ERR_INVALID_ARG;
    if (sv->S.br.empty()) return FALCON_ERR_INVALID_ARG;
    Magnetogram M;
    M.init(sv->seed + (uint64_t)problem, sv->r_surface);
    *n = (int32_t)M.q.size();
    if (!xyzq) return FALCON_OK;
    if (cap < *n) return FALCON_ERR_BOUNDS;
    for (size_t c = 0; c < M.q.size(); ++c) {
        xyzq[4 * c] = M.px[c];
        xyzq[4 * c + 1] = M.py[c];
        xyzq[4 * c + 2] = M.pz[c];
        xyzq[4 * c + 3] = M.q[c];
    }
    return FALCON_OK;
}

int falcon_solver_set_guess(falcon_solver* sv, const double* x0) {
    if (!sv || !x0) return FALCON_ERR_INVALID_ARG;
    if (!all_finite(x0, sv->S.x0.size())) return sv->fail(FALCON_ERR_INVALID_ARG, "falcon_solver_set_guess: non-finite value");
    std::memcpy(sv->S.x0.data(), x0, sv->S.x0.size() * 8);
    return FALCON_OK;
}

int falcon_solver_create(falcon_solver** out, const falcon_solver_spec* spec) {
    if (!out || !spec) return FALCON_ERR_INVALID_ARG;
    falcon_solver* sv = new falcon_solver();
    *out = sv;
    if (spec->nproblems < 1 || spec->nproblems > FALCON_MAX_PROBLEMS) return sv->fail(FALCON_ERR_INVALID_ARG, "nproblems out of range");
    if (spec->block < 2 || spec->block > 32 || (spec->block & 1)) return sv->fail(FALCON_ERR_INVALID_ARG, "block must be even, 2..32");
    sv->device = spec->device;
    sv->seed = spec->seed;
    if (spec->kind == FALCON_SOLVER_CONDUCTION) {
        sv->nu_coarse = 4;
    } else {   // PFSS: one sweep each way, 32 on the coarsest level (measured fastest to 1e-10)
        sv->nu_pre = sv->nu_post = 1;
        sv->nu_coarse = 32;
    }
    std::vector<falcon_config> cfgs(spec->nproblems);
    const double kRsun = (double)6.955e10f;
    for (int q = 0; q < spec->nproblems; ++q) {
        falcon_config& c = cfgs[q];
        std::memset(&c, 0, sizeof c);
        falcon_tree_spec& t = c.tree;
        t.ni = t.nj = t.nk = spec->block;
        t.ng = 2;
        const int B = spec->block;
        if (spec->kind == FALCON_SOLVER_PFSS) {
            // (nr, ntheta) -> per panel (nr, ntheta/2, 3 ntheta/2) rounded up to whole blocks
            const int Nr = (spec->nr[q] + B - 1) / B;
            const int Nt = (spec->nt[q] / 2 + B - 1) / B;
            t.root_tiles[0] = Nr; t.root_tiles[1] = Nt; t.root_tiles[2] = 3 * Nt;
            t.radial_levels = 0; t.radial_option = 2; t.n_amr = 0;
        } else {
            // conduction: per panel nr x nt x np cells, uniform radial blocks
            const int Nr = spec->nr[q] / B, Nt = spec->nt[q] / B, Np = spec->np[q] / B;
            if (Nr * B != spec->nr[q] || Nt * B != spec->nt[q] || Np * B != spec->np[q] || Np != 3 * Nt)
                return sv->fail(FALCON_ERR_INVALID_ARG, "conduction grid must be whole blocks with np = 3 nt");
            t.root_tiles[0] = Nr; t.root_tiles[1] = Nt; t.root_tiles[2] = Np;
            t.radial_option = 2;
        }
        t.r_range_rsun[0] = spec->r_range_rsun[0];
        t.r_range_rsun[1] = spec->r_range_rsun[1];
        c.phys.cfl = 0.4;
        c.bg.poly_n = 1.5; c.bg.density_contrast = 100.0; c.bg.mu = 0.6; c.bg.xi_mode = 1;
        c.device = spec->device;
    }
    std::string e = build_solver_levels(sv->S, cfgs, spec->nlevels);
    if (!e.empty()) return sv->fail(FALCON_ERR_INVALID_ARG, e);
    SolverProblemSet& S = sv->S;
    if (spec->kind == FALCON_SOLVER_PFSS) {
        // magnetogram Br at the bottom face centres of bottom blocks (Yin frame)
        const SolverLevel& L = S.L[0];
        const int mj = L.m[1], mk = L.m[2];
        std::vector<double> br((size_t)S.nblocks * mj * mk, 0.0);
        for (int q = 0; q < S.nproblems; ++q) {
            Magnetogram M;
            sv->r_surface = spec->r_range_rsun[0] * kRsun;
            M.init(spec->seed + (uint64_t)q, sv->r_surface);
            for (int gb = S.problem_first_block[q]; gb < S.problem_first_block[q + 1]; ++gb) {
                if (!(S.block_flags[gb] & 4)) continue;
                const bool yin = S.block_flags[gb] & 1;
                const Grid& g = S.grids[q];
                const int b = gb - S.problem_first_block[q];
                const double r0 = g.ranges[(size_t)b * 6 + 0];
                for (int k = 1; k <= mk; ++k)
                    for (int j = 1; j <= mj; ++j) {
                        double t = L.xj[(size_t)gb * (mj + 2) + j], ph = L.xk[(size_t)gb * (mk + 2) + k];
                        if (!yin) {
                            const double a[3] = {r0, t, ph};
                            const double st_ = std::sin(a[1]), ct = std::cos(a[1]), sp = std::sin(a[2]), cp = std::cos(a[2]);
                            t = std::acos(st_ * sp);
                            ph = std::copysign(std::fabs(std::acos(-(st_ * cp) / std::sqrt(st_ * st_ * (cp * cp) + ct * ct))), ct);
                        }
                        br[((size_t)gb * mk + (k - 1)) * mj + (j - 1)] = M.br(r0, t, ph);
                    }
            }
        }
        assemble_pfss(S, br);
    } else {
        ConductionField F;
        F.init(&S.grids[0].bg, spec->seed, S.grids[0].r_range[0]);
        assemble_conduction(S, F, spec->dt_factor > 0 ? spec->dt_factor : 50.0, &sv->dt_conduction);
    }
    galerkin_coarsen(S);
    if (spec->device < 0) return FALCON_OK;
    return setup(sv);
}

void falcon_solver_destroy(falcon_solver* sv) {
    if (!sv) return;
    if (sv->st) {
        cudaSetDevice(sv->device);
        cudaStreamSynchronize(sv->st);
        sv->clear_graphs();
        for (void* q : sv->allocs) cudaFree(q);
        cudaStreamDestroy(sv->st);
    }
    delete sv;
}

int falcon_solver_last_error(const falcon_solver* sv, char* buf, size_t len) {
    if (!sv || !buf || !len) return FALCON_ERR_INVALID_ARG;
    snprintf(buf, len, "%s", sv->err.c_str());
    return FALCON_OK;
}

int falcon_solver_info(const falcon_solver* sv, int32_t* info) {
    if (!sv || !info) return FALCON_ERR_INVALID_ARG;
    info[0] = sv->S.nblocks;
    info[1] = sv->S.nproblems;
    info[2] = sv->S.nlevels;
    for (int d = 0; d < 3; ++d) info[3 + d] = sv->S.nlevels ? sv->S.L[0].m[d] : 0;
    return FALCON_OK;
}

int falcon_solver_problem_blocks(const falcon_solver* sv, int32_t* first) {
    if (!sv || !first) return FALCON_ERR_INVALID_ARG;
    std::memcpy(first, sv->S.problem_first_block.data(), sv->S.problem_first_block.size() * 4);
    return FALCON_OK;
}

int falcon_solver_rhs(const falcon_solver* sv, double* b) {
    if (!sv || !b) return FALCON_ERR_INVALID_ARG;
    std::memcpy(b, sv->S.b.data(), sv->S.b.size() * 8);
    return FALCON_OK;
}

int falcon_solver_operator(const falcon_solver* sv, int32_t level, double* Aii, double* Ai, double* Aj, double* Ak) {
    if (!sv || level < 0 || level >= sv->S.nlevels) return FALCON_ERR_INVALID_ARG;
    const SolverLevel& L = sv->S.L[level];
    if (Aii) std::memcpy(Aii, L.Aii.data(), L.Aii.size() * 8);
    if (Ai) std::memcpy(Ai, L.Ai.data(), L.Ai.size() * 8);
    if (Aj) std::memcpy(Aj, L.Aj.data(), L.Aj.size() * 8);
    if (Ak) std::memcpy(Ak, L.Ak.data(), L.Ak.size() * 8);
    return FALCON_OK;
}

int falcon_solver_halo_count(const falcon_solver* sv, int32_t level, int64_t* n) {
    if (!sv || !n || level < 0 || level >= sv->S.nlevels) return FALCON_ERR_INVALID_ARG;
    *n = (int64_t)sv->S.L[level].halo.size();
    return FALCON_OK;
}

// entries: [n][8] int32 (tb,ti,tj,tk,sb,i0,j0,k0) and [n][6] double (w, src_x)
int falcon_solver_halo_map(const falcon_solver* sv, int32_t level, int32_t* idx, double* wx) {
    if (!sv || level < 0 || level >= sv->S.nlevels) return FALCON_ERR_INVALID_ARG;
    const auto& H = sv->S.L[level].halo;
    for (size_t q = 0; q < H.size(); ++q) {
        const HaloEntry& h = H[q];
        const int32_t v[8] = {h.tb, h.ti, h.tj, h.tk, h.sb, h.i0, h.j0, h.k0};
        std::memcpy(idx + 8 * q, v, sizeof v);
        for (int d = 0; d < 3; ++d) { wx[6 * q + d] = h.w[d]; wx[6 * q + 3 + d] = h.src_x[d]; }
    }
    return FALCON_OK;
}

// y = A x at level 0 on the GPU (x interior [b][nint]; halo filled on the device)
int falcon_solver_apply(falcon_solver* sv, const double* x, double* y) {
    if (!sv || !x || !y) return FALCON_ERR_INVALID_ARG;
    if (!sv->st) return sv->fail(FALCON_ERR_NO_DEVICE, "solver created without a device");
    cudaSetDevice(sv->device);
    const LevelDims& d = sv->lv[0].d;
    const int nb = sv->S.nblocks;
    SCK(cudaMemcpyAsync(sv->z, x, (size_t)nb * d.nint * 8, cudaMemcpyHostToDevice, sv->st), "apply");
    SCK(cudaMemsetAsync(sv->p, 0, (size_t)nb * d.npad * 8, sv->st), "apply");
    k_scatter_pad<double><<<grid_cells(d, nb), tpb(d), 0, sv->st>>>(d, sv->z, sv->p);
    SCK(halo_fill<double>(sv, 0, sv->p), "apply halo");
    SCK(cudaMemsetAsync(sv->dots, 0, (size_t)6 * sv->S.nproblems * 8, sv->st), "apply");
    k_spmv_dots<<<grid_cells(d, nb), tpb(d), 0, sv->st>>>(sv->lv[0].ops64(), d, sv->p, sv->Ap, sv->r, sv->D());
    SCK(cudaGetLastError(), "apply");
    SCK(cudaMemcpyAsync(y, sv->Ap, (size_t)nb * d.nint * 8, cudaMemcpyDeviceToHost, sv->st), "apply");
    SCK(cudaStreamSynchronize(sv->st), "apply");
    return FALCON_OK;
}

int falcon_solver_solve(falcon_solver* sv, double tol, int32_t max_iter, int32_t precond, falcon_solve_report* rep) {
    if (!sv || !rep) return FALCON_ERR_INVALID_ARG;
    if (!sv->st) return sv->fail(FALCON_ERR_NO_DEVICE, "solver created without a device");
    if (precond != FALCON_PRECOND_NONE && precond != FALCON_PRECOND_MG && precond != FALCON_PRECOND_MG_LCC)
        return sv->fail(FALCON_ERR_INVALID_ARG, "unknown preconditioner");
    if (precond == FALCON_PRECOND_MG_LCC && (!sv->net || !sv->cmap_ok))
        return sv->fail(FALCON_ERR_INVALID_ARG, "FALCON_PRECOND_MG_LCC needs falcon_solver_attach_lcc first");
    if (!(tol > 0.0) || max_iter < 0) return sv->fail(FALCON_ERR_INVALID_ARG, "tol must be positive and max_iter >= 0");
    cudaSetDevice(sv->device);
    const SolverProblemSet& S = sv->S;
    const int nb = S.nblocks, np = S.nproblems;
    const LevelDims& d = sv->lv[0].d;
    std::memset(rep, 0, sizeof *rep);
    // Structure (ModLinearSolver_Multigrid_CG, 3_5/ModLinearSolver.f90:313-427,
    // made an FP64 iterative refinement):
    //   outer, FP64: r = b - A x with FP64 dots; a problem is done when
    //     ||r||/||b|| <= tol -- the only convergence test;
    //   inner, float-float FCG + FP32 V-cycle: A' d' = r' on the correction
    //     equation scaled per problem (A' = A / sA, r' = r / sr), to a relative
    //     recursive residual of 0.5 tol ||b|| / ||r|| (at least 2^-40);
    //   x += d' sr / sA in FP64.
    // A problem whose FP64 residual is at the attainable accuracy of b - A x
    // (4 x 8 eps64 (|b| + |A||x|) / ||b||) or that a refinement no longer
    // halves stops unconverged; its residual is reported as floor_residual.
    constexpr double kEps64 = 1.1102230246251565e-16;   // 2^-53
    constexpr double kEtaMin = 9.094947017729282e-13;   // 2^-40: float-float recursive residual limit
    constexpr int kMaxPasses = 30;
    {
        float* rec = sv->rec;   // the tuning iterations record nothing
        sv->rec = nullptr;
        const int rc = autotune_tile(sv);
        sv->rec = rec;
        if (rc) return rc;
    }
    // the launch grid of the tuned tile (the autotuner may just have changed it)
    const dim3 g = grid_cells(d, nb);
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    // x = x0 (FP64, padded; ghost cells 0 until the halo fill)
    SCK(cudaMemcpyAsync(sv->z, S.x0.data(), S.x0.size() * 8, cudaMemcpyHostToDevice, sv->st), "init");
    SCK(cudaMemsetAsync(sv->x, 0, (size_t)nb * d.npad * 8, sv->st), "init");
    SCK(cudaStreamSynchronize(sv->st), "init");
    cudaEventRecord(t0, sv->st);
    k_scatter_pad<double><<<g, tpb(d), 0, sv->st>>>(d, sv->z, sv->x);
    SCK(cudaGetLastError(), "init");
    // per problem: 0 being solved, 1 converged (FP64 residual <= tol), 2 stopped at its floor
    std::vector<int> state(np, 0);
    std::vector<int32_t> act(np, 0);
    std::vector<double> rr(np), bb(np), ab(np), rel(np, 0.0), prev(np, 0.0), rr0(np), eta(np);
    std::vector<double> inv_sr(np, 1.0), fac(np, 1.0);
    int pc = precond;   // FALCON_PRECOND_MG_LCC falls back to FALCON_PRECOND_MG on stagnation
    int it = 0, passes = 0;
    for (bool first = true;; first = false) {
        // FP64 true residual of every problem
        SCK(cudaMemsetAsync(sv->dots + 3 * np, 0, (size_t)(first ? 3 : 1) * np * 8, sv->st), "dots");
        SCK(cudaMemsetAsync(sv->dots + 5 * np, 0, (size_t)np * 8, sv->st), "dots");
        SCK(halo_fill<double>(sv, 0, sv->x), "halo");
        k_residual64<<<g, tpb(d), 0, sv->st>>>(sv->lv[0].ops64(), d, sv->x, sv->bvec, sv->r, sv->lv[0].r, sv->D(),
                                               first ? 1 : 0);
        SCK(cudaGetLastError(), "residual");
        SCK(cudaMemcpyAsync(rr.data(), sv->dots + 3 * np, np * 8, cudaMemcpyDeviceToHost, sv->st), "rr");
        SCK(cudaMemcpyAsync(ab.data(), sv->dots + 5 * np, np * 8, cudaMemcpyDeviceToHost, sv->st), "rr");
        if (first) SCK(cudaMemcpyAsync(bb.data(), sv->dots + 4 * np, np * 8, cudaMemcpyDeviceToHost, sv->st), "bb");
        SCK(cudaStreamSynchronize(sv->st), "rr");
        if (first)
            for (int q = 0; q < np; ++q) if (!(bb[q] > 0)) bb[q] = 1.0;   // b = 0: absolute residual
        bool any = false;
        for (int q = 0; q < np; ++q) {
            if (state[q] != 0) continue;
            const double r_q = std::sqrt(rr[q] / bb[q]);
            if (!std::isfinite(r_q))
                return sv->fail(FALCON_ERR_NAN_DETECTED, "solver: non-finite FP64 residual in problem " + std::to_string(q));
            const double floor_q = 4.0 * 8.0 * kEps64 * std::sqrt(ab[q] / bb[q]);
            rel[q] = r_q;
            if (r_q <= tol) {
                state[q] = 1;
            } else if (r_q <= floor_q || (!first && r_q > 0.5 * prev[q])) {
                state[q] = 2;
                rep->floor_residual = std::max(rep->floor_residual, r_q);
            } else {
                any = true;
            }
            prev[q] = r_q;
        }
        if (!any || it >= max_iter || passes >= kMaxPasses) break;
        // inner solve of A' d' = r' for the problems still being solved
        ++passes;
        for (int q = 0; q < np; ++q) {
            act[q] = state[q] == 0;
            int e2 = 0;
            std::frexp(std::sqrt(rr[q]), &e2);
            const double sr = act[q] && rr[q] > 0 ? std::ldexp(1.0, e2) : 1.0;
            inv_sr[q] = 1.0 / sr;
            fac[q] = sr / sv->sA[q];
            eta[q] = std::max(0.5 * tol / std::max(rel[q], tol), kEtaMin);
        }
        SCK(cudaMemcpyAsync(sv->active, act.data(), np * 4, cudaMemcpyHostToDevice, sv->st), "active");
        SCK(cudaMemcpyAsync(sv->ir_par, inv_sr.data(), np * 8, cudaMemcpyHostToDevice, sv->st), "scale");
        SCK(cudaMemcpyAsync(sv->ir_par + np, fac.data(), np * 8, cudaMemcpyHostToDevice, sv->st), "scale");
        SCK(cudaMemsetAsync(sv->x2, 0, (size_t)nb * d.npad * sizeof(float2), sv->st), "init");
        SCK(cudaMemsetAsync(sv->p2, 0, (size_t)nb * d.npad * sizeof(float2), sv->st), "init");
        SCK(cudaMemsetAsync(sv->dots, 0, (size_t)5 * np * 8, sv->st), "dots");
        k_ir_start<<<g, tpb(d), 0, sv->st>>>(d, sv->r, sv->ir_par, sv->r2, sv->lv[0].r, sv->D());
        SCK(cudaGetLastError(), "inner start");
        SCK(cudaMemcpyAsync(rr0.data(), sv->dots + 3 * np, np * 8, cudaMemcpyDeviceToHost, sv->st), "rr");
        SCK(cudaStreamSynchronize(sv->st), "rr");
        for (int q = 0; q < np; ++q) if (!(rr0[q] > 0)) { rr0[q] = 1.0; act[q] = 0; }
        SCK(cudaMemcpyAsync(sv->active, act.data(), np * 4, cudaMemcpyHostToDevice, sv->st), "active");
        SCK(cudaMemcpyAsync(sv->rr0, rr0.data(), np * 8, cudaMemcpyHostToDevice, sv->st), "inner start");
        SCK(cudaMemcpyAsync(sv->eta, eta.data(), np * 8, cudaMemcpyHostToDevice, sv->st), "inner start");
        // the inner FCG: one graph launch, its loop controlled on the device
        for (;;) {
            InnerCtl ctl;
            SCK(run_inner(sv, pc, max_iter - it, &ctl), "inner solve");
            it += ctl.it;
            if (pc != FALCON_PRECOND_NONE) rep->vcycles += ctl.it;
            if (ctl.nan) return sv->fail(FALCON_ERR_NAN_DETECTED, "solver: non-finite residual in the inner solve");
            if (ctl.stalled && pc == FALCON_PRECOND_MG_LCC && it < max_iter) {
                // the learned stage stalls: plain MG for the rest, restarted from the current iterate
                pc = FALCON_PRECOND_MG;
                ++rep->fallbacks;
                continue;
            }
            break;   // done, stalled (the refinement restarts from the FP64 residual) or out of iterations
        }
        // x += d' sr / sA (inactive problems: d' = 0)
        k_ir_accum<<<g, tpb(d), 0, sv->st>>>(d, sv->x2, sv->ir_par + np, sv->bprob, sv->x);
        SCK(cudaGetLastError(), "refine");
    }
    cudaEventRecord(t1, sv->st);
    SCK(cudaEventSynchronize(t1), "solve");
    float ms = 0;
    cudaEventElapsedTime(&ms, t0, t1);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    double worst = 0;
    bool done = true;
    for (int q = 0; q < np; ++q) {
        worst = std::max(worst, rel[q]);
        if (state[q] != 1) done = false;
    }
    rep->iterations = it;
    rep->refinements = std::max(0, passes - 1);
    rep->converged = done ? 1 : 0;
    rep->rel_residual = worst;
    rep->ms = ms;
    if (!done) {
        char buf[256];
        snprintf(buf, sizeof buf,
                 "not converged: FP64 relative residual %.3e above tol %.3e (%d inner iterations, %d refinement passes%s)",
                 worst, tol, it, passes, rep->floor_residual > 0 ? "; stopped at the FP64 attainable accuracy" : "");
        sv->err = buf;
        return FALCON_ERR_NOT_CONVERGED;
    }
    return FALCON_OK;
}

int falcon_solver_solution(falcon_solver* sv, double* x) {
    if (!sv || !x) return FALCON_ERR_INVALID_ARG;
    if (!sv->st) return sv->fail(FALCON_ERR_NO_DEVICE, "solver created without a device");
    cudaSetDevice(sv->device);
    const LevelDims& d = sv->lv[0].d;
    const int nb = sv->S.nblocks;
    k_gather_pad<double><<<grid_cells(d, nb), tpb(d), 0, sv->st>>>(d, sv->x, sv->z);
    SCK(cudaMemcpyAsync(x, sv->z, (size_t)nb * d.nint * 8, cudaMemcpyDeviceToHost, sv->st), "solution");
    SCK(cudaStreamSynchronize(sv->st), "solution");
    return FALCON_OK;
}

int falcon_solver_timestep(const falcon_solver* sv, double* dt) {
    if (!sv || !dt) return FALCON_ERR_INVALID_ARG;
    *dt = sv->dt_conduction;
    return FALCON_OK;
}

int falcon_solver_set_smoothing(falcon_solver* sv, int32_t nu_pre, int32_t nu_post, int32_t nu_coarse) {
    if (!sv || nu_pre < 0 || nu_post < 0 || nu_coarse < 0 || nu_pre > 64 || nu_post > 64 || nu_coarse > 4096)
        return FALCON_ERR_INVALID_ARG;
    sv->nu_pre = nu_pre;
    sv->nu_post = nu_post;
    sv->nu_coarse = nu_coarse;
    return FALCON_OK;
}

int falcon_solver_problem_residuals(falcon_solver* sv, double* rel) {
    if (!sv || !rel) return FALCON_ERR_INVALID_ARG;
    if (!sv->st) return sv->fail(FALCON_ERR_NO_DEVICE, "solver created without a device");
    cudaSetDevice(sv->device);
    const int np = sv->S.nproblems, nb = sv->S.nblocks;
    const LevelDims& d = sv->lv[0].d;
    SCK(cudaMemsetAsync(sv->dots, 0, (size_t)6 * np * 8, sv->st), "residuals");
    SCK(halo_fill<double>(sv, 0, sv->x), "residuals");
    k_residual64<<<grid_cells(d, nb), tpb(d), 0, sv->st>>>(sv->lv[0].ops64(), d, sv->x, sv->bvec, sv->r, sv->lv[0].r,
                                                        sv->D(), 1);
    std::vector<double> rr(np), bb(np);
    SCK(cudaMemcpyAsync(rr.data(), sv->dots + 3 * np, np * 8, cudaMemcpyDeviceToHost, sv->st), "residuals");
    SCK(cudaMemcpyAsync(bb.data(), sv->dots + 4 * np, np * 8, cudaMemcpyDeviceToHost, sv->st), "residuals");
    SCK(cudaStreamSynchronize(sv->st), "residuals");
    for (int q = 0; q < np; ++q) rel[q] = bb[q] > 0 ? std::sqrt(rr[q] / bb[q]) : std::sqrt(rr[q]);
    return FALCON_OK;
}

int falcon_solver_set_rhs(falcon_solver* sv, const double* b) {
    if (!sv || !b) return FALCON_ERR_INVALID_ARG;
    std::memcpy(sv->S.b.data(), b, sv->S.b.size() * 8);
    if (sv->st) {
        cudaSetDevice(sv->device);
        SCK(cudaStreamSynchronize(sv->st), "rhs");
        SCK(cudaMemcpy(sv->bvec, b, sv->S.b.size() * 8, cudaMemcpyHostToDevice), "rhs");
    }
    return FALCON_OK;
}

int falcon_solver_coarse_shape(falcon_solver* sv, int32_t* shape) {
    if (!sv || !shape) return FALCON_ERR_INVALID_ARG;
    if (sv->st) cudaSetDevice(sv->device);
    const int rc = ensure_coarse_map(sv);
    if (rc) return rc;
    shape[0] = 2; shape[1] = sv->cD; shape[2] = sv->cH; shape[3] = sv->cW;
    return FALCON_OK;
}

int falcon_solver_attach_lcc(falcon_solver* sv, falcon_lcc* net, int32_t sweeps) {
    if (!sv || !net || sweeps < 0 || sweeps > 64) return FALCON_ERR_INVALID_ARG;
    if (sv->st) cudaSetDevice(sv->device);
    const int rc = ensure_coarse_map(sv);
    if (rc) return rc;
    sv->net = net;
    sv->clear_graphs();
    sv->net_sweeps = sweeps;
    // size the network's buffers for this grid now, not inside a timed solve
    SCK(lcc::forward_device(net, sv->feat, 2, sv->cD, sv->cH, sv->cW, sv->yout, sv->st), "lcc");
    SCK(cudaStreamSynchronize(sv->st), "lcc");
    return FALCON_OK;
}

int falcon_solver_record(falcon_solver* sv, double tol, int32_t max_iter, int32_t max_records, float* x, float* t,
                         int32_t* nrecords) {
    if (!sv || !x || !t || !nrecords || max_records < 1) return FALCON_ERR_INVALID_ARG;
    if (sv->st) cudaSetDevice(sv->device);
    int rc = ensure_coarse_map(sv);
    if (rc) return rc;
    const int lc = sv->S.nlevels - 1, nb = sv->S.nblocks;
    SvLevel& L = sv->lv[lc];
    const size_t per = (size_t)nb * L.d.nint;
    float* rec = nullptr;
    SCK(cudaMalloc(&rec, (size_t)max_records * per * 4), "record buffer");
    sv->rec = rec;
    sv->rec_max = max_records;
    sv->rec_n = 0;
    falcon_solve_report rep;
    rc = falcon_solver_solve(sv, tol, max_iter, FALCON_PRECOND_MG, &rep);
    sv->rec = nullptr;
    const int n = sv->rec_n;
    *nrecords = 0;
    if (rc == FALCON_OK || rc == FALCON_ERR_NOT_CONVERGED) {
        rc = FALCON_OK;
        const size_t vox = (size_t)2 * sv->cD * sv->cH * sv->cW;
        float* tdev = nullptr;
        cudaError_t e = cudaMalloc(&tdev, vox * 4);
        for (int q = 0; q < n && rc == FALCON_OK && e == cudaSuccess; ++q) {
            const float* rq = rec + (size_t)q * per;
            rc = coarse_solve(sv, rq);
            if (rc) break;
            const int64_t N = (int64_t)per;
            e = cudaMemsetAsync(sv->csum, 0, 8, sv->st);
            if (e != cudaSuccess) break;
            k_lcc_sumsq<<<grid_cells(L.d, nb), tpb(L.d), 0, sv->st>>>(L.d, rq, L.fAii, sv->csum);
            k_lcc_feat<<<grid_cells(L.d, nb), tpb(L.d), 0, sv->st>>>(L.d, rq, L.fAii, sv->gmap, sv->csum, N, sv->feat);
            k_lcc_target<<<grid_cells(L.d, nb), tpb(L.d), 0, sv->st>>>(L.d, sv->x, sv->gmap, sv->csum, N, tdev);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaMemcpyAsync(x + (size_t)q * vox * 8, sv->feat, vox * 8 * 4, cudaMemcpyDeviceToHost, sv->st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(t + (size_t)q * vox, tdev, vox * 4, cudaMemcpyDeviceToHost, sv->st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(sv->st);
            if (e == cudaSuccess) *nrecords = q + 1;
        }
        cudaFree(tdev);
        if (e != cudaSuccess && rc == FALCON_OK) rc = sv->fail(FALCON_ERR_CUDA, std::string("record: ") + cudaGetErrorString(e));
    }
    cudaStreamSynchronize(sv->st);
    cudaFree(rec);
    return rc;
}

}  // extern "C"
