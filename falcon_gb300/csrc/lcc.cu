// lcc.cu -- the learned coarse-correction network on the GPU: BF16 tensor-core
// forward, backward and training kernels.
//
// The network (architecture fixed in include/falcon_gb300.h, falcon_lcc_*) is
// a 4-level 3D U-Net over the coarsest multigrid level of the conduction
// solver, gathered into one dense grid per Yin-Yang panel. It replaces the
// coarsest-level smoothing of the V-cycle inside the flexible CG; the plain
// V-cycle stays the fallback. The reference has no learned component.
//
// Layout: activations channels-last [n][D][H][W][C] in BF16, C padded to a
// multiple of 16. 3x3x3 convolutions are implicit GEMMs with BF16 operands
// and FP32 accumulation: M = voxels, N = output channels, K = 27 taps x input
// channels. Two tensor-core paths (falcon_lcc_set_tensor_path):
//  - tcgen05 (the default): tcgen05.mma with the accumulator in tensor
//    memory, one elected thread issuing the MMAs, operands in shared memory;
//    the forward and backward-data kernels load a halo block once and view it
//    per tap, weight tiles and weight-gradient bricks arrive by TMA
//    (k_conv_tc, k_wgrad_tc, below);
//  - mma.sync.m16n8k16: the A fragments gathered straight from the
//    (L2-resident) activation tensor with zero padding at the grid edge, the
//    B fragments from a per-tap weight copy laid out so each fragment
//    register is one 32-bit load (k_conv, k_conv_wgrad).
// Weights have FP32 master copies updated by Adam; BF16 copies are
// regenerated after every update.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/falcon_gb300.h"
#include "lcc.h"

namespace falcon {
namespace lcc {

// layer table: input channels, output channels, relu
struct LayerSpec { int ci, co; bool relu; };
constexpr int kLayers = 10;
constexpr LayerSpec kSpec[kLayers] = {{8, 16, true},  {16, 16, true}, {16, 32, true}, {32, 32, true},
                                      {32, 64, true}, {64, 64, true}, {64, 32, true}, {32, 16, true},
                                      {16, 16, true}, {16, 1, false}};
__host__ __device__ constexpr int pad16(int c) { return (c + 15) / 16 * 16; }

struct Grid3 { int n, D, H, W; };   // samples and grid extents of one tensor
__device__ __forceinline__ int64_t nvox(const Grid3& g) { return (int64_t)g.n * g.D * g.H * g.W; }

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// grid coordinates of voxel v (computed once per row, outside the tap loop)
struct Vox { int64_t base; int d, h, w; bool ok; };   // base: first voxel of v's sample
__device__ __forceinline__ Vox decompose(const Grid3& g, int64_t v, int64_t total) {
    Vox x{0, 0, 0, 0, v >= 0 && v < total};
    if (!x.ok) return x;
    const int64_t plane = (int64_t)g.H * g.W, vol = plane * g.D;
    const int64_t s = v / vol, r = v - s * vol;
    x.base = s * vol;
    x.d = (int)(r / plane);
    const int r2 = (int)(r - (int64_t)x.d * plane);
    x.h = r2 / g.W;
    x.w = r2 - x.h * g.W;
    return x;
}
__device__ __forceinline__ int64_t shifted(const Grid3& g, const Vox& x, int dd, int dh, int dw) {
    const int d2 = x.d + dd, h2 = x.h + dh, w2 = x.w + dw;
    if (!x.ok || d2 < 0 || d2 >= g.D || h2 < 0 || h2 >= g.H || w2 < 0 || w2 >= g.W) return -1;
    return x.base + ((int64_t)d2 * g.H + h2) * g.W + w2;
}

// neighbour of voxel v at tap offset (dd, dh, dw) in {-1,0,1}^3, -1 if outside
__device__ __forceinline__ int64_t neighbour(const Grid3& g, int64_t v, int dd, int dh, int dw) {
    if (v < 0) return -1;
    const int64_t plane = (int64_t)g.H * g.W, vol = plane * g.D;
    const int64_t s = v / vol, r = v - s * vol;
    const int d = (int)(r / plane), h = (int)((r / g.W) % g.H), w = (int)(r % g.W);
    const int d2 = d + dd, h2 = h + dh, w2 = w + dw;
    if (d2 < 0 || d2 >= g.D || h2 < 0 || h2 >= g.H || w2 < 0 || w2 >= g.W) return -1;
    return s * vol + ((int64_t)d2 * g.H + h2) * g.W + w2;
}

// ---------------------------------------------------------------------------
// Implicit-GEMM 3x3x3 convolution. KC: channels of the gathered operand (a
// multiple of 16), NC: output channels (a multiple of 16).
// MODE 0: forward, out = bf16(relu?(acc + bias)), taps at +offset
// MODE 1: forward of the last layer, out32[v] = acc(channel 0) + bias[0]
// MODE 2: backward data, out32[v][c] = acc, taps at -offset
// w: [27][NC][KC] BF16 (for MODE 2 the caller passes the transposed copy).
// 4 warps, each 16 voxels x NC channels; a CTA covers 64 voxels.
template <int KC, int NC, int MODE>
__global__ void __launch_bounds__(128) k_conv(const __nv_bfloat16* __restrict__ x, Grid3 g,
                                              const __nv_bfloat16* __restrict__ w, const float* __restrict__ bias,
                                              int relu, __nv_bfloat16* __restrict__ out16, float* __restrict__ out32) {
    constexpr int NT = NC / 8;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gid = lane >> 2, tig = lane & 3;
    const int64_t total = nvox(g);
    const int64_t vbase = ((int64_t)blockIdx.x * 4 + warp) * 16;
    const int64_t v0 = vbase + gid, v1 = vbase + gid + 8;
    float acc[NT][4];
#pragma unroll
    for (int j = 0; j < NT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    const Vox x0 = decompose(g, v0, total), x1 = decompose(g, v1, total);
    for (int tap = 0; tap < 27; ++tap) {
        const int sgn = MODE == 2 ? -1 : 1;
        const int dd = sgn * (tap / 9 - 1), dh = sgn * ((tap / 3) % 3 - 1), dw = sgn * (tap % 3 - 1);
        const int64_t n0 = shifted(g, x0, dd, dh, dw);
        const int64_t n1 = shifted(g, x1, dd, dh, dw);
        const __nv_bfloat16* wt = w + (size_t)tap * NC * KC;
#pragma unroll
        for (int kc = 0; kc < KC; kc += 16) {
            uint32_t a[4];
            const int c = kc + tig * 2;
            a[0] = n0 >= 0 ? ld32(x + n0 * KC + c) : 0u;
            a[1] = n1 >= 0 ? ld32(x + n1 * KC + c) : 0u;
            a[2] = n0 >= 0 ? ld32(x + n0 * KC + c + 8) : 0u;
            a[3] = n1 >= 0 ? ld32(x + n1 * KC + c + 8) : 0u;
#pragma unroll
            for (int j = 0; j < NT; ++j) {
                const __nv_bfloat16* wr = wt + (size_t)(j * 8 + gid) * KC + c;
                mma_bf16(acc[j], a, ld32(wr), ld32(wr + 8));
            }
        }
    }
#pragma unroll
    for (int j = 0; j < NT; ++j) {
        const int co = j * 8 + tig * 2;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const int64_t v = half ? v1 : v0;
            if (v >= total) continue;
            float y0 = acc[j][2 * half], y1 = acc[j][2 * half + 1];
            if (MODE == 0) {
                y0 += bias[co];
                y1 += bias[co + 1];
                if (relu) { y0 = fmaxf(y0, 0.f); y1 = fmaxf(y1, 0.f); }
                __nv_bfloat162 p;
                p.x = __float2bfloat16_rn(y0);
                p.y = __float2bfloat16_rn(y1);
                *reinterpret_cast<__nv_bfloat162*>(out16 + v * NC + co) = p;
            } else if (MODE == 1) {
                if (co == 0) out32[v] = y0 + bias[0];
            } else {
                out32[v * NC + co] = y0;
                out32[v * NC + co + 1] = y1;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// The same convolutions on the 5th-generation tensor cores: tcgen05.mma
// (kind::f16, BF16 operands, FP32 accumulation in tensor memory), with TMA
// tensor copies (cp.async.bulk.tensor) feeding a ring of shared-memory stages.
//
// Roles in a CTA of 128 threads: lane 0 of warp 0 issues the copies, lane 0 of
// warp 1 waits for each stage, issues its MMAs and commits them to the
// stage's `empty` barrier (which frees the stage for the next copy); the
// other lanes of those two warps wait at __syncwarp, so no polling lane
// shares a warp with a role lane. All four warps then read the accumulator
// (warp w: TMEM lanes 32w..32w+31) for the epilogue.
//
// Forward and backward data (k_conv_tc): the CTA's 128 voxels are one row
// block; its halo is loaded once and every tap's A operand is a view of it
// (see the kernel); only the tap's weight tile [N][K] is copied per tap.
// Weight gradient (k_wgrad_tc): K runs over voxel bricks of 4 x 4 x 8; per
// brick two 5-D box copies of [n][D][H][W][C] (gy, and x shifted by the tap;
// the copy engine fills voxels outside the grid with zeros, the
// convolution's padding). Copied rows are one voxel's C channels, C x 2 bytes
// = the swizzle span (32, 64 or 128 B), so the copies write exactly the
// canonical swizzled layouts that the MMA descriptors name.
// Every wait is bounded; one that runs out sets *err, the CTA waits (bounded)
// for its copies in flight, frees its tensor memory and discards its tile.
namespace tc {
constexpr int kStages = 4;                          // ring depth of the weight-gradient tiles
constexpr int kConvStages = 8;                      // ring depth of the convolutions' weight tiles
constexpr int kBW = 8, kBH = 4, kBD = 4;            // voxel brick (w, h, d) of a weight-gradient tile
constexpr int kRowW = 8, kRowH = 16;                // row block (w, h; one d) of a convolution tile
constexpr int kPolls = 1 << 22;
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
// UMMA layout code of a swizzle span (bytes): 32 -> 6, 64 -> 4, 128 -> 2
__host__ __device__ constexpr uint32_t umma_layout(int span) { return span == 32 ? 6u : span == 64 ? 4u : 2u; }
// shared-memory matrix descriptor: start, LBO, SBO (>> 4), version 1, layout
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo, uint32_t layout) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46) | ((uint64_t)layout << 61);
}
// instruction descriptor, kind::f16: D F32, A and B BF16, majors (0 K, 1 MN), N, M
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N, int a_mn, int b_mn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)a_mn << 15) | ((uint32_t)b_mn << 16) |
           ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mbar_init(uint64_t* b) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
// polls: the caller's limit (the network's wait limit, or kPolls for the
// drains after a wait ran out)
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, int polls = kPolls) {
    for (int it = 0; it < polls; ++it) {
        uint32_t ok;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(ok)
                     : "r"(smem_u32(b)), "r"(parity)
                     : "memory");
        if (ok) return true;
    }
    return false;
}
__device__ __forceinline__ void tma_5d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2, int c3,
                                       int c4) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5, %6, "
        "%7}], [%2];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4)
        : "memory");
}
__device__ __forceinline__ void tma_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            smem_u32(dst)),
        "l"(map), "r"(smem_u32(bar)), "r"(c0), "r"(c1)
        : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void commit(uint64_t* b) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(b))
                 : "memory");
}
__device__ __forceinline__ void ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}
__host__ __device__ constexpr uint32_t up1024(uint32_t b) { return (b + 1023u) / 1024u * 1024u; }

// tensor memory of the tile (warp 0), barriers (thread 0); all threads synced
template <int NCOLS, int STAGES>
__device__ __forceinline__ uint32_t tile_setup(uint64_t* bars, uint32_t* slot) {
    const int tid = threadIdx.x;
    if (tid == 0) {
        for (int q = 0; q < 2 * STAGES + 1; ++q) mbar_init(&bars[q]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    if ((tid >> 5) == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"(NCOLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    return *slot;
}
template <int NCOLS>
__device__ __forceinline__ void tile_release(uint32_t tmem) {
    fence_before();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NCOLS) : "memory");
    }
}
// after a wait ran out somewhere: thread 0 waits (bounded) for the copies it
// issued into the last STAGES stages, so none lands after the CTA exits
template <int STAGES>
__device__ __forceinline__ void drain_copies(uint64_t* full, int issued) {
    for (int t = issued - STAGES < 0 ? 0 : issued - STAGES; t < issued; ++t)
        mbar_wait(&full[t % STAGES], (uint32_t)((t / STAGES) & 1));
}
// brick of tile index `t`: sample and first voxel (d0, h0, w0)
struct Brick { int s, d0, h0, w0; };
__device__ __forceinline__ Brick brick_of(const Grid3& g, int64_t t) {
    const int tw = (g.W + kBW - 1) / kBW, th = (g.H + kBH - 1) / kBH, td = (g.D + kBD - 1) / kBD;
    Brick b;
    b.w0 = (int)(t % tw) * kBW;
    t /= tw;
    b.h0 = (int)(t % th) * kBH;
    t /= th;
    b.d0 = (int)(t % td) * kBD;
    b.s = (int)(t / td);
    return b;
}
}  // namespace tc

// Forward / backward-data convolution: KC channels gathered (the K of each
// tap), NC output channels, MODE as k_conv. A CTA owns a row block of 1 x 16 x
// 8 voxels (d, h, w): M = 128, TMEM lane m = voxel (h0 + m / 8, w0 + m % 8).
// Its 3 x 18 x 10 halo is loaded once, by all threads, into shared memory in
// the no-swizzle K-major core-matrix layout: chunk c of 8 channels is a slab
// [540 halo voxels][16 B] at c x 8640 B. For tap (dd, dh, dw) the A operand
// is then a view of that slab: the 8 rows of core group j (h = j) start at
// halo voxel ((dd + 1) x 18 + j + dh + 1) x 10 + dw + 1, i.e. a fixed start
// and a group stride (SBO) of 10 voxels = 160 B; the next 8 channels are one
// slab further (LBO). No data moves between taps. The tap's weight tile
// [NC][KC] comes by TMA into a ring of kConvStages stages (swizzled K-major).
// wmap: tensor map of the weights [27 * NC][KC].
template <int KC, int NC, int MODE>
__global__ void __launch_bounds__(128) k_conv_tc(const __nv_bfloat16* __restrict__ x,
                                                 const __grid_constant__ CUtensorMap wmap, Grid3 g,
                                                 const float* __restrict__ bias, int relu,
                                                 __nv_bfloat16* __restrict__ out16, float* __restrict__ out32,
                                                 int32_t* err, int polls) {
    using namespace tc;
    constexpr int ST = kConvStages;
    constexpr int HD = 3, HH = kRowH + 2, HW = kRowW + 2, HROWS = HD * HH * HW;
    constexpr uint32_t SLAB = HROWS * 16u;                               // one chunk of 8 channels
    constexpr uint32_t SPAN = KC * 2, B_BYTES = (uint32_t)NC * SPAN, B_STRIDE = up1024(B_BYTES);
    constexpr int NCOLS = NC < 32 ? 32 : NC;
    constexpr uint32_t IDESC = idesc_bf16(128, NC, 0, 0);
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t bars[2 * ST + 1];
    __shared__ uint32_t tmem_slot;
    unsigned char* bbase = smem + ((1024u - (smem_u32(smem) & 1023u)) & 1023u);   // swizzle atoms: 1 KB aligned
    unsigned char* abase = bbase + ST * B_STRIDE;
    const int tid = threadIdx.x, warp = tid >> 5;
    uint64_t *full = bars, *empty = bars + ST, *done = bars + 2 * ST;
    // row block of this CTA
    const int tw = (g.W + kRowW - 1) / kRowW, th = (g.H + kRowH - 1) / kRowH;
    int64_t q = blockIdx.x;
    const int w0 = (int)(q % tw) * kRowW;
    q /= tw;
    const int h0 = (int)(q % th) * kRowH;
    q /= th;
    const int d0 = (int)(q % g.D), smp = (int)(q / g.D);
    const uint32_t tmem = tile_setup<NCOLS, ST>(bars, &tmem_slot);
    int late = 0, issued = 0;
    auto issue_b = [&](int t) {
        const int s = t % ST;
        mbar_expect_tx(&full[s], B_BYTES);
        tma_2d(bbase + s * B_STRIDE, &wmap, &full[s], 0, t * NC);
        issued = t + 1;
    };
    if (tid == 0)
        for (int t = 0; t < ST; ++t) issue_b(t);
    // halo: voxel (d0 - 1 + r / 180, h0 - 1 + (r / 10) % 18, w0 - 1 + r % 10), zero outside the grid
    const int64_t plane = (int64_t)g.H * g.W, sbase = (int64_t)smp * g.D * plane;
    constexpr int NITEM = HROWS * (KC / 8), UNR = 4;  // 16-B items; UNR loads in flight per thread
    for (int i0 = 0; i0 < NITEM; i0 += 128 * UNR) {
        uint4 val[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const int i = i0 + u * 128 + tid, c = i % (KC / 8), r = i / (KC / 8);
            const int d = d0 - 1 + r / (HH * HW), h = h0 - 1 + (r / HW) % HH, w = w0 - 1 + r % HW;
            val[u] = make_uint4(0u, 0u, 0u, 0u);
            if (i < NITEM && d >= 0 && d < g.D && h >= 0 && h < g.H && w >= 0 && w < g.W)
                val[u] = *reinterpret_cast<const uint4*>(x + (sbase + d * plane + (int64_t)h * g.W + w) * KC + c * 8);
        }
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const int i = i0 + u * 128 + tid;
            if (i < NITEM) *reinterpret_cast<uint4*>(abase + (i % (KC / 8)) * SLAB + (i / (KC / 8)) * 16u) = val[u];
        }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");      // the halo -> the MMA's async proxy
    __syncthreads();
    // one lane of warp 0 copies, one of warp 1 issues the MMAs; the other lanes
    // of those warps wait at __syncwarp, not in a polling loop beside them
    if (tid == 0) {                                  // weight copies of the later taps
        for (int t = ST; t < 27; ++t) {
            if (!mbar_wait(&empty[t % ST], (uint32_t)((t / ST - 1) & 1), polls)) { late = 1; break; }
            issue_b(t);
        }
    } else if (tid == 32) {                          // MMAs
        fence_after();
        const uint32_t a0 = smem_u32(abase);
        for (int t = 0; t < 27; ++t) {
            const int s = t % ST;
            if (!mbar_wait(&full[s], (uint32_t)((t / ST) & 1), polls)) { late = 1; break; }
            fence_after();
            const int sgn = MODE == 2 ? -1 : 1;
            const int dd = sgn * (t / 9 - 1), dh = sgn * ((t / 3) % 3 - 1), dw = sgn * (t % 3 - 1);
            const uint32_t at = a0 + (uint32_t)((((dd + 1) * HH + dh + 1) * HW + dw + 1) * 16);
            const uint32_t b0 = smem_u32(bbase + s * B_STRIDE);
#pragma unroll
            for (int kk = 0; kk < KC / 16; ++kk)
                mma(tmem, sdesc(at + kk * 2 * SLAB, SLAB, HW * 16u, 0u),
                    sdesc(b0 + kk * 32u, 16u, 8 * SPAN, umma_layout(SPAN)), IDESC, (t > 0 || kk > 0) ? 1u : 0u);
            commit(&empty[s]);
        }
        commit(done);                                // completes when every MMA issued above has
    }
    if (warp < 2) __syncwarp();
    // the MMAs issued complete whatever the limit: after a wait that ran out
    // they are drained with the default bound before tensor memory is read or freed
    if (!mbar_wait(done, 0u, polls)) {
        late = 1;
        mbar_wait(done, 0u);
    }
    late = __syncthreads_or(late);
    if (late && tid == 0) {
        drain_copies<ST>(full, issued);
        atomicOr(err, 1);
    }
    fence_after();
    // epilogue: warp w reads TMEM lanes 32w..32w+31; row m = tid
    const int h = h0 + tid / kRowW, w = w0 + tid % kRowW;
    const bool ok = !late && h < g.H && w < g.W;
    const int64_t v = sbase + d0 * plane + (int64_t)h * g.W + w;
#pragma unroll
    for (int c0 = 0; c0 < (MODE == 1 ? 16 : NC); c0 += 16) {
        float acc[16];
        ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, acc);
        if (!ok) continue;
        if constexpr (MODE == 0) {
#pragma unroll
            for (int k = 0; k < 16; k += 2) {
                float y0 = acc[k] + bias[c0 + k], y1 = acc[k + 1] + bias[c0 + k + 1];
                if (relu) { y0 = fmaxf(y0, 0.f); y1 = fmaxf(y1, 0.f); }
                __nv_bfloat162 p;
                p.x = __float2bfloat16_rn(y0);
                p.y = __float2bfloat16_rn(y1);
                *reinterpret_cast<__nv_bfloat162*>(out16 + v * NC + c0 + k) = p;
            }
        } else if constexpr (MODE == 1) {
            out32[v] = acc[0] + bias[0];
        } else {
#pragma unroll
            for (int k = 0; k < 16; k += 4)
                *reinterpret_cast<float4*>(out32 + v * NC + c0 + k) = make_float4(acc[k], acc[k + 1], acc[k + 2], acc[k + 3]);
        }
    }
    tile_release<NCOLS>(tmem);
}

// Weight gradient of one tap over a run of bricks: D[co][ci] (M = 128 rows,
// co < CO real; N = CI) += sum over the bricks' voxels of gy[v][co] x[v +
// off][ci]. Both tiles are [128 voxels][C] as copied, i.e. MN-major with the
// voxels as K: 8 voxel rows form a swizzle atom (SBO = 8 rows), and the 16
// voxels of one MMA are 16 rows further on. M = 128 covers CO with LBO = 0:
// the rows past CO repeat the first ones and their accumulators are unused.
// The sums of all bricks are added into dw[co][ci][tap] with FP32 atomics.
template <int CO, int CI>
__global__ void __launch_bounds__(128) k_wgrad_tc(const __grid_constant__ CUtensorMap gmap,
                                                  const __grid_constant__ CUtensorMap xmap, Grid3 g, int64_t nbricks,
                                                  int per_cta, int co_real, int ci_real, float* __restrict__ dw,
                                                  int32_t* err, int polls) {
    using namespace tc;
    constexpr uint32_t SPAN_A = CO * 2, SPAN_B = CI * 2;
    constexpr uint32_t A_BYTES = 128u * SPAN_A, B_BYTES = 128u * SPAN_B;
    constexpr uint32_t A_STRIDE = up1024(A_BYTES), B_STRIDE = up1024(B_BYTES);
    constexpr int NCOLS = CI < 32 ? 32 : CI;
    constexpr uint32_t IDESC = idesc_bf16(128, CI, 1, 1);
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t bars[2 * kStages + 1];
    __shared__ uint32_t tmem_slot;
    unsigned char* abase = smem + ((1024u - (smem_u32(smem) & 1023u)) & 1023u);   // swizzle atoms: 1 KB aligned
    unsigned char* bbase = abase + kStages * A_STRIDE;
    const int tid = threadIdx.x, warp = tid >> 5;
    uint64_t *full = bars, *empty = bars + kStages, *done = bars + 2 * kStages;
    const int tap = blockIdx.y;
    const int dd = tap / 9 - 1, dh = (tap / 3) % 3 - 1, dwo = tap % 3 - 1;
    const int64_t b0 = (int64_t)blockIdx.x * per_cta;
    const int nb = (int)((nbricks - b0) < per_cta ? (nbricks - b0) : per_cta);
    const uint32_t tmem = tile_setup<NCOLS, kStages>(bars, &tmem_slot);
    int late = 0, issued = 0;
    if (tid == 0) {
        for (int t = 0; t < nb; ++t) {
            const int s = t % kStages;
            if (t >= kStages && !mbar_wait(&empty[s], (uint32_t)((t / kStages - 1) & 1), polls)) { late = 1; break; }
            const Brick bk = brick_of(g, b0 + t);
            mbar_expect_tx(&full[s], A_BYTES + B_BYTES);
            tma_5d(abase + s * A_STRIDE, &gmap, &full[s], 0, bk.w0, bk.h0, bk.d0, bk.s);
            tma_5d(bbase + s * B_STRIDE, &xmap, &full[s], 0, bk.w0 + dwo, bk.h0 + dh, bk.d0 + dd, bk.s);
            issued = t + 1;
        }
    } else if (tid == 32) {
        for (int t = 0; t < nb; ++t) {
            const int s = t % kStages;
            if (!mbar_wait(&full[s], (uint32_t)((t / kStages) & 1), polls)) { late = 1; break; }
            fence_after();
            const uint32_t a0 = smem_u32(abase + s * A_STRIDE), bb = smem_u32(bbase + s * B_STRIDE);
#pragma unroll
            for (int kk = 0; kk < 8; ++kk)
                mma(tmem, sdesc(a0 + kk * 16u * SPAN_A, 0u, 8 * SPAN_A, umma_layout(SPAN_A)),
                    sdesc(bb + kk * 16u * SPAN_B, 0u, 8 * SPAN_B, umma_layout(SPAN_B)), IDESC,
                    (t > 0 || kk > 0) ? 1u : 0u);
            commit(&empty[s]);
        }
        commit(done);
    }
    if (warp < 2) __syncwarp();                      // the role lanes' warps reconverge before polling
    // the MMAs issued complete whatever the limit: after a wait that ran out
    // they are drained with the default bound before tensor memory is read or freed
    if (!mbar_wait(done, 0u, polls)) {
        late = 1;
        mbar_wait(done, 0u);
    }
    late = __syncthreads_or(late);
    if (late && tid == 0) {
        drain_copies<kStages>(full, issued);
        atomicOr(err, 1);
    }
    fence_after();
    if (warp * 32 < CO && nb > 0) {                  // warp-uniform: TMEM lanes 32w.. hold co = 32w..
        const int co = tid;
#pragma unroll
        for (int c0 = 0; c0 < CI; c0 += 16) {
            float acc[16];
            ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, acc);
            if (late || co >= co_real) continue;
#pragma unroll
            for (int q = 0; q < 16; ++q)
                if (c0 + q < ci_real) atomicAdd(&dw[((size_t)co * ci_real + c0 + q) * 27 + tap], acc[q]);
        }
    }
    tile_release<NCOLS>(tmem);
}

// Backward weights: dw[co][ci][tap] += sum_v gy[v][co] * x[v + off(tap)][ci].
// One CTA per (chunk of `chunk` voxels, tap); warp = (m-tile of 16 output
// channels, share of the chunk). CO, CI: padded output and input channels
// (16, 32 or 64). gy: [v][CO] BF16, x: [v][CI] BF16.
template <int CO, int CI>
__global__ void __launch_bounds__(128) k_conv_wgrad(const __nv_bfloat16* __restrict__ gy, const __nv_bfloat16* __restrict__ x,
                                                    Grid3 g, int chunk, int co_real, int ci_real, float* __restrict__ dw) {
    constexpr int MT = (CO + 15) / 16;          // m-tiles of output channels
    constexpr int PARTS = 4 / MT > 0 ? 4 / MT : 1;
    constexpr int NT = CI / 8;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp >= MT * PARTS) return;
    const int gid = lane >> 2, tig = lane & 3;
    const int mt = warp % MT, part = warp / MT;
    const int tap = blockIdx.y;
    const int dd = tap / 9 - 1, dh = (tap / 3) % 3 - 1, dw_ = tap % 3 - 1;
    const int64_t total = nvox(g);
    const int64_t c0 = (int64_t)blockIdx.x * chunk;
    const int64_t c1 = c0 + chunk < total ? c0 + chunk : total;
    const int per = (chunk / PARTS + 15) / 16 * 16;
    const int64_t k0 = c0 + (int64_t)part * per;
    const int64_t k1 = k0 + per < c1 ? k0 + per : c1;
    float acc[NT][4];
#pragma unroll
    for (int j = 0; j < NT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    const int r0 = mt * 16 + gid, r1 = r0 + 8;   // output channels of this thread's A rows
    for (int64_t kb = k0; kb < k1; kb += 16) {
        // A[m = co][k = v] = gy[v][co]; this thread: k = kb + tig*2 + {0,1} and + 8
        uint32_t a[4];
        __nv_bfloat16 e[8];
        const int64_t kv[4] = {kb + tig * 2, kb + tig * 2 + 1, kb + tig * 2 + 8, kb + tig * 2 + 9};
        const __nv_bfloat16 z = __float2bfloat16_rn(0.f);
        // a0,a1: row r0, k = tig*2, +1; a2,a3: row r1, same k; a4,a5: row r0, k+8; a6,a7: row r1, k+8
        auto G = [&](int row, int64_t v) -> __nv_bfloat16 {
            return (row < co_real && v < k1) ? gy[v * CO + row] : z;
        };
        e[0] = G(r0, kv[0]); e[1] = G(r0, kv[1]);
        e[2] = G(r1, kv[0]); e[3] = G(r1, kv[1]);
        e[4] = G(r0, kv[2]); e[5] = G(r0, kv[3]);
        e[6] = G(r1, kv[2]); e[7] = G(r1, kv[3]);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            __nv_bfloat162 p;
            p.x = e[2 * q];
            p.y = e[2 * q + 1];
            a[q] = *reinterpret_cast<uint32_t*>(&p);
        }
        // B[k = v][n = ci] = x[v + off][ci]; b0,b1: k = tig*2, +1; b2,b3: k + 8, + 9; n = gid
        int64_t nb[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) nb[q] = kv[q] < k1 ? neighbour(g, kv[q], dd, dh, dw_) : -1;
#pragma unroll
        for (int j = 0; j < NT; ++j) {
            const int ci = j * 8 + gid;
            __nv_bfloat162 p0, p1;
            p0.x = (nb[0] >= 0 && ci < ci_real) ? x[nb[0] * CI + ci] : z;
            p0.y = (nb[1] >= 0 && ci < ci_real) ? x[nb[1] * CI + ci] : z;
            p1.x = (nb[2] >= 0 && ci < ci_real) ? x[nb[2] * CI + ci] : z;
            p1.y = (nb[3] >= 0 && ci < ci_real) ? x[nb[3] * CI + ci] : z;
            mma_bf16(acc[j], a, *reinterpret_cast<uint32_t*>(&p0), *reinterpret_cast<uint32_t*>(&p1));
        }
    }
    // acc[j]: rows (co) r0 / r1, cols (ci) j*8 + tig*2 + {0,1}
#pragma unroll
    for (int j = 0; j < NT; ++j) {
        const int ci = j * 8 + tig * 2;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int co = q < 2 ? r0 : r1;
            const int cc = ci + (q & 1);
            if (co < co_real && cc < ci_real) atomicAdd(&dw[((size_t)co * ci_real + cc) * 27 + tap], acc[j][q]);
        }
    }
}

// ---- elementwise kernels -----------------------------------------------------
#define GRID_STRIDE(i, n) for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

// fp32 [v][8] features -> bf16 [v][16] (channels 8..15 zero)
__global__ void k_prep_input(const float* __restrict__ x, int64_t nv, __nv_bfloat16* __restrict__ out) {
    GRID_STRIDE(i, nv * 16) {
        const int64_t v = i >> 4;
        const int c = (int)(i & 15);
        out[i] = __float2bfloat16_rn(c < 8 ? x[v * 8 + c] : 0.f);
    }
}

// 2x2x2 average pool (grid g is the fine grid), C channels
__global__ void k_pool(const __nv_bfloat16* __restrict__ x, Grid3 g, int C, __nv_bfloat16* __restrict__ out) {
    const int D2 = g.D / 2, H2 = g.H / 2, W2 = g.W / 2;
    const int64_t n = (int64_t)g.n * D2 * H2 * W2 * C;
    GRID_STRIDE(i, n) {
        const int c = (int)(i % C);
        int64_t v = i / C;
        const int w = (int)(v % W2); v /= W2;
        const int h = (int)(v % H2); v /= H2;
        const int d = (int)(v % D2);
        const int64_t s = v / D2;
        float acc = 0.f;
        for (int q = 0; q < 8; ++q) {
            const int64_t f = ((s * g.D + 2 * d + (q >> 2)) * g.H + 2 * h + ((q >> 1) & 1)) * g.W + 2 * w + (q & 1);
            acc += __bfloat162float(x[f * C + c]);
        }
        out[i] = __float2bfloat16_rn(acc * 0.125f);
    }
}

// out = bf16(up2(a) + skip); g is the fine grid
__global__ void k_up_add(const __nv_bfloat16* __restrict__ a, const __nv_bfloat16* __restrict__ skip, Grid3 g, int C,
                         __nv_bfloat16* __restrict__ out) {
    const int64_t n = nvox(g) * C;
    GRID_STRIDE(i, n) {
        const int c = (int)(i % C);
        int64_t v = i / C;
        const int w = (int)(v % g.W); v /= g.W;
        const int h = (int)(v % g.H); v /= g.H;
        const int d = (int)(v % g.D);
        const int64_t s = v / g.D;
        const int64_t cv = ((s * (g.D / 2) + d / 2) * (g.H / 2) + h / 2) * (g.W / 2) + w / 2;
        out[i] = __float2bfloat16_rn(__bfloat162float(a[cv * C + c]) + __bfloat162float(skip[i]));
    }
}

// G = bf16(dy * (y > 0)) for relu layers, bf16(dy) otherwise; channels C of
// the padded layout (padded channels carry zeros)
__global__ void k_relu_grad(const float* __restrict__ dy, const __nv_bfloat16* __restrict__ y, int64_t n, int relu,
                            __nv_bfloat16* __restrict__ g) {
    GRID_STRIDE(i, n) {
        float v = dy[i];
        if (relu && !(__bfloat162float(y[i]) > 0.f)) v = 0.f;
        g[i] = __float2bfloat16_rn(v);
    }
}

// out[fine] = g[coarse] / 8 + skip[fine] (pool backward plus the skip gradient)
__global__ void k_pool_back_add(const float* __restrict__ gc, const float* __restrict__ skip, Grid3 g, int C,
                                float* __restrict__ out) {
    const int64_t n = nvox(g) * C;
    GRID_STRIDE(i, n) {
        const int c = (int)(i % C);
        int64_t v = i / C;
        const int w = (int)(v % g.W); v /= g.W;
        const int h = (int)(v % g.H); v /= g.H;
        const int d = (int)(v % g.D);
        const int64_t s = v / g.D;
        const int64_t cv = ((s * (g.D / 2) + d / 2) * (g.H / 2) + h / 2) * (g.W / 2) + w / 2;
        out[i] = gc[cv * C + c] * 0.125f + (skip ? skip[i] : 0.f);
    }
}

// out[coarse] = sum of the 8 fine children (up backward); g is the fine grid
__global__ void k_up_back(const float* __restrict__ gf, Grid3 g, int C, float* __restrict__ out) {
    const int D2 = g.D / 2, H2 = g.H / 2, W2 = g.W / 2;
    const int64_t n = (int64_t)g.n * D2 * H2 * W2 * C;
    GRID_STRIDE(i, n) {
        const int c = (int)(i % C);
        int64_t v = i / C;
        const int w = (int)(v % W2); v /= W2;
        const int h = (int)(v % H2); v /= H2;
        const int d = (int)(v % D2);
        const int64_t s = v / D2;
        float acc = 0.f;
        for (int q = 0; q < 8; ++q) {
            const int64_t f = ((s * g.D + 2 * d + (q >> 2)) * g.H + 2 * h + ((q >> 1) & 1)) * g.W + 2 * w + (q & 1);
            acc += gf[f * C + c];
        }
        out[i] = acc;
    }
}

// bias gradient: db[c] += sum_v g[v][c], c < creal
__global__ void k_bias_grad(const __nv_bfloat16* __restrict__ g, int64_t nv, int C, int creal, float* __restrict__ db) {
    __shared__ float red[64];
    for (int c = threadIdx.x; c < 64; c += blockDim.x) red[c] = 0.f;
    __syncthreads();
    GRID_STRIDE(i, nv * C) {
        const int c = (int)(i % C);
        if (c < creal) atomicAdd(&red[c], __bfloat162float(g[i]));
    }
    __syncthreads();
    for (int c = threadIdx.x; c < creal; c += blockDim.x) atomicAdd(&db[c], red[c]);
}

// loss += sum (y - t)^2; dy = 2 (y - t) / count, written into the [v][16]
// layout of the last layer (channel 0; the padded channels get 0)
__global__ void k_mse(const float* __restrict__ y, const float* __restrict__ t, int64_t nv, float inv_count,
                      float* __restrict__ dy16, double* __restrict__ loss) {
    double local = 0.0;
    GRID_STRIDE(v, nv) {
        const float d = y[v] - t[v];
        local += (double)d * d;
        dy16[v * 16] = 2.f * d * inv_count;
        for (int c = 1; c < 16; ++c) dy16[v * 16 + c] = 0.f;
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, local);
}

// Adam (Kingma & Ba 2015) on the FP32 master parameters
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ gr, float* __restrict__ m, float* __restrict__ v,
                       int64_t n, float lr, float b1, float b2, float c1, float c2, float eps) {
    GRID_STRIDE(i, n) {
        const float gi = gr[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    }
}

// master W[co][ci][27] -> forward copy wf[27][COp][CIp] and backward-data copy
// wb[27][CIp][COp] (the roles of the channel axes swapped), zero padded
__global__ void k_weights_bf16(const float* __restrict__ wm, int ci, int co, int cip, int cop,
                               __nv_bfloat16* __restrict__ wf, __nv_bfloat16* __restrict__ wb) {
    const int64_t n = (int64_t)27 * cop * cip;
    GRID_STRIDE(i, n) {
        const int c_in = (int)(i % cip);
        const int c_out = (int)((i / cip) % cop);
        const int tap = (int)(i / ((int64_t)cip * cop));
        const float val = (c_in < ci && c_out < co) ? wm[((size_t)c_out * ci + c_in) * 27 + tap] : 0.f;
        const __nv_bfloat16 b = __float2bfloat16_rn(val);
        wf[i] = b;
        wb[((size_t)tap * cip + c_in) * cop + c_out] = b;
    }
}

#undef GRID_STRIDE

// ---- launch helpers ----------------------------------------------------------
inline unsigned ew_grid(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16)); }

// cuTensorMapEncodeTiled, through the runtime's driver entry point
inline PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}
inline CUtensorMapSwizzle swizzle_of(int span) {
    return span == 32 ? CU_TENSOR_MAP_SWIZZLE_32B : span == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B;
}
// activations [n][D][H][W][C] BF16, copied as bricks of C x 8 x 4 x 4 x 1
// (out-of-range voxels read as zeros); rows of C x 2 bytes, swizzled to match
inline cudaError_t act_map(CUtensorMap* m, const __nv_bfloat16* x, Grid3 g, int C) {
    const auto fn = encode_tiled();
    if (!fn) return cudaErrorNotSupported;
    const cuuint64_t row = (cuuint64_t)C * 2;
    const cuuint64_t dims[5] = {(cuuint64_t)C, (cuuint64_t)g.W, (cuuint64_t)g.H, (cuuint64_t)g.D, (cuuint64_t)g.n};
    const cuuint64_t strides[4] = {row, row * g.W, row * g.W * g.H, row * g.W * g.H * g.D};
    const cuuint32_t box[5] = {(cuuint32_t)C, tc::kBW, tc::kBH, tc::kBD, 1};
    const cuuint32_t es[5] = {1, 1, 1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<__nv_bfloat16*>(x), dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_of(C * 2), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS
               ? cudaSuccess
               : cudaErrorInvalidValue;
}
// weights [27 * N][K] BF16, copied one tap (N rows of K) at a time
inline cudaError_t weight_map(CUtensorMap* m, const __nv_bfloat16* w, int K, int N) {
    const auto fn = encode_tiled();
    if (!fn) return cudaErrorNotSupported;
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)27 * N};
    const cuuint64_t strides[1] = {(cuuint64_t)K * 2};
    const cuuint32_t box[2] = {(cuuint32_t)K, (cuuint32_t)N};
    const cuuint32_t es[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(w), dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_of(K * 2), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS
               ? cudaSuccess
               : cudaErrorInvalidValue;
}
inline int64_t bricks(Grid3 g) {
    return (int64_t)g.n * ((g.D + tc::kBD - 1) / tc::kBD) * ((g.H + tc::kBH - 1) / tc::kBH) *
           ((g.W + tc::kBW - 1) / tc::kBW);
}
// dynamic shared memory of a ring with A and B tiles (plus 1 KB to align it)
constexpr uint32_t ring_bytes(uint32_t a, uint32_t b) { return tc::kStages * (tc::up1024(a) + tc::up1024(b)) + 1024u; }

template <int K, int N, int MODE>
cudaError_t conv_tc_launch(const __nv_bfloat16* x, Grid3 g, const __nv_bfloat16* w, const float* bias, int relu,
                           __nv_bfloat16* out16, float* out32, int32_t* err, int polls, cudaStream_t st) {
    // the weight ring, then the halo (3 x 18 x 10 voxels of K channels)
    constexpr uint32_t smem = tc::kConvStages * tc::up1024((uint32_t)N * K * 2) + 3u * (tc::kRowH + 2) * (tc::kRowW + 2) * K * 2 + 1024u;
    CUtensorMap wm;
    cudaError_t e = weight_map(&wm, w, K, N);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_conv_tc<K, N, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t blocks = (int64_t)g.n * g.D * ((g.H + tc::kRowH - 1) / tc::kRowH) * ((g.W + tc::kRowW - 1) / tc::kRowW);
    k_conv_tc<K, N, MODE><<<(unsigned)blocks, 128, smem, st>>>(x, wm, g, bias, relu, out16, out32, err, polls);
    return cudaGetLastError();
}

template <int CO, int CI>
cudaError_t wgrad_tc_launch(const __nv_bfloat16* gy, const __nv_bfloat16* x, Grid3 g, int co_real, int ci_real,
                            float* dw, int32_t* err, int polls, cudaStream_t st) {
    constexpr uint32_t smem = ring_bytes(128u * CO * 2, 128u * CI * 2);
    CUtensorMap gm, xm;
    cudaError_t e = act_map(&gm, gy, g, CO);
    if (e == cudaSuccess) e = act_map(&xm, x, g, CI);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_wgrad_tc<CO, CI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t nb = bricks(g);
    const int per = (int)std::max<int64_t>(1, std::min<int64_t>(16, nb / 64));   // bricks (K = 128 each) per CTA
    const dim3 grid((unsigned)((nb + per - 1) / per), 27);
    k_wgrad_tc<CO, CI><<<grid, 128, smem, st>>>(gm, xm, g, nb, per, co_real, ci_real, dw, err, polls);
    return cudaGetLastError();
}

// tc: the tcgen05 kernel (else mma.sync); err: its wait-timeout flag
template <int MODE>
cudaError_t conv_launch(int kc, int nc, const __nv_bfloat16* x, Grid3 g, const __nv_bfloat16* w, const float* bias,
                        int relu, __nv_bfloat16* out16, float* out32, cudaStream_t st, bool tc = false,
                        int32_t* err = nullptr, int polls = tc::kPolls) {
    const int64_t nv = (int64_t)g.n * g.D * g.H * g.W;
    const unsigned blocks = (unsigned)((nv + 63) / 64);
#define LCC_CONV(K, N)                                                                                   \
    if (kc == K && nc == N) {                                                                            \
        if (tc) return conv_tc_launch<K, N, MODE>(x, g, w, bias, relu, out16, out32, err, polls, st);    \
        k_conv<K, N, MODE><<<blocks, 128, 0, st>>>(x, g, w, bias, relu, out16, out32);                   \
        return cudaGetLastError();                                                                       \
    }
    LCC_CONV(16, 16) LCC_CONV(16, 32) LCC_CONV(16, 64) LCC_CONV(32, 16) LCC_CONV(32, 32) LCC_CONV(32, 64)
    LCC_CONV(64, 16) LCC_CONV(64, 32) LCC_CONV(64, 64)
#undef LCC_CONV
    return cudaErrorInvalidValue;
}

inline cudaError_t wgrad_launch(int co, int ci, const __nv_bfloat16* gy, const __nv_bfloat16* x, Grid3 g, int co_real,
                                int ci_real, float* dw, cudaStream_t st, bool tc = false, int32_t* err = nullptr,
                                int polls = tc::kPolls) {
    const int64_t nv = (int64_t)g.n * g.D * g.H * g.W;
    const int chunk = 512;
    const dim3 grid((unsigned)((nv + chunk - 1) / chunk), 27);
#define LCC_WG(CO, CI)                                                                                   \
    if (co == CO && ci == CI) {                                                                          \
        if (tc) return wgrad_tc_launch<CO, CI>(gy, x, g, co_real, ci_real, dw, err, polls, st);          \
        k_conv_wgrad<CO, CI><<<grid, 128, 0, st>>>(gy, x, g, chunk, co_real, ci_real, dw);               \
        return cudaGetLastError();                                                                       \
    }
    LCC_WG(16, 16) LCC_WG(16, 32) LCC_WG(16, 64) LCC_WG(32, 16) LCC_WG(32, 32) LCC_WG(32, 64)
    LCC_WG(64, 16) LCC_WG(64, 32) LCC_WG(64, 64)
#undef LCC_WG
    return cudaErrorInvalidValue;
}

}  // namespace lcc
}  // namespace falcon

using namespace falcon;
using namespace falcon::lcc;

typedef __nv_bfloat16 bf16;

struct falcon_lcc {
    int device = 0;
    cudaStream_t st = nullptr;
    std::string err;
    std::vector<void*> allocs;        // parameters (live as long as the network)
    std::vector<void*> act_allocs;    // activation buffers of the current shape
    int64_t nparam = 0;
    float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
    int64_t woff[kLayers] = {}, boff[kLayers] = {};
    bf16 *wf[kLayers] = {}, *wb[kLayers] = {};
    int64_t adam_t = 0;
    Grid3 shape{0, 0, 0, 0};
    bool use_tc = true;               // convolutions on tcgen05 (else mma.sync)
    int32_t* dflag = nullptr;         // device: a tcgen05 kernel's wait ran out
    int polls = tc::kPolls;           // the tcgen05 kernels' wait limit
    struct Acts {
        bf16 *x0, *a1, *s0, *p0, *a2, *s1, *p1, *s2, *p2, *a5, *u2, *a6, *u1, *a7, *u0, *a8, *gb;
        float *y, *xin, *t;
        float *dy9, *d_a8, *d_u0, *d_a7, *d_u1, *d_a6, *d_u2, *d_a5, *d_p2, *d_s2, *d_p1, *d_s1, *d_a2, *d_p0, *d_s0, *d_a1;
        double* loss;
    } A{};
    int fail(int c, const std::string& s) { err = s; return c; }
    template <class P> cudaError_t alloc(P** ptr, size_t bytes, std::vector<void*>& list) {
        cudaError_t e = cudaMalloc((void**)ptr, bytes ? bytes : 16);
        if (e == cudaSuccess) { list.push_back(*ptr); e = cudaMemsetAsync(*ptr, 0, bytes ? bytes : 16, st); }
        return e;
    }
};

namespace {

#define LCK(call, where)                                                                             \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return net->fail(FALCON_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e_)); \
    } while (0)

cudaError_t refresh_weights(falcon_lcc* net) {
    for (int l = 0; l < kLayers; ++l) {
        const int ci = kSpec[l].ci, co = kSpec[l].co;
        k_weights_bf16<<<ew_grid((int64_t)27 * pad16(ci) * pad16(co)), 256, 0, net->st>>>(
            net->p + net->woff[l], ci, co, pad16(ci), pad16(co), net->wf[l], net->wb[l]);
    }
    return cudaGetLastError();
}

// (re)allocate the activation buffers for n samples of D x H x W
cudaError_t ensure_shape(falcon_lcc* net, int n, int D, int H, int W) {
    const Grid3 s{n, D, H, W};
    if (s.n == net->shape.n && s.D == net->shape.D && s.H == net->shape.H && s.W == net->shape.W) return cudaSuccess;
    cudaStreamSynchronize(net->st);
    for (void* q : net->act_allocs) cudaFree(q);
    net->act_allocs.clear();
    net->shape = Grid3{0, 0, 0, 0};
    const size_t V0 = (size_t)n * D * H * W, V1 = V0 / 8, V2 = V1 / 8, V3 = V2 / 8;
    auto& A = net->A;
    auto& L = net->act_allocs;
    cudaError_t e = cudaSuccess;
    auto b16 = [&](bf16** ptr, size_t n_) { if (e == cudaSuccess) e = net->alloc(ptr, n_ * 2, L); };
    auto f32 = [&](float** ptr, size_t n_) { if (e == cudaSuccess) e = net->alloc(ptr, n_ * 4, L); };
    b16(&A.x0, V0 * 16); b16(&A.a1, V0 * 16); b16(&A.s0, V0 * 16); b16(&A.p0, V1 * 16);
    b16(&A.a2, V1 * 32); b16(&A.s1, V1 * 32); b16(&A.p1, V2 * 32); b16(&A.s2, V2 * 64);
    b16(&A.p2, V3 * 64); b16(&A.a5, V3 * 64); b16(&A.u2, V2 * 64); b16(&A.a6, V2 * 32);
    b16(&A.u1, V1 * 32); b16(&A.a7, V1 * 16); b16(&A.u0, V0 * 16); b16(&A.a8, V0 * 16);
    b16(&A.gb, V0 * 16);
    f32(&A.y, V0); f32(&A.xin, V0 * 8); f32(&A.t, V0);
    f32(&A.dy9, V0 * 16); f32(&A.d_a8, V0 * 16); f32(&A.d_u0, V0 * 16); f32(&A.d_a7, V1 * 16);
    f32(&A.d_u1, V1 * 32); f32(&A.d_a6, V2 * 32); f32(&A.d_u2, V2 * 64); f32(&A.d_a5, V3 * 64);
    f32(&A.d_p2, V3 * 64); f32(&A.d_s2, V2 * 64); f32(&A.d_p1, V2 * 32); f32(&A.d_s1, V1 * 32);
    f32(&A.d_a2, V1 * 32); f32(&A.d_p0, V1 * 16); f32(&A.d_s0, V0 * 16); f32(&A.d_a1, V0 * 16);
    if (e == cudaSuccess) e = net->alloc(&A.loss, 8, L);
    if (e == cudaSuccess) net->shape = s;
    return e;
}

cudaError_t forward(falcon_lcc* net, cudaStream_t st) {
    auto& A = net->A;
    const Grid3 G0 = net->shape, G1{G0.n, G0.D / 2, G0.H / 2, G0.W / 2}, G2{G0.n, G0.D / 4, G0.H / 4, G0.W / 4},
                G3{G0.n, G0.D / 8, G0.H / 8, G0.W / 8};
    const int64_t V0 = (int64_t)G0.n * G0.D * G0.H * G0.W;
    cudaError_t e;
    k_prep_input<<<ew_grid(V0 * 16), 256, 0, st>>>(A.xin, V0, A.x0);
    auto conv = [&](int l, const bf16* x, Grid3 g, bf16* y) {
        return conv_launch<0>(pad16(kSpec[l].ci), pad16(kSpec[l].co), x, g, net->wf[l], net->p + net->boff[l],
                              kSpec[l].relu, y, nullptr, st, net->use_tc, net->dflag, net->polls);
    };
    auto pool = [&](const bf16* x, Grid3 g, int C, bf16* y) {
        k_pool<<<ew_grid((int64_t)g.n * g.D * g.H * g.W * C / 8), 256, 0, st>>>(x, g, C, y);
        return cudaGetLastError();
    };
    auto upadd = [&](const bf16* a, const bf16* skip, Grid3 g, int C, bf16* y) {
        k_up_add<<<ew_grid((int64_t)g.n * g.D * g.H * g.W * C), 256, 0, st>>>(a, skip, g, C, y);
        return cudaGetLastError();
    };
    if ((e = conv(0, A.x0, G0, A.a1)) != cudaSuccess) return e;
    if ((e = conv(1, A.a1, G0, A.s0)) != cudaSuccess) return e;
    if ((e = pool(A.s0, G0, 16, A.p0)) != cudaSuccess) return e;
    if ((e = conv(2, A.p0, G1, A.a2)) != cudaSuccess) return e;
    if ((e = conv(3, A.a2, G1, A.s1)) != cudaSuccess) return e;
    if ((e = pool(A.s1, G1, 32, A.p1)) != cudaSuccess) return e;
    if ((e = conv(4, A.p1, G2, A.s2)) != cudaSuccess) return e;
    if ((e = pool(A.s2, G2, 64, A.p2)) != cudaSuccess) return e;
    if ((e = conv(5, A.p2, G3, A.a5)) != cudaSuccess) return e;
    if ((e = upadd(A.a5, A.s2, G2, 64, A.u2)) != cudaSuccess) return e;
    if ((e = conv(6, A.u2, G2, A.a6)) != cudaSuccess) return e;
    if ((e = upadd(A.a6, A.s1, G1, 32, A.u1)) != cudaSuccess) return e;
    if ((e = conv(7, A.u1, G1, A.a7)) != cudaSuccess) return e;
    if ((e = upadd(A.a7, A.s0, G0, 16, A.u0)) != cudaSuccess) return e;
    if ((e = conv(8, A.u0, G0, A.a8)) != cudaSuccess) return e;
    return conv_launch<1>(16, 16, A.a8, G0, net->wf[9], net->p + net->boff[9], 0, nullptr, A.y, st, net->use_tc,
                          net->dflag, net->polls);
}

// loss and parameter gradients (net->g zeroed here) for targets in A.t
cudaError_t backward(falcon_lcc* net, cudaStream_t st) {
    auto& A = net->A;
    const Grid3 G0 = net->shape, G1{G0.n, G0.D / 2, G0.H / 2, G0.W / 2}, G2{G0.n, G0.D / 4, G0.H / 4, G0.W / 4},
                G3{G0.n, G0.D / 8, G0.H / 8, G0.W / 8};
    auto nv = [](Grid3 g) { return (int64_t)g.n * g.D * g.H * g.W; };
    const int64_t V0 = nv(G0);
    cudaError_t e = cudaMemsetAsync(net->g, 0, (size_t)net->nparam * 4, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(A.loss, 0, 8, st);
    if (e != cudaSuccess) return e;
    k_mse<<<ew_grid(V0), 256, 0, st>>>(A.y, A.t, V0, 1.f / (float)V0, A.dy9, A.loss);
    // one layer: mask the upstream gradient, accumulate dW and db, propagate dX
    auto back = [&](int l, const float* dy, const bf16* y, const bf16* x, Grid3 g, float* dx) -> cudaError_t {
        const int ci = kSpec[l].ci, co = kSpec[l].co, cip = pad16(ci), cop = pad16(co);
        const int64_t n = nv(g) * cop;
        k_relu_grad<<<ew_grid(n), 256, 0, st>>>(dy, y, n, kSpec[l].relu ? 1 : 0, A.gb);
        k_bias_grad<<<ew_grid(n), 256, 0, st>>>(A.gb, nv(g), cop, co, net->g + net->boff[l]);
        cudaError_t e2 =
            wgrad_launch(cop, cip, A.gb, x, g, co, ci, net->g + net->woff[l], st, net->use_tc, net->dflag, net->polls);
        if (e2 != cudaSuccess || !dx) return e2;
        return conv_launch<2>(cop, cip, A.gb, g, net->wb[l], nullptr, 0, nullptr, dx, st, net->use_tc, net->dflag,
                              net->polls);
    };
    auto upback = [&](const float* gf, Grid3 gfine, int C, float* out) {
        k_up_back<<<ew_grid(nv(gfine) * C / 8), 256, 0, st>>>(gf, gfine, C, out);
        return cudaGetLastError();
    };
    auto poolback = [&](const float* gc, const float* skip, Grid3 gfine, int C, float* out) {
        k_pool_back_add<<<ew_grid(nv(gfine) * C), 256, 0, st>>>(gc, skip, gfine, C, out);
        return cudaGetLastError();
    };
    if ((e = back(9, A.dy9, nullptr, A.a8, G0, A.d_a8)) != cudaSuccess) return e;
    if ((e = back(8, A.d_a8, A.a8, A.u0, G0, A.d_u0)) != cudaSuccess) return e;
    if ((e = upback(A.d_u0, G0, 16, A.d_a7)) != cudaSuccess) return e;
    if ((e = back(7, A.d_a7, A.a7, A.u1, G1, A.d_u1)) != cudaSuccess) return e;
    if ((e = upback(A.d_u1, G1, 32, A.d_a6)) != cudaSuccess) return e;
    if ((e = back(6, A.d_a6, A.a6, A.u2, G2, A.d_u2)) != cudaSuccess) return e;
    if ((e = upback(A.d_u2, G2, 64, A.d_a5)) != cudaSuccess) return e;
    if ((e = back(5, A.d_a5, A.a5, A.p2, G3, A.d_p2)) != cudaSuccess) return e;
    if ((e = poolback(A.d_p2, A.d_u2, G2, 64, A.d_s2)) != cudaSuccess) return e;
    if ((e = back(4, A.d_s2, A.s2, A.p1, G2, A.d_p1)) != cudaSuccess) return e;
    if ((e = poolback(A.d_p1, A.d_u1, G1, 32, A.d_s1)) != cudaSuccess) return e;
    if ((e = back(3, A.d_s1, A.s1, A.a2, G1, A.d_a2)) != cudaSuccess) return e;
    if ((e = back(2, A.d_a2, A.a2, A.p0, G1, A.d_p0)) != cudaSuccess) return e;
    if ((e = poolback(A.d_p0, A.d_u0, G0, 16, A.d_s0)) != cudaSuccess) return e;
    if ((e = back(1, A.d_s0, A.s0, A.a1, G0, A.d_a1)) != cudaSuccess) return e;
    return back(0, A.d_a1, A.a1, A.x0, G0, nullptr);
}

// a tcgen05 kernel's bounded wait that ran out (cleared when read)
int check_flag(falcon_lcc* net) {
    int32_t f = 0;
    if (cudaMemcpy(&f, net->dflag, sizeof f, cudaMemcpyDeviceToHost) != cudaSuccess)
        return net->fail(FALCON_ERR_CUDA, "lcc: flag");
    if (!f) return FALCON_OK;
    cudaMemset(net->dflag, 0, sizeof f);
    return net->fail(FALCON_ERR_TIMEOUT, "lcc: a tensor-core convolution's wait ran out; its result was discarded");
}

int check_shape(falcon_lcc* net, int n, int D, int H, int W) {
    if (n < 1 || D < 8 || H < 8 || W < 8 || D % 8 || H % 8 || W % 8)
        return net->fail(FALCON_ERR_INVALID_ARG, "lcc: need n >= 1 and D, H, W positive multiples of 8");
    if ((double)n * D * H * W * 64.0 > 9.0e18) return net->fail(FALCON_ERR_INVALID_ARG, "lcc: tensor too large");
    return FALCON_OK;
}

}  // namespace

namespace falcon {
namespace lcc {
cudaError_t forward_device(falcon_lcc* net, const float* x, int n, int D, int H, int W, float* y, cudaStream_t st) {
    cudaError_t e = ensure_shape(net, n, D, H, W);
    if (e != cudaSuccess) return e;
    const size_t V0 = (size_t)n * D * H * W;
    e = cudaMemcpyAsync(net->A.xin, x, V0 * 8 * 4, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = forward(net, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(y, net->A.y, V0 * 4, cudaMemcpyDeviceToDevice, st);
    return e;
}
}  // namespace lcc
}  // namespace falcon

extern "C" {

int falcon_lcc_create(falcon_lcc** out, int32_t device, uint64_t seed) {
    if (!out) return FALCON_ERR_INVALID_ARG;
    falcon_lcc* net = new falcon_lcc();
    *out = net;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0 || device < 0 || device >= ndev)
        return net->fail(FALCON_ERR_NO_DEVICE, "lcc: no such CUDA device");
    net->device = device;
    LCK(cudaSetDevice(device), "cudaSetDevice");
    LCK(cudaStreamCreateWithFlags(&net->st, cudaStreamNonBlocking), "stream");
    // parameter layout: per layer W[co][ci][27] then b[co]; He-normal weights
    std::vector<float> h;
    std::mt19937_64 rng(seed);
    for (int l = 0; l < kLayers; ++l) {
        const int ci = kSpec[l].ci, co = kSpec[l].co;
        std::normal_distribution<double> nd(0.0, std::sqrt(2.0 / (27.0 * ci)));
        net->woff[l] = (int64_t)h.size();
        for (int q = 0; q < co * ci * 27; ++q) h.push_back((float)nd(rng));
        net->boff[l] = (int64_t)h.size();
        for (int q = 0; q < co; ++q) h.push_back(0.f);
    }
    net->nparam = (int64_t)h.size();
    LCK(net->alloc(&net->p, h.size() * 4, net->allocs), "params");
    LCK(net->alloc(&net->g, h.size() * 4, net->allocs), "grads");
    LCK(net->alloc(&net->m, h.size() * 4, net->allocs), "adam");
    LCK(net->alloc(&net->v, h.size() * 4, net->allocs), "adam");
    LCK(net->alloc(&net->dflag, sizeof(int32_t), net->allocs), "flag");
    for (int l = 0; l < kLayers; ++l) {
        const size_t n = (size_t)27 * pad16(kSpec[l].ci) * pad16(kSpec[l].co);
        LCK(net->alloc(&net->wf[l], n * 2, net->allocs), "weights");
        LCK(net->alloc(&net->wb[l], n * 2, net->allocs), "weights");
    }
    LCK(cudaMemcpyAsync(net->p, h.data(), h.size() * 4, cudaMemcpyHostToDevice, net->st), "params");
    LCK(refresh_weights(net), "weights");
    LCK(cudaStreamSynchronize(net->st), "create");
    return FALCON_OK;
}

void falcon_lcc_destroy(falcon_lcc* net) {
    if (!net) return;
    if (net->st) {
        cudaSetDevice(net->device);
        cudaStreamSynchronize(net->st);
        for (void* q : net->act_allocs) cudaFree(q);
        for (void* q : net->allocs) cudaFree(q);
        cudaStreamDestroy(net->st);
    }
    delete net;
}

int falcon_lcc_last_error(const falcon_lcc* net, char* buf, size_t len) {
    if (!net || !buf || !len) return FALCON_ERR_INVALID_ARG;
    snprintf(buf, len, "%s", net->err.c_str());
    return FALCON_OK;
}

int falcon_lcc_num_params(const falcon_lcc* net, int64_t* n) {
    if (!net || !n) return FALCON_ERR_INVALID_ARG;
    *n = net->nparam;
    return FALCON_OK;
}

int falcon_lcc_get_params(falcon_lcc* net, float* params) {
    if (!net || !params || !net->st) return FALCON_ERR_INVALID_ARG;
    cudaSetDevice(net->device);
    LCK(cudaMemcpyAsync(params, net->p, (size_t)net->nparam * 4, cudaMemcpyDeviceToHost, net->st), "params");
    LCK(cudaStreamSynchronize(net->st), "params");
    return FALCON_OK;
}

int falcon_lcc_set_params(falcon_lcc* net, const float* params) {
    if (!net || !params || !net->st) return FALCON_ERR_INVALID_ARG;
    cudaSetDevice(net->device);
    LCK(cudaMemcpyAsync(net->p, params, (size_t)net->nparam * 4, cudaMemcpyHostToDevice, net->st), "params");
    LCK(cudaMemsetAsync(net->m, 0, (size_t)net->nparam * 4, net->st), "params");
    LCK(cudaMemsetAsync(net->v, 0, (size_t)net->nparam * 4, net->st), "params");
    net->adam_t = 0;
    LCK(refresh_weights(net), "weights");
    LCK(cudaStreamSynchronize(net->st), "params");
    return FALCON_OK;
}

int falcon_lcc_forward(falcon_lcc* net, const float* x, int32_t n, int32_t D, int32_t H, int32_t W, float* y) {
    if (!net || !x || !y || !net->st) return FALCON_ERR_INVALID_ARG;
    int rc = check_shape(net, n, D, H, W);
    if (rc) return rc;
    cudaSetDevice(net->device);
    LCK(ensure_shape(net, n, D, H, W), "buffers");
    const size_t V0 = (size_t)n * D * H * W;
    LCK(cudaMemcpyAsync(net->A.xin, x, V0 * 8 * 4, cudaMemcpyHostToDevice, net->st), "input");
    LCK(forward(net, net->st), "forward");
    LCK(cudaMemcpyAsync(y, net->A.y, V0 * 4, cudaMemcpyDeviceToHost, net->st), "output");
    LCK(cudaStreamSynchronize(net->st), "forward");
    return check_flag(net);
}

int falcon_lcc_loss_grad(falcon_lcc* net, const float* x, const float* t, int32_t n, int32_t D, int32_t H, int32_t W,
                         double* loss, float* grad) {
    if (!net || !x || !t || !loss || !grad || !net->st) return FALCON_ERR_INVALID_ARG;
    int rc = check_shape(net, n, D, H, W);
    if (rc) return rc;
    cudaSetDevice(net->device);
    LCK(ensure_shape(net, n, D, H, W), "buffers");
    const size_t V0 = (size_t)n * D * H * W;
    LCK(cudaMemcpyAsync(net->A.xin, x, V0 * 8 * 4, cudaMemcpyHostToDevice, net->st), "input");
    LCK(cudaMemcpyAsync(net->A.t, t, V0 * 4, cudaMemcpyHostToDevice, net->st), "target");
    LCK(forward(net, net->st), "forward");
    LCK(backward(net, net->st), "backward");
    double sum = 0;
    LCK(cudaMemcpyAsync(&sum, net->A.loss, 8, cudaMemcpyDeviceToHost, net->st), "loss");
    LCK(cudaMemcpyAsync(grad, net->g, (size_t)net->nparam * 4, cudaMemcpyDeviceToHost, net->st), "grad");
    LCK(cudaStreamSynchronize(net->st), "backward");
    *loss = sum / (double)V0;
    return check_flag(net);
}

int falcon_lcc_set_wait_limit(falcon_lcc* net, int32_t polls) {
    if (!net) return FALCON_ERR_INVALID_ARG;
    net->polls = polls < 0 ? tc::kPolls : polls;
    return FALCON_OK;
}

int falcon_lcc_set_tensor_path(falcon_lcc* net, int32_t path) {
    if (!net || (path != FALCON_LCC_MMA_SYNC && path != FALCON_LCC_TCGEN05)) return FALCON_ERR_INVALID_ARG;
    net->use_tc = path == FALCON_LCC_TCGEN05;
    return FALCON_OK;
}

int falcon_lcc_train(falcon_lcc* net, const float* x, const float* t, int32_t nsamples, int32_t D, int32_t H, int32_t W,
                     int32_t epochs, int32_t batch, float lr, uint64_t seed, float* epoch_loss) {
    if (!net || !x || !t || !net->st || nsamples < 1 || epochs < 1 || batch < 1) return FALCON_ERR_INVALID_ARG;
    batch = std::min(batch, nsamples);
    int rc = check_shape(net, batch, D, H, W);
    if (rc) return rc;
    cudaSetDevice(net->device);
    LCK(ensure_shape(net, batch, D, H, W), "buffers");
    const size_t V = (size_t)D * H * W;
    float *dx = nullptr, *dt = nullptr;
    auto cleanup = [&] { cudaStreamSynchronize(net->st); cudaFree(dx); cudaFree(dt); };
    cudaError_t e = cudaMalloc(&dx, (size_t)nsamples * V * 8 * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dt, (size_t)nsamples * V * 4);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, (size_t)nsamples * V * 8 * 4, cudaMemcpyHostToDevice, net->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dt, t, (size_t)nsamples * V * 4, cudaMemcpyHostToDevice, net->st);
    if (e != cudaSuccess) { cleanup(); return net->fail(FALCON_ERR_CUDA, std::string("lcc train data: ") + cudaGetErrorString(e)); }
    std::vector<int> order(nsamples);
    for (int q = 0; q < nsamples; ++q) order[q] = q;
    std::mt19937_64 rng(seed);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int ep = 0; ep < epochs && e == cudaSuccess; ++ep) {
        std::shuffle(order.begin(), order.end(), rng);
        double ep_loss = 0;
        int nb = 0;
        for (int s0 = 0; s0 + batch <= nsamples && e == cudaSuccess; s0 += batch) {
            for (int q = 0; q < batch && e == cudaSuccess; ++q) {
                const int smp = order[s0 + q];
                e = cudaMemcpyAsync(net->A.xin + (size_t)q * V * 8, dx + (size_t)smp * V * 8, V * 8 * 4,
                                    cudaMemcpyDeviceToDevice, net->st);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(net->A.t + (size_t)q * V, dt + (size_t)smp * V, V * 4, cudaMemcpyDeviceToDevice, net->st);
            }
            if (e == cudaSuccess) e = forward(net, net->st);
            if (e == cudaSuccess) e = backward(net, net->st);
            if (e != cudaSuccess) break;
            ++net->adam_t;
            const float c1 = 1.f / (1.f - std::pow(b1, (float)net->adam_t));
            const float c2 = 1.f / (1.f - std::pow(b2, (float)net->adam_t));
            k_adam<<<ew_grid(net->nparam), 256, 0, net->st>>>(net->p, net->g, net->m, net->v, net->nparam, lr, b1, b2, c1,
                                                              c2, eps);
            e = refresh_weights(net);
            double l = 0;
            if (e == cudaSuccess) e = cudaMemcpyAsync(&l, net->A.loss, 8, cudaMemcpyDeviceToHost, net->st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(net->st);
            ep_loss += l / (double)(batch * V);
            ++nb;
        }
        if (epoch_loss) epoch_loss[ep] = (float)(ep_loss / std::max(nb, 1));
    }
    cleanup();
    if (e != cudaSuccess) return net->fail(FALCON_ERR_CUDA, std::string("lcc train: ") + cudaGetErrorString(e));
    return check_flag(net);
}

}  // extern "C"
