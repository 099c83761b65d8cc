// capi.cu -- the C ABI (include/falcon_gb300.h): context, device tables,
// state transfer, the captured step graph and kernel timing.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/falcon_gb300.h"
#include "host_setup.h"
#include "kernels.cuh"
#include "synth.cuh"

namespace falcon {
// state_range.cu: range download through the library's static device array
size_t static_scratch_elems();
std::string download_range_static(int dev, cudaStream_t st, const void* U, const int8_t* Ulo, const void* P,
                                  bool mixed, const StepDims& dm, size_t first, size_t count, double* u);
}  // namespace falcon

using namespace falcon;

namespace {
const char* const kKernelNames[] = {"stage", "diffusion", "cfl", "finalize_dt", "ghost_fill"};
enum { KN_STAGE = 0, KN_DIFF, KN_CFL, KN_FIN, KN_GHOST, KN_COUNT };
}  // namespace

struct falcon_ctx {
    Grid grid;
    std::string err;
    falcon_config cfg;
    bool on_device = false;
    int device = -1;
    cudaStream_t st = nullptr;
    StepDims dims{};
    size_t elem = 8;            // bytes per state element
    void* U = nullptr;          // u^n (primitive_IV)
    void* RK = nullptr;         // stage state (primitive_rk_IV)
    int8_t* Ulo = nullptr;      // mixed mode: 8-bit correction of u^n (interior cells)
    void *P = nullptr, *Prk = nullptr, *P2 = nullptr;   // psi of U, RK, R2 (GLM only) [b][cell]
    double* stage64 = nullptr;  // FP64 staging buffer for mixed-mode transfers (lazy)
    int32_t* dflag = nullptr;   // device flag of the upload's psi check (lazy)
    std::vector<std::pair<uintptr_t, size_t>> pinned;   // host ranges pinned through falcon_pin_host
    double *gi = nullptr, *gj = nullptr, *gs = nullptr;
    float *gi_f = nullptr, *gj_f = nullptr, *gs_f = nullptr;
    int32_t* flags = nullptr;
    StepScalars* sc = nullptr;
    GhostLists gl{};          // every ghost cell (the exchange after the diffusion pass)
    GhostLists gl_stage{};    // face ghosts not pushed by the stage kernel (exchanges after stages)
    GhostLists gl_final{};    // mixed: ghost entries the exchange ending a step fills (see setup_device)
    bool stale_edges = false; // mixed: edge/corner ghosts not refreshed since the last step
    bool cfl_ready = false;   // mixed: the last diffusion pass formed this state's CFL minimum
    PushTable push{};         // mixed path: faces the stage kernel writes into its output
    void* R2 = nullptr;       // mixed path: second stage buffer (pushing needs out != in)
    int64_t ghost_counts[3] = {0, 0, 0};   // copy, 1-D, general entries on the device
    int64_t stage_counts[3] = {0, 0, 0};   // the same for the stage exchanges
    int64_t final_counts[3] = {0, 0, 0};   // the same for the exchange ending a mixed step
    int64_t pushed_faces = 0, pushed_cells = 0;
    int kpar_stage = 0, kpar_diff = 0;      // chosen by the autotuner (0 = not tuned yet)
    int step_mode = FALCON_STEP_GRAPH;      // FALCON_STEP_PERSISTENT: one cooperative launch per step
    unsigned int* gbar = nullptr;           // persistent step: grid-barrier counter, generation, block tickets
    // step graphs: the mixed step writes u^{n+1} into the second stage buffer
    // and the two buffers swap roles, so one graph per assignment (index 0
    // while U is the first allocation)
    // [buffer assignment][CFL minimum already formed by the previous step]
    cudaGraphExec_t graphs[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    // block sharding (FP64 phases): this context computes blocks [first, last)
    // of the global tree; ghost entries whose source and target it owns are
    // filled on the device, the others travel through per-peer pack buffers
    struct Shard {
        bool on = false;
        int nranks = 1, rank = 0, first = 0, last = 0;
        GhostLists local{};
        std::vector<GhostInterpList> send;     // [peer] outgoing entries (source owned, target on the peer)
        std::vector<int32_t*> recv_dst;        // [peer] target offsets of the incoming entries
        std::vector<int64_t> nrecv;
        double* pack = nullptr;                // device staging for host pack buffers
        size_t pack_elems = 0;
        void* last_out = nullptr;              // the buffer the last shard phase or exchange filled
    } shard;
    void* bufA = nullptr;
    int64_t steps_done = 0;
    int64_t dev_bytes = 0;
    // timing
    bool ktiming = false;
    struct Rec { int k; cudaEvent_t a, b; };
    std::vector<Rec> pending;
    std::vector<cudaEvent_t> pool;
    double kms[KN_COUNT] = {0};
    int64_t kcount[KN_COUNT] = {0};
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    std::vector<void*> allocs;

    int fail(int code, const std::string& m) { err = m; return code; }
    int cuda_fail(cudaError_t e, const char* where) {
        err = std::string(where) + ": " + cudaGetErrorString(e);
        return FALCON_ERR_CUDA;
    }
    template <class P> cudaError_t alloc(P** p, size_t bytes) {
        cudaError_t e = cudaMalloc((void**)p, bytes ? bytes : 16);
        if (e == cudaSuccess) { allocs.push_back((void*)*p); dev_bytes += (int64_t)bytes; }
        return e;
    }
    cudaEvent_t ev() {
        if (pool.empty()) { cudaEvent_t e; cudaEventCreate(&e); return e; }
        cudaEvent_t e = pool.back(); pool.pop_back(); return e;
    }
    Geometry geom() const { return Geometry{gi, gj, gs, gi_f, gj_f, gs_f, flags}; }
    bool mixed() const { return cfg.precision == FALCON_PREC_MIXED; }
};

#define CK(call, where)                                         \
    do {                                                        \
        cudaError_t e_ = (call);                                \
        if (e_ != cudaSuccess) return ctx->cuda_fail(e_, where); \
    } while (0)

namespace {

// Launch one kernel, bracketed by events when per-kernel timing is on.
template <class F> cudaError_t timed(falcon_ctx* ctx, int k, F&& f) {
    if (!ctx->ktiming) return f();
    cudaEvent_t a = ctx->ev(), b = ctx->ev();
    cudaEventRecord(a, ctx->st);
    cudaError_t e = f();
    cudaEventRecord(b, ctx->st);
    ctx->pending.push_back({k, a, b});
    return e;
}

void collect(falcon_ctx* ctx) {
    for (auto& r : ctx->pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
            ctx->kms[r.k] += ms;
            ctx->kcount[r.k] += 1;
        }
        ctx->pool.push_back(r.a);
        ctx->pool.push_back(r.b);
    }
    ctx->pending.clear();
}

// Ghost fill of every ghost cell (faces, edges and corners), as the reference's
// exchange does.
cudaError_t ghost(falcon_ctx* ctx, void* u) {
    return timed(ctx, KN_GHOST, [&] {
        return ctx->mixed() ? launch_ghost_mixed(ctx->dims, ctx->gl, (float*)u, ctx->st)
                            : launch_ghost_fp64(ctx->dims, ctx->gl, (double*)u, ctx->st);
    });
}

// Ghost fill between RK stages: face ghosts only (every stencil of the step
// is axis-aligned, so edge and corner ghosts are never read before the full
// exchange that ends the step), minus the faces the stage kernel pushed.
cudaError_t ghost_stage(falcon_ctx* ctx, void* u) {
    return timed(ctx, KN_GHOST, [&] {
        return ctx->mixed() ? launch_ghost_mixed(ctx->dims, ctx->gl_stage, (float*)u, ctx->st)
                            : launch_ghost_fp64(ctx->dims, ctx->gl_stage, (double*)u, ctx->st);
    });
}

cudaError_t cfl(falcon_ctx* ctx) {
    ctx->cfl_ready = false;   // the minimum formed by a diffusion pass is replaced and consumed here
    cudaError_t e = timed(ctx, KN_CFL, [&] {
        return ctx->mixed() ? launch_cfl_mixed(ctx->dims, ctx->geom(), (const float*)ctx->U, ctx->sc, ctx->st)
                            : launch_cfl_fp64(ctx->dims, ctx->geom(), (const double*)ctx->U, ctx->sc, ctx->st);
    });
    if (e != cudaSuccess) return e;
    return timed(ctx, KN_FIN, [&] { return launch_finalize_dt(ctx->sc, ctx->st); });
}

// GLM psi through a stage: read psi_in (global memory, so never the array
// being written), write P2, then copy to the stage array (RK's psi) for
// stages 1-3; stage 4 writes u^{n+1}'s psi in place of u^n's cell by cell.
DivBArgs psi_args(const falcon_ctx* ctx, int s) {
    if (!ctx->P) return DivBArgs{nullptr, nullptr, nullptr, ctx->cfg.phys.divb_option == 2 ? 2 : 0};
    return DivBArgs{s == 1 ? ctx->P : ctx->Prk, ctx->P, s == 4 ? ctx->P : ctx->P2, 1};
}
cudaError_t psi_after_stage(falcon_ctx* ctx, int s) {
    if (!ctx->P) return cudaSuccess;
    void* tgt = s == 4 ? ctx->P : ctx->Prk;
    if (s < 4) {
        cudaError_t e = cudaMemcpyAsync(ctx->Prk, ctx->P2, (size_t)ctx->dims.nblocks * ctx->dims.ncell * ctx->elem,
                                        cudaMemcpyDeviceToDevice, ctx->st);
        if (e != cudaSuccess) return e;
    }
    return timed(ctx, KN_GHOST, [&] {
        return ctx->mixed() ? launch_psi_ghost_mixed(ctx->dims, ctx->gl, (float*)tgt, ctx->st)
                            : launch_psi_ghost_fp64(ctx->dims, ctx->gl, (double*)tgt, ctx->st);
    });
}

// Stage s from `in` into `out` (ModAdvance.f90:59-97), GLM terms included.
cudaError_t stage(falcon_ctx* ctx, int s, void* in, void* out, const PushTable& push) {
    const DivBArgs ps = psi_args(ctx, s);
    cudaError_t e = timed(ctx, KN_STAGE, [&] {
        return ctx->mixed()
                   ? launch_stage_mixed(ctx->dims, ctx->geom(), (const float*)in, (const float*)ctx->U, (float*)out,
                                        ctx->Ulo, push, ps, s, 1, ctx->sc, 1, ctx->kpar_stage, ctx->st)
                   : launch_stage_fp64(ctx->dims, ctx->geom(), (const double*)in, (const double*)ctx->U, (double*)out,
                                       ps, s, 1, ctx->sc, 1, ctx->kpar_stage, ctx->st);
    });
    if (e != cudaSuccess) return e;
    return psi_after_stage(ctx, s);
}

// Artificial diffusion of every variable (ModAdvance.f90:101-109); psi's runs
// first, from the same pre-diffusion state, into P2.
cudaError_t diffusion(falcon_ctx* ctx, void* out, const PushTable& push, int cfl_next = 0) {
    cudaError_t e = cudaSuccess;
    if (ctx->P) {
        e = timed(ctx, KN_DIFF, [&] {
            return ctx->mixed() ? launch_psi_diffusion_mixed(ctx->dims, ctx->geom(), (const float*)ctx->U,
                                                             (const float*)ctx->P, (float*)ctx->P2, ctx->sc, ctx->st)
                                : launch_psi_diffusion_fp64(ctx->dims, ctx->geom(), (const double*)ctx->U,
                                                            (const double*)ctx->P, (double*)ctx->P2, ctx->sc, ctx->st);
        });
        if (e != cudaSuccess) return e;
    }
    e = timed(ctx, KN_DIFF, [&] {
        return ctx->mixed() ? launch_diffusion_mixed(ctx->dims, ctx->geom(), (const float*)ctx->U, (float*)out,
                                                     ctx->Ulo, push, ctx->sc, ctx->kpar_diff, ctx->st, cfl_next)
                            : launch_diffusion_fp64(ctx->dims, ctx->geom(), (double*)ctx->U, ctx->sc, ctx->kpar_diff, ctx->st);
    });
    if (e != cudaSuccess || !ctx->P) return e;
    e = cudaMemcpyAsync(ctx->P, ctx->P2, (size_t)ctx->dims.nblocks * ctx->dims.ncell * ctx->elem,
                        cudaMemcpyDeviceToDevice, ctx->st);
    if (e != cudaSuccess) return e;
    return timed(ctx, KN_GHOST, [&] {
        return ctx->mixed() ? launch_psi_ghost_mixed(ctx->dims, ctx->gl, (float*)ctx->P, ctx->st)
                            : launch_psi_ghost_fp64(ctx->dims, ctx->gl, (double*)ctx->P, ctx->st);
    });
}

// One ModAdvance_rk4 (3_6/ModAdvance.f90:18-112) as a kernel sequence.
// FP64: stages 2-4 read and write the stage buffer in place. Mixed: the stage
// kernels push ghost faces into their output, so input and output differ:
// U -> RK -> R2 -> RK -> U (stage 4 writes u^{n+1} over u^n cell by cell).
cudaError_t enqueue_step(falcon_ctx* ctx) {
    const bool fused_cfl = ctx->mixed() && ctx->R2;
    cudaError_t e = (fused_cfl && ctx->cfl_ready) ? timed(ctx, KN_FIN, [&] { return launch_finalize_dt(ctx->sc, ctx->st); })
                                                   : cfl(ctx);
    if (e != cudaSuccess) return e;
    for (int s = 1; s <= 4; ++s) {
        void* in;
        void* out;
        if (ctx->mixed()) {
            void* const seq[5] = {ctx->U, ctx->RK, ctx->R2, ctx->RK, ctx->U};
            in = seq[s - 1];
            out = seq[s];
        } else {
            in = (s == 1) ? ctx->U : ctx->RK;
            out = (s < 4) ? ctx->RK : ctx->U;
        }
        e = stage(ctx, s, in, out, ctx->mixed() ? ctx->push : PushTable{});
        if (e != cudaSuccess) return e;
        e = ghost_stage(ctx, out);
        if (e != cudaSuccess) return e;
    }
    if (ctx->mixed() && ctx->R2) {
        // u^{n+1} into the second stage buffer, regular faces pushed by the
        // diffusion pass, then the remaining ghost entries; end_step swaps
        // the two buffers' roles
        e = diffusion(ctx, ctx->R2, ctx->push, 1);
        if (e != cudaSuccess) return e;
        return timed(ctx, KN_GHOST, [&] { return launch_ghost_mixed(ctx->dims, ctx->gl_final, (float*)ctx->R2, ctx->st); });
    }
    e = diffusion(ctx, ctx->U, PushTable{});
    if (e != cudaSuccess) return e;
    return ghost(ctx, ctx->U);
}

// After a step has been enqueued: the mixed step left u^{n+1} in R2, with
// edge and corner ghosts not refreshed.
void end_step(falcon_ctx* ctx) {
    if (ctx->mixed() && ctx->R2) {
        std::swap(ctx->U, ctx->R2);
        ctx->stale_edges = true;
        ctx->cfl_ready = true;
    }
}

// Before the state is read from outside the step: complete its ghost cells.
// Every ghost entry is a function of interior cells only, so this gives the
// values the reference's exchange would have left.
cudaError_t fresh_state(falcon_ctx* ctx) {
    if (!ctx->stale_edges) return cudaSuccess;
    cudaError_t e = ghost(ctx, ctx->U);
    if (e == cudaSuccess) ctx->stale_edges = false;
    return e;
}

// The second stage buffer starts as a copy of the state: cells that no
// kernel writes (ghost cells outside every exchange list) then agree in both
// buffers whichever holds the state.
// A new state (upload, synthetic initial condition, restart) starts with the
// step flags clear: no NaN seen, no copy wait run out.
cudaError_t clear_step_flags(falcon_ctx* ctx) {
    cudaError_t e = cudaMemsetAsync(&ctx->sc->nan_flag, 0, sizeof(int32_t), ctx->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(&ctx->sc->nan_step, 0xFF, sizeof(int32_t), ctx->st);   // -1
    return e;
}

// The state or its background changed outside the fused step (upload,
// synthetic initial condition, restart, new background, phases): the CFL
// minimum that the last diffusion pass left pending belongs to the state it
// wrote, so it is dropped; the next minimum is formed from +inf.
cudaError_t drop_pending_cfl(falcon_ctx* ctx) {
    static const unsigned long long inf_bits = 0x7FF0000000000000ull;
    ctx->cfl_ready = false;
    return cudaMemcpyAsync(&ctx->sc->min_ratio_bits, &inf_bits, sizeof inf_bits, cudaMemcpyHostToDevice, ctx->st);
}

// The state copied into the second state buffer and, with stage, into the
// stage buffer too (primitive_rk_IV = primitive_IV, as the reference's
// initialisation leaves it): one pass that reads the state once.
__global__ void k_copy2(const uint4* __restrict__ src, uint4* __restrict__ a, uint4* __restrict__ b, size_t n) {
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (size_t)gridDim.x * blockDim.x) {
        const uint4 v = src[x];
        a[x] = v;
        if (b) b[x] = v;
    }
}
cudaError_t mirror_state(falcon_ctx* ctx, bool stage = false) {
    const size_t bytes = (size_t)ctx->dims.nblocks * NV * ctx->dims.ncell * ctx->elem;
    void* a = stage ? ctx->RK : ctx->R2;
    void* b = stage ? ctx->R2 : nullptr;
    if (!a) return cudaSuccess;
    if (bytes % 16 != 0) {   // not for the supported block sizes (ncell even, 4- or 8-byte cells)
        cudaError_t e = cudaMemcpyAsync(a, ctx->U, bytes, cudaMemcpyDeviceToDevice, ctx->st);
        if (e == cudaSuccess && b) e = cudaMemcpyAsync(b, ctx->U, bytes, cudaMemcpyDeviceToDevice, ctx->st);
        return e;
    }
    int nsm = 0;
    cudaError_t e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
    if (e != cudaSuccess) return e;
    k_copy2<<<nsm * 8, 256, 0, ctx->st>>>((const uint4*)ctx->U, (uint4*)a, (uint4*)b, bytes / 16);
    return cudaGetLastError();
}

// Autotuner: time every instantiated k-chunk depth of the stage and diffusion
// kernels on this grid and keep the fastest. Runs on the stage buffer only
// (dead between steps: stage 1 rewrites it), so the state is untouched.
int autotune(falcon_ctx* ctx) {
    if (ctx->kpar_stage && ctx->kpar_diff) return FALCON_OK;
    int cand[8];
    const int n = ctx->mixed() ? kpar_candidates_mixed(ctx->dims, cand) : kpar_candidates_fp64(ctx->dims, cand);
    if (n == 0) return ctx->fail(FALCON_ERR_INVALID_ARG, "no kernel instantiation for this block size");
    // the candidates take turns within each round of launches, so that a drift
    // of the clocks over the tuning touches every candidate alike; the first
    // round pays for set-up and is not counted
    constexpr int kRounds = 5;
    float tot[8][2] = {};
    bool ok[8][2];
    for (int q = 0; q < n; ++q) ok[q][0] = ok[q][1] = true;
    cudaEvent_t a = ctx->ev(), b = ctx->ev();
    for (int rep = 0; rep < kRounds; ++rep)
        for (int q = 0; q < n; ++q)
            for (int which = 0; which < 2; ++which) {
                if (!ok[q][which]) continue;
                const int kp = cand[q];
                cudaEventRecord(a, ctx->st);
                cudaError_t e;
                if (which == 0)
                    e = ctx->mixed() ? launch_stage_mixed(ctx->dims, ctx->geom(), (const float*)ctx->RK, (const float*)ctx->U,
                                                          (float*)ctx->R2, nullptr, ctx->push, psi_args(ctx, 2),
                                                          2, 1, ctx->sc, 1, kp, ctx->st)
                                     : launch_stage_fp64(ctx->dims, ctx->geom(), (const double*)ctx->RK, (const double*)ctx->U,
                                                         (double*)ctx->RK, psi_args(ctx, 2), 2, 1,
                                                         ctx->sc, 1, kp, ctx->st);
                else
                    e = ctx->mixed() ? launch_diffusion_mixed(ctx->dims, ctx->geom(), (const float*)ctx->RK,
                                                              (float*)ctx->RK, nullptr, PushTable{}, ctx->sc, kp, ctx->st)
                                     : launch_diffusion_fp64(ctx->dims, ctx->geom(), (double*)ctx->RK, ctx->sc, kp, ctx->st);
                cudaEventRecord(b, ctx->st);
                if (e != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess) { ok[q][which] = false; cudaGetLastError(); continue; }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, a, b);
                if (rep > 0) tot[q][which] += ms;
            }
    float best_s = 1e30f, best_d = 1e30f;
    int ks = cand[0], kd = cand[0];
    for (int q = 0; q < n; ++q) {
        if (ok[q][0] && tot[q][0] < best_s) { best_s = tot[q][0]; ks = cand[q]; }
        if (ok[q][1] && tot[q][1] < best_d) { best_d = tot[q][1]; kd = cand[q]; }
    }
    ctx->pool.push_back(a);
    ctx->pool.push_back(b);
    if (best_s >= 1e30f || best_d >= 1e30f) return ctx->fail(FALCON_ERR_CUDA, "autotune: no variant launched");
    ctx->kpar_stage = ks;
    ctx->kpar_diff = kd;
    // undo the tuning launches' side effects: the device flags, and the stage
    // buffer, which before the first step equals primitive_IV in the reference
    CK(cudaMemsetAsync(&ctx->sc->nan_flag, 0, sizeof(int32_t), ctx->st), "autotune");
    const size_t nelem = (size_t)ctx->dims.nblocks * NV * ctx->dims.ncell;
    CK(cudaMemcpyAsync(ctx->RK, ctx->U, nelem * ctx->elem, cudaMemcpyDeviceToDevice, ctx->st), "autotune");
    CK(cudaStreamSynchronize(ctx->st), "autotune");
    return FALCON_OK;
}

int check_nan(falcon_ctx* ctx) {
    int32_t flag = 0, stp = -1;
    cudaError_t e = cudaMemcpy(&flag, &ctx->sc->nan_flag, sizeof(int32_t), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "nan flag");
    cudaMemcpy(&stp, &ctx->sc->nan_step, sizeof(int32_t), cudaMemcpyDeviceToHost);
    if (flag & 2) {
        // a step kernel's wait for a bulk copy ran out: its CTAs left cleanly,
        // the step's results are discarded (the state is undefined until the
        // next upload, synthetic initial condition or restart)
        int32_t polls = 0;
        cudaMemcpy(&polls, &ctx->sc->wait_polls, sizeof(int32_t), cudaMemcpyDeviceToHost);
        char buf[192];
        snprintf(buf, sizeof buf, "a step kernel's bulk-copy wait ran out (poll limit %d); the state is undefined", polls);
        ctx->err = buf;
        return FALCON_ERR_TIMEOUT;
    }
    if (flag) {
        char buf[128];
        snprintf(buf, sizeof buf, "NaN detected in the state at the start of step %d", stp);
        ctx->err = buf;
        return FALCON_ERR_NAN_DETECTED;
    }
    return FALCON_OK;
}

// global element offset of var 0 of padded cell (i,j,k) (Fortran indices) of block b
inline int64_t cell_off(const Grid& g, int b, int i, int j, int k) {
    return (int64_t)b * NV * g.ncell + ((int64_t)(k + 1) * g.njp + (j + 1)) * g.nip + (i + 1);
}

// ---- block sharding ------------------------------------------------------------
// The reference's partition of leaves over ranks (ModAllocation_Init,
// 3_6/ModAllocation.f90:25-39): contiguous ranges, the first nb % R ranks one
// leaf longer. first[r] .. first[r+1]-1 are rank r's blocks (0-based).
std::vector<int> shard_ranges(int nb, int R) {
    std::vector<int> first(R + 1, 0);
    for (int r = 0; r < R; ++r) first[r + 1] = first[r] + nb / R + (r < nb % R ? 1 : 0);
    return first;
}
int rank_of(const std::vector<int>& first, int b) {
    return (int)(std::upper_bound(first.begin(), first.end(), b) - first.begin()) - 1;
}
// Entries of the canonical ghost map (falcon_ghost_map order) from the
// blocks of rank `src` to the blocks of rank `dst`: in map order on both
// sides, so the sender's pack order is the receiver's scatter order (the
// reference's per-peer send/receive lists, 3_6/ModCommunication.f90:375-634).
std::vector<int64_t> shard_entries(const Grid& g, const std::vector<int>& first, int src, int dst) {
    std::vector<int64_t> out;
    for (size_t k = 0; k < g.ghosts.size(); ++k) {
        const auto& e = g.ghosts[k].e;
        if (rank_of(first, e.sblock) == src && rank_of(first, e.tblock) == dst) out.push_back((int64_t)k);
    }
    return out;
}

// FP64 device lists of the given map entries: the trilinear/rotated form of
// the exchange for every entry (a copy is an entry of kind 0), target offsets
// and source base offsets into the state.
cudaError_t upload_interp_list(falcon_ctx* ctx, const std::vector<int64_t>& ks, GhostInterpList& out, int32_t** dst_out) {
    const Grid& g = ctx->grid;
    const size_t n = ks.size();
    std::vector<int32_t> dst(n), src(n);
    std::vector<double> w(3 * n), rot(2 * n);
    std::vector<uint8_t> kind(n);
    for (size_t q = 0; q < n; ++q) {
        const GhostMapEntry& e = g.ghosts[ks[q]];
        dst[q] = (int32_t)cell_off(g, e.e.tblock, e.e.ti, e.e.tj, e.e.tk);
        src[q] = (int32_t)cell_off(g, e.e.sblock, e.i0, e.j0, e.k0);
        const int nz = (e.w[0] != 0.0) + (e.w[1] != 0.0) + (e.w[2] != 0.0);
        for (int t = 0; t < 3; ++t) w[3 * q + t] = e.w[t];
        rot[2 * q] = e.rotate ? e.rot[0] : 0.0;
        rot[2 * q + 1] = e.rotate ? e.rot[1] : 0.0;
        kind[q] = (uint8_t)((nz ? 1 : 0) | (e.rotate ? 2 : 0));
    }
    auto up = [&](auto** dptr, const auto& vec) -> cudaError_t {
        using E = typename std::decay_t<decltype(vec)>::value_type;
        cudaError_t r = ctx->alloc(dptr, vec.size() * sizeof(E));
        if (r == cudaSuccess && !vec.empty()) r = cudaMemcpy(*dptr, vec.data(), vec.size() * sizeof(E), cudaMemcpyHostToDevice);
        return r;
    };
    int32_t *d_dst, *d_src;
    double *d_w, *d_rot;
    uint8_t* d_kind;
    cudaError_t e = up(&d_dst, dst);
    if (e == cudaSuccess) e = up(&d_src, src);
    if (e == cudaSuccess) e = up(&d_w, w);
    if (e == cudaSuccess) e = up(&d_rot, rot);
    if (e == cudaSuccess) e = up(&d_kind, kind);
    if (e != cudaSuccess) return e;
    out = GhostInterpList{(int64_t)n, d_dst, d_src, d_w, d_rot, d_kind, nullptr, nullptr};
    if (dst_out) *dst_out = d_dst;
    return cudaSuccess;
}

// Geometry of blocks [first, ..): the per-block tables advanced, so a kernel
// launched over nlocal blocks computes the owned ones with its own indexing.
Geometry geom_from(const falcon_ctx* ctx, int first) {
    const Grid& g = ctx->grid;
    const size_t fi = (size_t)first * GI_COUNT * g.nip, fj = (size_t)first * GJ_COUNT * g.njp,
                 fs = (size_t)first * GS_COUNT;
    return Geometry{ctx->gi + fi, ctx->gj + fj, ctx->gs + fs, ctx->gi_f + fi, ctx->gj_f + fj, ctx->gs_f + fs,
                    ctx->flags + first};
}

// Per-block 1-D geometry and background tables on the device, from the grid's
// radial profiles g.prof (the outputs of ModStratification_new_get_vars at the
// cell centres, 3_6/ModBlock.f90:232-264): built at set-up and again when a
// driver supplies its own profiles (falcon_set_background).
int upload_tables(falcon_ctx* ctx, bool first) {
    const Grid& g = ctx->grid;
    const int nb = g.nblocks;
    std::vector<double> gi((size_t)nb * GI_COUNT * g.nip), gj((size_t)nb * GJ_COUNT * g.njp), gs((size_t)nb * GS_COUNT);
    const double ratio = ctx->cfg.phys.heating_ratio;
    for (int b = 0; b < nb; ++b) {
        double* I = &gi[(size_t)b * GI_COUNT * g.nip];
        const double* P = &g.prof[(size_t)b * FALCON_NPROF * g.nip];
        for (int i = 0; i < g.nip; ++i) {
            const double r = g.xi[(size_t)b * g.nip + i];
            const double gg = P[0 * g.nip + i], rho0 = P[1 * g.nip + i], p0 = P[2 * g.nip + i], T0 = P[3 * g.nip + i];
            const double g1 = P[4 * g.nip + i], g3 = P[5 * g.nip + i];
            const double heat = P[6 * g.nip + i] + P[7 * g.nip + i], Xi = P[8 * g.nip + i];
            const double p0r0 = p0 / rho0, rho0T0 = rho0 * T0;
            I[GI_R * g.nip + i] = r;
            I[GI_R2 * g.nip + i] = r * r;
            I[GI_RINV * g.nip + i] = 1. / r;
            I[GI_R2INV * g.nip + i] = 1. / (r * r);
            I[GI_A1 * g.nip + i] = g1 * p0r0;
            I[GI_A2 * g.nip + i] = (g3 - 1.0) * rho0T0;
            I[GI_RHO0 * g.nip + i] = rho0;
            I[GI_RHO0INV * g.nip + i] = 1. / rho0;
            I[GI_GOR0 * g.nip + i] = gg / rho0;
            I[GI_HEAT * g.nip + i] = ratio * heat / rho0T0;
            I[GI_XI2INV * g.nip + i] = 1.0 / (Xi * Xi);
            I[GI_CS * g.nip + i] = 1. / Xi * std::sqrt(g1 * p0r0);
        }
        double* J = &gj[(size_t)b * GJ_COUNT * g.njp];
        for (int j = 0; j < g.njp; ++j) {
            const double t = g.xj[(size_t)b * g.njp + j];
            J[GJ_SIN * g.njp + j] = std::sin(t);
            J[GJ_SININV * g.njp + j] = 1. / std::sin(t);
            J[GJ_COT * g.njp + j] = std::cos(t) / std::sin(t);
        }
        double* S = &gs[(size_t)b * GS_COUNT];
        const double c = (double)(1.0f / 12.0f);   // the FP32 constant 1./12. of ModDerivative
        S[GS_C1] = c / g.dx[3 * b];
        S[GS_C2] = c / g.dx[3 * b + 1];
        S[GS_C3] = c / g.dx[3 * b + 2];
        S[GS_DXI] = g.dx[3 * b];
        S[GS_DXJ] = g.dx[3 * b + 1];
        S[GS_DXK] = g.dx[3 * b + 2];
    }
    std::vector<float> gif(gi.begin(), gi.end()), gjf(gj.begin(), gj.end()), gsf(gs.begin(), gs.end());
    if (first) {
        CK(ctx->alloc(&ctx->gi, gi.size() * 8), "alloc gi");
        CK(ctx->alloc(&ctx->gj, gj.size() * 8), "alloc gj");
        CK(ctx->alloc(&ctx->gs, gs.size() * 8), "alloc gs");
        CK(ctx->alloc(&ctx->gi_f, gif.size() * 4), "alloc gi_f");
        CK(ctx->alloc(&ctx->gj_f, gjf.size() * 4), "alloc gj_f");
        CK(ctx->alloc(&ctx->gs_f, gsf.size() * 4), "alloc gs_f");
    }
    // ordered after the context stream's earlier work (the tables are read
    // by every step kernel): plain copies wait for nothing on a non-blocking stream
    CK(cudaStreamSynchronize(ctx->st), "tables");
    CK(cudaMemcpy(ctx->gi, gi.data(), gi.size() * 8, cudaMemcpyHostToDevice), "upload gi");
    CK(cudaMemcpy(ctx->gj, gj.data(), gj.size() * 8, cudaMemcpyHostToDevice), "upload gj");
    CK(cudaMemcpy(ctx->gs, gs.data(), gs.size() * 8, cudaMemcpyHostToDevice), "upload gs");
    CK(cudaMemcpy(ctx->gi_f, gif.data(), gif.size() * 4, cudaMemcpyHostToDevice), "upload gi_f");
    CK(cudaMemcpy(ctx->gj_f, gjf.data(), gjf.size() * 4, cudaMemcpyHostToDevice), "upload gj_f");
    CK(cudaMemcpy(ctx->gs_f, gsf.data(), gsf.size() * 4, cudaMemcpyHostToDevice), "upload gs_f");

    return FALCON_OK;
}

int setup_device(falcon_ctx* ctx) {
    const Grid& g = ctx->grid;
    const int nb = g.nblocks;
    if ((int64_t)nb * NV * g.ncell >= (int64_t)INT32_MAX) return ctx->fail(FALCON_ERR_INVALID_ARG, "grid too large for 32-bit offsets");
    const bool sup = (g.ni == 8 && g.nj == 8 && g.nk == 8) || (g.ni == 16 && g.nj == 16 && g.nk == 16);
    if (!sup) return ctx->fail(FALCON_ERR_INVALID_ARG, "device kernels are built for 8^3 and 16^3 blocks");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return ctx->fail(FALCON_ERR_NO_DEVICE, "no CUDA device");
    if (ctx->cfg.device >= ndev) return ctx->fail(FALCON_ERR_INVALID_ARG, "device ordinal out of range");
    CK(cudaSetDevice(ctx->cfg.device), "cudaSetDevice");
    ctx->device = ctx->cfg.device;
    CK(cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking), "stream");
    CK(cudaEventCreate(&ctx->t0), "event");
    CK(cudaEventCreate(&ctx->t1), "event");
    ctx->dims = StepDims{nb, g.ni, g.nj, g.nk, g.nip, g.njp, g.nkp, g.ncell};
    ctx->elem = ctx->mixed() ? 4 : 8;
    const size_t sbytes = (size_t)nb * NV * g.ncell * ctx->elem;
    CK(ctx->alloc(&ctx->U, sbytes), "alloc U");
    ctx->bufA = ctx->U;
    CK(ctx->alloc(&ctx->RK, sbytes), "alloc RK");
    CK(cudaMemsetAsync(ctx->U, 0, sbytes, ctx->st), "memset");
    CK(cudaMemsetAsync(ctx->RK, 0, sbytes, ctx->st), "memset");
    if (ctx->cfg.phys.divb_option == 1) {
        const size_t pbytes = (size_t)nb * g.ncell * ctx->elem;
        for (void** q : {&ctx->P, &ctx->Prk, &ctx->P2}) {
            CK(ctx->alloc(q, pbytes), "alloc psi");
            CK(cudaMemsetAsync(*q, 0, pbytes, ctx->st), "memset");
        }
    }
    if (ctx->mixed()) {
        CK(ctx->alloc(&ctx->Ulo, lo_elems(ctx->dims)), "alloc U correction");
        CK(cudaMemsetAsync(ctx->Ulo, 0, lo_elems(ctx->dims), ctx->st), "memset");
    }

    // geometry and background tables (3_6/ModBlock.f90:188-265, 288-438)
    {
        const int rc = upload_tables(ctx, true);
        if (rc) return rc;
    }
    CK(ctx->alloc(&ctx->flags, (size_t)nb * 4), "alloc flags");
    CK(cudaMemcpy(ctx->flags, g.flags.data(), (size_t)nb * 4, cudaMemcpyHostToDevice), "upload flags");

    // Ghost lists. FP64 keeps the reference's weights exactly (trilinear for
    // every entry whose weights are not all exactly zero). The mixed path snaps
    // weights within 1e-6 of 0 or 1 (an error of 1e-6*|du|, far below FP32
    // resolution of the stencil inputs' differences) so aligned neighbours
    // become plain copies and radial neighbours of other spacing 1-D blends.
    // Two sets: every ghost cell (the exchange that ends a step) and the face
    // ghosts the stage kernel does not push (the exchanges between stages).
    const bool snap = ctx->mixed();
    const int n3[3] = {g.ni, g.nj, g.nk};
    struct GE {
        int32_t d, src;
        double w[3];
        int nz, face;             // face: 2*axis + side of the target, -1 for edges and corners
        int32_t tb, sb, t[3], base[3];
        bool rotate;
        double rot[2];
    };
    // one derived entry per ghost, in parallel into uninitialised storage
    std::vector<GE, DefaultInitAlloc<GE>> ges(g.ghosts.size());
#pragma omp parallel for schedule(static)
    for (long k = 0; k < (long)g.ghosts.size(); ++k) {
        const auto& e = g.ghosts[k];
        GE q{};
        q.base[0] = e.i0; q.base[1] = e.j0; q.base[2] = e.k0;
        q.w[0] = e.w[0]; q.w[1] = e.w[1]; q.w[2] = e.w[2];
        if (snap)
            for (int a = 0; a < 3; ++a) {
                if (q.w[a] < 1e-6) q.w[a] = 0.0;
                else if (q.w[a] > 1.0 - 1e-6) { q.w[a] = 0.0; q.base[a] += 1; }
            }
        q.nz = (q.w[0] != 0.0) + (q.w[1] != 0.0) + (q.w[2] != 0.0);
        q.tb = e.e.tblock; q.sb = e.e.sblock;
        q.t[0] = e.e.ti; q.t[1] = e.e.tj; q.t[2] = e.e.tk;
        q.d = (int32_t)cell_off(g, q.tb, q.t[0], q.t[1], q.t[2]);
        q.src = (int32_t)cell_off(g, q.sb, q.base[0], q.base[1], q.base[2]);
        q.rotate = e.rotate;
        q.rot[0] = e.rotate ? e.rot[0] : 0.0;
        q.rot[1] = e.rotate ? e.rot[1] : 0.0;
        int nghost = 0, axis = -1, side = 0;
        for (int a = 0; a < 3; ++a)
            if (q.t[a] < 1 || q.t[a] > n3[a]) { ++nghost; axis = a; side = q.t[a] > n3[a]; }
        q.face = nghost == 1 ? 2 * axis + side : -1;
        ges[k] = q;
    }
    // the entries of a target block are contiguous (canonical order): segments
    std::vector<size_t> seg((size_t)nb + 1, 0);
    for (size_t k = 0; k < ges.size(); ++k) ++seg[(size_t)ges[k].tb + 1];
    for (int b = 0; b < nb; ++b) seg[b + 1] += seg[b];
    for (size_t k = 1; k < ges.size(); ++k)
        if (ges[k].tb < ges[k - 1].tb) return ctx->fail(FALCON_ERR_INVALID_ARG, "ghost map not in target-block order");

    // Faces pushed by the stage kernel (mixed path): every ghost cell of the
    // target face from one source block, no rotation; theta/phi: plain copies
    // shifted by the block extent; radial: same (j,k), one blend per layer.
    std::vector<int32_t> ptgt((size_t)nb * 6, -1), prsrc((size_t)nb * 4, 0), prdst((size_t)nb * 4, 0);
    std::vector<float> prw((size_t)nb * 4, 0.f);
    std::vector<uint8_t> pushed(ges.size(), 0);
    if (snap) {
        struct FaceState { int32_t sb = -1; bool ok = true; int64_t count = 0; int32_t rsrc[2] = {-1, -1}; double rw[2] = {0, 0}; };
        std::vector<FaceState> fs((size_t)nb * 6);
#pragma omp parallel for schedule(dynamic, 16)
        for (int tb = 0; tb < nb; ++tb)
          for (size_t k = seg[tb]; k < seg[tb + 1]; ++k) {
            const GE& q = ges[k];
            if (q.face < 0) continue;
            FaceState& f = fs[(size_t)q.tb * 6 + q.face];
            if (!f.ok) continue;
            const int a = q.face / 2, side = q.face % 2;
            bool ok = !q.rotate && (f.sb < 0 || f.sb == q.sb) && q.sb != q.tb;
            for (int c = 0; c < 3 && ok; ++c) {
                if (c == a) continue;
                ok = q.base[c] == q.t[c] && q.w[c] == 0.0;
            }
            if (ok && a != 0) ok = q.nz == 0 && q.base[a] - q.t[a] == (side == 0 ? n3[a] : -n3[a]);
            if (ok && a == 0) {
                const int layer = (q.t[0] == (side == 0 ? -1 : n3[0] + 1)) ? 0 : 1;
                const int32_t sp = q.base[0] + 1;   // padded
                const bool inb = q.w[0] == 0.0 ? (sp >= 2 && sp <= n3[0] + 1) : (sp >= 2 && sp <= n3[0]);
                if (!inb) ok = false;
                else if (f.rsrc[layer] < 0) { f.rsrc[layer] = sp; f.rw[layer] = q.w[0]; }
                else ok = f.rsrc[layer] == sp && f.rw[layer] == q.w[0];
            }
            if (!ok) { f.ok = false; continue; }
            f.sb = q.sb;
            ++f.count;
        }
        for (int tb = 0; tb < nb; ++tb)
            for (int face = 0; face < 6; ++face) {
                FaceState& f = fs[(size_t)tb * 6 + face];
                const int a = face / 2, side = face % 2;
                const int64_t full = 2LL * (a == 0 ? n3[1] * n3[2] : a == 1 ? n3[0] * n3[2] : n3[0] * n3[1]);
                if (!f.ok || f.sb < 0 || f.count != full) { f.ok = false; continue; }
                const size_t slot = (size_t)f.sb * 6 + 2 * a + (1 - side);   // the source's side facing the target
                if (ptgt[slot] >= 0) { f.ok = false; continue; }
                ptgt[slot] = tb;
                if (a == 0)
                    for (int layer = 0; layer < 2; ++layer) {
                        const size_t r = ((size_t)f.sb * 2 + (1 - side)) * 2 + layer;
                        prsrc[r] = f.rsrc[layer];
                        prw[r] = (float)f.rw[layer];
                        // padded target index of the layer: side 0 -> Fortran -1, 0; side 1 -> n+1, n+2
                        prdst[r] = side == 0 ? (layer == 0 ? 0 : 1) : (layer == 0 ? n3[0] + 2 : n3[0] + 3);
                    }
                ++ctx->pushed_faces;
            }
        int64_t pc = 0;
#pragma omp parallel for schedule(static) reduction(+ : pc)
        for (long k = 0; k < (long)ges.size(); ++k) {
            const GE& q = ges[k];
            if (q.face >= 0 && fs[(size_t)q.tb * 6 + q.face].ok) { pushed[k] = 1; ++pc; }
        }
        ctx->pushed_cells += pc;
    }

    auto up = [&](auto** dptr, const auto& vec) -> cudaError_t {
        using E = typename std::remove_reference<decltype(vec)>::type::value_type;
        cudaError_t e = ctx->alloc(dptr, vec.size() * sizeof(E));
        if (e == cudaSuccess && !vec.empty()) e = cudaMemcpy(*dptr, vec.data(), vec.size() * sizeof(E), cudaMemcpyHostToDevice);
        return e;
    };
    const int32_t strides[3] = {1, g.nip, g.nip * g.njp};
    // build and upload one set of lists over the entries `keep` selects
    auto build_lists = [&](auto keep, GhostLists& out, int64_t* counts) -> cudaError_t {
        struct Lin { int32_t d, s, st; float w; };
        // kind of an entry: 0 copy, 1 one-direction blend (mixed), 2 general
        auto kind = [&](const GE& q) { return (!q.rotate && q.nz == 0) ? 0 : (snap && !q.rotate && q.nz == 1) ? 1 : 2; };
        // per target block counts, offsets, then a parallel fill (blocks are
        // contiguous and their target offsets ascend with the block)
        std::vector<size_t> oc((size_t)nb + 1, 0), ol((size_t)nb + 1, 0), oi((size_t)nb + 1, 0);
#pragma omp parallel for schedule(dynamic, 16)
        for (int b = 0; b < nb; ++b) {
            size_t n3k[3] = {0, 0, 0};
            for (size_t k = seg[b]; k < seg[b + 1]; ++k)
                if (keep(k)) ++n3k[kind(ges[k])];
            oc[b + 1] = n3k[0]; ol[b + 1] = n3k[1]; oi[b + 1] = n3k[2];
        }
        for (int b = 0; b < nb; ++b) { oc[b + 1] += oc[b]; ol[b + 1] += ol[b]; oi[b + 1] += oi[b]; }
        std::vector<std::pair<int32_t, int32_t>> copies(oc[nb]);
        std::vector<Lin> lins(ol[nb]);
        std::vector<int32_t> idst(oi[nb]), isrc(oi[nb]);
        std::vector<double> iw(3 * oi[nb]), irot(2 * oi[nb]);
        std::vector<uint8_t> ikind(oi[nb]);
#pragma omp parallel for schedule(dynamic, 16)
        for (int b = 0; b < nb; ++b) {
            size_t c = oc[b], l = ol[b], i = oi[b];
            for (size_t k = seg[b]; k < seg[b + 1]; ++k) {
                if (!keep(k)) continue;
                const GE& q = ges[k];
                const int kd = kind(q);
                if (kd == 0) { copies[c++] = {q.d, q.src}; continue; }
                if (kd == 1) {
                    const int a = q.w[0] != 0.0 ? 0 : (q.w[1] != 0.0 ? 1 : 2);
                    lins[l++] = Lin{q.d, q.src, strides[a], (float)q.w[a]};
                    continue;
                }
                idst[i] = q.d;
                isrc[i] = q.src;
                for (int t = 0; t < 3; ++t) iw[3 * i + t] = q.w[t];
                irot[2 * i] = q.rot[0];
                irot[2 * i + 1] = q.rot[1];
                ikind[i] = (uint8_t)((q.nz ? 1 : 0) | (q.rotate ? 2 : 0));
                ++i;
            }
            std::sort(copies.begin() + (long)oc[b], copies.begin() + (long)oc[b + 1]);
            std::sort(lins.begin() + (long)ol[b], lins.begin() + (long)ol[b + 1],
                      [](const Lin& x, const Lin& y) { return x.d < y.d; });
        }
        {   // interpolated entries in target order: a warp's eight stores per
            // entry then write neighbouring ghost cells (its gathers still read
            // neighbouring source rows; measured faster than source order)
            std::vector<size_t> ord(idst.size());
            for (size_t q = 0; q < ord.size(); ++q) ord[q] = q;
            std::stable_sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return idst[a] < idst[b]; });
            std::vector<int32_t> d2(ord.size()), s2(ord.size());
            std::vector<double> w2(3 * ord.size()), r2(2 * ord.size());
            std::vector<uint8_t> k2(ord.size());
            for (size_t q = 0; q < ord.size(); ++q) {
                const size_t o = ord[q];
                d2[q] = idst[o];
                s2[q] = isrc[o];
                for (int t = 0; t < 3; ++t) w2[3 * q + t] = iw[3 * o + t];
                for (int t = 0; t < 2; ++t) r2[2 * q + t] = irot[2 * o + t];
                k2[q] = ikind[o];
            }
            idst.swap(d2);
            isrc.swap(s2);
            iw.swap(w2);
            irot.swap(r2);
            ikind.swap(k2);
        }
        std::vector<int32_t> cdst(copies.size()), csrc(copies.size());
        for (size_t q = 0; q < copies.size(); ++q) { cdst[q] = copies[q].first; csrc[q] = copies[q].second; }
        std::vector<int32_t> ldst(lins.size()), lsrc(lins.size()), lst(lins.size());
        std::vector<float> lw(lins.size());
        for (size_t q = 0; q < lins.size(); ++q) { ldst[q] = lins[q].d; lsrc[q] = lins[q].s; lst[q] = lins[q].st; lw[q] = lins[q].w; }
        int32_t *cp_dst, *cp_src, *ln_dst, *ln_src, *ln_st, *ip_dst, *ip_src;
        float* ln_w;
        double *ip_w, *ip_rot;
        uint8_t* ip_kind;
        cudaError_t e = up(&cp_dst, cdst);
        if (e == cudaSuccess) e = up(&cp_src, csrc);
        if (e == cudaSuccess) e = up(&ln_dst, ldst);
        if (e == cudaSuccess) e = up(&ln_src, lsrc);
        if (e == cudaSuccess) e = up(&ln_st, lst);
        if (e == cudaSuccess) e = up(&ln_w, lw);
        if (e == cudaSuccess) e = up(&ip_dst, idst);
        if (e == cudaSuccess) e = up(&ip_src, isrc);
        if (e == cudaSuccess) e = up(&ip_w, iw);
        if (e == cudaSuccess) e = up(&ip_rot, irot);
        if (e == cudaSuccess) e = up(&ip_kind, ikind);
        if (e != cudaSuccess) return e;
        out.cp = GhostCopyList{(int64_t)cdst.size(), cp_dst, cp_src};
        out.ln = GhostLinList{(int64_t)ldst.size(), ln_dst, ln_src, ln_st, ln_w};
        float *ip_wf = nullptr, *ip_rotf = nullptr;
        if (snap) {
            std::vector<float> wf(iw.begin(), iw.end()), rf(irot.begin(), irot.end());
            e = up(&ip_wf, wf);
            if (e == cudaSuccess) e = up(&ip_rotf, rf);
            if (e != cudaSuccess) return e;
        }
        out.ip = GhostInterpList{(int64_t)idst.size(), ip_dst, ip_src, ip_w, ip_rot, ip_kind, ip_wf, ip_rotf};
        counts[0] = (int64_t)cdst.size();
        counts[1] = (int64_t)ldst.size();
        counts[2] = (int64_t)idst.size();
        return cudaSuccess;
    };
    CK(build_lists([&](size_t) { return true; }, ctx->gl, ctx->ghost_counts), "upload ghosts");
    // The exchange ending a mixed step: every face entry not pushed by the
    // diffusion pass, plus the theta-phi edge ghosts of the two planes next to
    // a radial boundary (the boundary condition of the next stage 1 mirrors
    // those planes whole). No kernel of a step reads the other edge and
    // corner ghosts; they are filled before the state is read (fresh_state).
    if (snap) {
        auto bc_edge = [&](const GE& q) {
            const int fl = g.flags[q.tb];
            const bool jg = q.t[1] < 1 || q.t[1] > n3[1], kg = q.t[2] < 1 || q.t[2] > n3[2];
            if (!jg || !kg) return false;
            return ((fl & 4) && (q.t[0] == 1 || q.t[0] == 2)) || ((fl & 2) && (q.t[0] == n3[0] || q.t[0] == n3[0] - 1));
        };
        CK(build_lists([&](size_t k) { return !pushed[k] && (ges[k].face >= 0 || bc_edge(ges[k])); }, ctx->gl_final,
                       ctx->final_counts),
           "upload final ghosts");
    }
    CK(build_lists([&](size_t k) { return ges[k].face >= 0 && !pushed[k]; }, ctx->gl_stage, ctx->stage_counts),
       "upload stage ghosts");
    if (snap) {
        int32_t *d_tgt, *d_rsrc, *d_rdst;
        float* d_rw;
        CK(up(&d_tgt, ptgt), "upload push table");
        CK(up(&d_rsrc, prsrc), "upload push table");
        CK(up(&d_rdst, prdst), "upload push table");
        CK(up(&d_rw, prw), "upload push table");
        ctx->push = PushTable{d_tgt, d_rsrc, d_rdst, d_rw};
        CK(ctx->alloc(&ctx->R2, sbytes), "alloc R2");
        CK(cudaMemsetAsync(ctx->R2, 0, sbytes, ctx->st), "memset");
    }

    StepScalars s0{};
    s0.min_ratio_bits = 0x7FF0000000000000ull;
    s0.cfl = ctx->cfg.phys.cfl;
    s0.nan_step = -1;
    s0.wait_polls = kDefaultWaitPolls;
    CK(ctx->alloc(&ctx->sc, sizeof(StepScalars)), "alloc scalars");
    CK(cudaMemcpy(ctx->sc, &s0, sizeof s0, cudaMemcpyHostToDevice), "upload scalars");
    CK(cudaStreamSynchronize(ctx->st), "sync");
    ctx->on_device = true;
    return FALCON_OK;
}

int need_device(falcon_ctx* ctx) {
    if (!ctx) return FALCON_ERR_INVALID_ARG;
    if (!ctx->on_device) return ctx->fail(FALCON_ERR_NO_DEVICE, "context was created without a device");
    cudaSetDevice(ctx->device);
    return FALCON_OK;
}

}  // namespace

extern "C" {

int falcon_create(falcon_ctx** out, const falcon_config* cfg) {
    if (!out || !cfg) return FALCON_ERR_INVALID_ARG;
    falcon_ctx* ctx = new falcon_ctx();
    *out = ctx;
    ctx->cfg = *cfg;
    if (cfg->precision != FALCON_PREC_FP64 && cfg->precision != FALCON_PREC_MIXED)
        return ctx->fail(FALCON_ERR_INVALID_ARG, "unknown precision mode");
    if (!(cfg->phys.cfl > 0.0)) return ctx->fail(FALCON_ERR_INVALID_ARG, "cfl must be positive");
    std::string e = ctx->grid.build(*cfg);
    if (!e.empty()) return ctx->fail(e.find("owner") != std::string::npos ? FALCON_ERR_UNCOVERED_GHOST : FALCON_ERR_INVALID_ARG, e);
    if (cfg->device < 0) return FALCON_OK;
    return setup_device(ctx);
}

void falcon_destroy(falcon_ctx* ctx) {
    if (!ctx) return;
    if (ctx->on_device) {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->st);
        for (auto& row : ctx->graphs)
            for (cudaGraphExec_t& gx : row)
                if (gx) cudaGraphExecDestroy(gx);
        for (auto& r : ctx->pending) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
        for (auto e : ctx->pool) cudaEventDestroy(e);
        for (void* p : ctx->allocs) cudaFree(p);
        if (ctx->t0) cudaEventDestroy(ctx->t0);
        if (ctx->t1) cudaEventDestroy(ctx->t1);
        cudaStreamDestroy(ctx->st);
    }
    delete ctx;
}

int falcon_last_error(const falcon_ctx* ctx, char* buf, size_t len) {
    if (!ctx || !buf || len == 0) return FALCON_ERR_INVALID_ARG;
    snprintf(buf, len, "%s", ctx->err.c_str());
    return FALCON_OK;
}

int falcon_num_blocks(const falcon_ctx* ctx, int32_t* nb, int32_t* ny) {
    if (!ctx || !nb || !ny) return FALCON_ERR_INVALID_ARG;
    *nb = ctx->grid.nblocks;
    *ny = ctx->grid.nblocks_yin;
    return FALCON_OK;
}

int falcon_block_ranges(const falcon_ctx* ctx, double* r) {
    if (!ctx || !r) return FALCON_ERR_INVALID_ARG;
    std::memcpy(r, ctx->grid.ranges.data(), ctx->grid.ranges.size() * sizeof(double));
    return FALCON_OK;
}

int falcon_block_flags(const falcon_ctx* ctx, int32_t* f) {
    if (!ctx || !f) return FALCON_ERR_INVALID_ARG;
    std::memcpy(f, ctx->grid.flags.data(), ctx->grid.flags.size() * sizeof(int32_t));
    return FALCON_OK;
}

int falcon_get_background(const falcon_ctx* ctx, double* p) {
    if (!ctx || !p) return FALCON_ERR_INVALID_ARG;
    std::memcpy(p, ctx->grid.prof.data(), ctx->grid.prof.size() * sizeof(double));
    return FALCON_OK;
}

int falcon_set_background(falcon_ctx* ctx, const double* p) {
    if (!ctx || !p) return FALCON_ERR_INVALID_ARG;
    Grid& g = ctx->grid;
    const size_t n = g.prof.size();
    // the derived tables divide by rho0, rho0*T0 and Xi, and take sqrt(gamma1 p0/rho0)
    for (int b = 0; b < g.nblocks; ++b)
        for (int i = 0; i < g.nip; ++i) {
            const double* P = p + (size_t)b * FALCON_NPROF * g.nip + i;
            bool ok = true;
            for (int q = 0; q < FALCON_NPROF; ++q) ok = ok && std::isfinite(P[(size_t)q * g.nip]);
            ok = ok && P[1 * g.nip] > 0 && P[2 * g.nip] > 0 && P[3 * g.nip] > 0 && P[4 * g.nip] > 0 && P[8 * g.nip] > 0;
            if (!ok)
                return ctx->fail(FALCON_ERR_INVALID_ARG, "falcon_set_background: block " + std::to_string(b) + " cell " +
                                                              std::to_string(i) +
                                                              ": profiles must be finite with rho0, p0, T0, gamma1, Xi > 0");
        }
    std::memcpy(g.prof.data(), p, n * sizeof(double));
    if (!ctx->on_device) return FALCON_OK;
    cudaSetDevice(ctx->device);
    const int rc = upload_tables(ctx, false);
    if (rc) return rc;
    CK(drop_pending_cfl(ctx), "background");   // the wave speed changed with the background
    CK(cudaStreamSynchronize(ctx->st), "background");
    return FALCON_OK;
}

int falcon_ghost_count(const falcon_ctx* ctx, int64_t* n) {
    if (!ctx || !n) return FALCON_ERR_INVALID_ARG;
    *n = (int64_t)ctx->grid.ghosts.size();
    return FALCON_OK;
}

int falcon_ghost_map(const falcon_ctx* ctx, falcon_ghost_entry* out, int64_t cap) {
    if (!ctx || !out) return FALCON_ERR_INVALID_ARG;
    if (cap < (int64_t)ctx->grid.ghosts.size()) return FALCON_ERR_BOUNDS;
    for (size_t q = 0; q < ctx->grid.ghosts.size(); ++q) out[q] = ctx->grid.ghosts[q].e;
    return FALCON_OK;
}

// Host block arrays are [b][FALCON_NVAR = 9][cell] (psi last, as the
// reference's MHD block); the device keeps the 8 evolved variables as
// [b][8][cell] and psi in an array of its own when GLM is on.
namespace {
size_t host_elems(const falcon_ctx* ctx) { return (size_t)ctx->dims.nblocks * FALCON_NVAR * ctx->dims.ncell; }

// Device address of the host range [p, p + bytes) when it lies inside one
// buffer pinned through falcon_pin_host: the GPU then reads or writes it in
// place over the host link (NVLink-C2C on GB300), with no staging copy.
// Any other host memory gives nullptr (staged through device memory).
void* mapped_host(falcon_ctx* ctx, const void* p, size_t bytes) {
    const uintptr_t a = (uintptr_t)p;
    for (const auto& r : ctx->pinned)
        if (a >= r.first && a + bytes <= r.first + r.second) {
            void* d = nullptr;
            if (cudaHostGetDevicePointer(&d, (void*)r.first, 0) != cudaSuccess || !d) {
                cudaGetLastError();
                return nullptr;
            }
            return (char*)d + (a - r.first);
        }
    return nullptr;
}

int put_state(falcon_ctx* ctx, const double* u, void* U, int8_t* lo, void* P) {
    const size_t nb = (size_t)ctx->dims.nblocks, nc = (size_t)ctx->dims.ncell;
    // psi is not evolved without GLM: it must be 0, as it then stays in the
    // reference (checked before anything on the device changes)
    const char* psi_msg = "psi must be 0 unless divb_option = 1";
    if (ctx->mixed()) {
        const size_t n9 = host_elems(ctx);
        if (!ctx->dflag) CK(ctx->alloc(&ctx->dflag, sizeof(int32_t)), "alloc flag");
        const double* src = (const double*)mapped_host(ctx, u, n9 * 8);
        if (!src) {
            if (!ctx->stage64) CK(ctx->alloc(&ctx->stage64, n9 * 8), "alloc staging");
            CK(cudaMemcpyAsync(ctx->stage64, u, n9 * 8, cudaMemcpyHostToDevice, ctx->st), "upload");
            src = ctx->stage64;
        }
        if (!P) {
            int32_t bad = 0;
            CK(launch_psi_nonzero(src, (int64_t)nb, (int64_t)nc, ctx->dflag, ctx->st), "upload check");
            CK(cudaMemcpyAsync(&bad, ctx->dflag, sizeof bad, cudaMemcpyDeviceToHost, ctx->st), "upload check");
            CK(cudaStreamSynchronize(ctx->st), "upload check");
            if (bad) return ctx->fail(FALCON_ERR_INVALID_ARG, psi_msg);
        }
        CK(launch_convert_state(src, (float*)U, lo, (int64_t)(nb * NV * nc), ctx->dims, ctx->st), "upload convert");
        if (P) CK(launch_convert_psi(src, (float*)P, (int64_t)nb, (int64_t)nc, ctx->st), "upload convert");
    } else {
        if (!P) {
            int bad = 0;
#pragma omp parallel for reduction(| : bad) schedule(static)
            for (long b = 0; b < (long)nb; ++b) {
                const double* q = u + ((size_t)b * FALCON_NVAR + NV) * nc;
                for (size_t c = 0; c < nc; ++c) bad |= q[c] != 0.0;
            }
            if (bad) return ctx->fail(FALCON_ERR_INVALID_ARG, psi_msg);
        }
        CK(cudaMemcpy2DAsync(U, NV * nc * 8, u, FALCON_NVAR * nc * 8, NV * nc * 8, nb, cudaMemcpyHostToDevice, ctx->st),
           "upload");
        if (P)
            CK(cudaMemcpy2DAsync(P, nc * 8, u + NV * nc, FALCON_NVAR * nc * 8, nc * 8, nb, cudaMemcpyHostToDevice, ctx->st),
               "upload");
    }
    return FALCON_OK;
}

int get_state(falcon_ctx* ctx, const void* U, const int8_t* lo, const void* P, double* u) {
    const size_t nb = (size_t)ctx->dims.nblocks, nc = (size_t)ctx->dims.ncell;
    if (ctx->mixed()) {
        const size_t n9 = host_elems(ctx);
        double* dst = (double*)mapped_host(ctx, u, n9 * 8);
        if (dst) {
            CK(launch_gather_host(U, lo, P, true, ctx->dims, 0, (int64_t)n9, (int64_t)nc, dst, ctx->st), "download convert");
        } else {
            if (!ctx->stage64) CK(ctx->alloc(&ctx->stage64, n9 * 8), "alloc staging");
            CK(launch_gather_host(U, lo, P, true, ctx->dims, 0, (int64_t)n9, (int64_t)nc, ctx->stage64, ctx->st),
               "download convert");
            CK(cudaMemcpyAsync(u, ctx->stage64, n9 * 8, cudaMemcpyDeviceToHost, ctx->st), "download");
        }
        CK(cudaStreamSynchronize(ctx->st), "download");
    } else {
        CK(cudaMemcpy2DAsync(u, FALCON_NVAR * nc * 8, U, NV * nc * 8, NV * nc * 8, nb, cudaMemcpyDeviceToHost, ctx->st),
           "download");
        if (P)
            CK(cudaMemcpy2DAsync(u + NV * nc, FALCON_NVAR * nc * 8, P, nc * 8, nc * 8, nb, cudaMemcpyDeviceToHost, ctx->st),
               "download");
        CK(cudaStreamSynchronize(ctx->st), "download");
        if (!P)
            for (size_t b = 0; b < nb; ++b) std::memset(u + (b * FALCON_NVAR + NV) * nc, 0, nc * 8);
    }
    return FALCON_OK;
}
}  // namespace

int falcon_upload_state(falcon_ctx* ctx, const double* u) {
    int rc = need_device(ctx);
    if (rc) return rc;
    if (!u) return ctx->fail(FALCON_ERR_INVALID_ARG, "null state");
    rc = put_state(ctx, u, ctx->U, ctx->Ulo, ctx->P);
    if (rc) return rc;
    ctx->stale_edges = false;   // the uploaded ghost cells are the state's
    CK(drop_pending_cfl(ctx), "upload");
    CK(clear_step_flags(ctx), "upload");
    // primitive_rk_IV = primitive_IV, as the reference's initialisation leaves it
    CK(mirror_state(ctx, true), "upload");
    // psi's stage array and the scratch it is copied from start equal too:
    // their ghost cells that no exchange writes (the radial boundary planes)
    // then stay at the uploaded values, as the reference's arrays do.
    if (ctx->P)
        for (void* q : {ctx->Prk, ctx->P2})
            CK(cudaMemcpyAsync(q, ctx->P, (size_t)ctx->dims.nblocks * ctx->dims.ncell * ctx->elem,
                               cudaMemcpyDeviceToDevice, ctx->st), "upload");
    CK(cudaStreamSynchronize(ctx->st), "upload");
    return FALCON_OK;
}

int falcon_download_state(falcon_ctx* ctx, double* u) {
    int rc = need_device(ctx);
    if (rc) return rc;
    if (!u) return ctx->fail(FALCON_ERR_INVALID_ARG, "null state");
    CK(fresh_state(ctx), "ghost fill");
    return get_state(ctx, ctx->U, ctx->Ulo, ctx->P, u);
}

int falcon_download_state_range(falcon_ctx* ctx, size_t first, size_t count, double* u) {
    int rc = need_device(ctx);
    if (rc) return rc;
    if (!u && count) return ctx->fail(FALCON_ERR_INVALID_ARG, "null state");
    // the size checks need only the host layout: a rejected call does no device work
    const size_t n = host_elems(ctx);
    const size_t cap = static_scratch_elems();
    if (count > cap)
        return ctx->fail(FALCON_ERR_INVALID_ARG,
                         "falcon_download_state_range: count " + std::to_string(count) +
                             " exceeds the static scratch limit of " + std::to_string(cap) + " elements (" +
                             std::to_string(FALCON_STATIC_SCRATCH_BYTES >> 20) + " MiB); download in smaller ranges");
    if (first > n || count > n - first)
        return ctx->fail(FALCON_ERR_INVALID_ARG, "falcon_download_state_range: first " + std::to_string(first) +
                                                     " + count " + std::to_string(count) + " exceeds the state size " +
                                                     std::to_string(n));
    CK(fresh_state(ctx), "ghost fill");
    const std::string e = download_range_static(ctx->device, ctx->st, ctx->U, ctx->Ulo, ctx->P, ctx->mixed(), ctx->dims,
                                                first, count, u);
    if (!e.empty()) return ctx->fail(FALCON_ERR_CUDA, e);
    return FALCON_OK;
}

// Core transfers: only the interior planes x interior rows of the host array
// move (64% of a 16^3 block's padded cells); the theta/phi ghost layers are
// recomputed on the device by a full exchange (upload) or left as they are
// in host memory (download). They need the array pinned with falcon_pin_host
// (read and written in place over the host link); otherwise, and for an
// upload into a context without a second state buffer (FP64 path), the full
// transfer runs instead.
int falcon_upload_state_core(falcon_ctx* ctx, const double* u) {
    int rc = need_device(ctx);
    if (rc) return rc;
    if (!u) return ctx->fail(FALCON_ERR_INVALID_ARG, "null state");
    const double* src = (const double*)mapped_host(ctx, u, host_elems(ctx) * 8);
    if (!src || !ctx->mixed() || !ctx->R2 || ((uintptr_t)src % 16) != 0) return falcon_upload_state(ctx, u);
    // into the second state buffer (and the stage buffer as int8 scratch for
    // the corrections), so that a rejected array (psi not 0) leaves the state
    // as it was
    if (!ctx->dflag) CK(ctx->alloc(&ctx->dflag, sizeof(int32_t)), "alloc flag");
    int8_t* lo_tmp = (int8_t*)ctx->RK;
    CK(launch_core_up(src, ctx->R2, lo_tmp, ctx->P ? ctx->P2 : nullptr, ctx->P ? nullptr : ctx->dflag, true, ctx->dims,
                      ctx->st),
       "upload core");
    int32_t bad = 0;
    if (!ctx->P) CK(cudaMemcpyAsync(&bad, ctx->dflag, sizeof bad, cudaMemcpyDeviceToHost, ctx->st), "upload core");
    CK(cudaStreamSynchronize(ctx->st), "upload core");
    if (bad) {   // the state is kept; both buffers written above start again from it
        CK(mirror_state(ctx, true), "upload core");
        CK(cudaStreamSynchronize(ctx->st), "upload core");
        return ctx->fail(FALCON_ERR_INVALID_ARG, "psi must be 0 unless divb_option = 1");
    }
    std::swap(ctx->U, ctx->R2);
    CK(cudaMemcpyAsync(ctx->Ulo, lo_tmp, lo_elems(ctx->dims), cudaMemcpyDeviceToDevice, ctx->st), "upload core");
    CK(launch_clear_outside_core_mixed(ctx->dims, (float*)ctx->U, NV, ctx->st), "upload core");
    if (ctx->P) CK(launch_clear_outside_core_mixed(ctx->dims, (float*)ctx->P2, 1, ctx->st), "upload core");
    CK(clear_step_flags(ctx), "upload core");
    CK(drop_pending_cfl(ctx), "upload core");
    // what the diffusion pass closing a step leaves besides u^{n+1}: the
    // regular faces pushed by k_push_state (which also forms the next step's
    // CFL minimum, so the step that follows skips k_cfl) and the other face
    // entries of the final exchange; edge and corner ghosts stay at the 0 set
    // above until the state is read (fresh_state)
    CK(launch_push_state_mixed(ctx->dims, ctx->geom(), (float*)ctx->U, ctx->push, ctx->sc, ctx->st), "upload core");
    CK(launch_ghost_mixed(ctx->dims, ctx->gl_final, (float*)ctx->U, ctx->st), "upload core");
    ctx->stale_edges = true;
    ctx->cfl_ready = true;
    // the stage buffer and the second state buffer start as copies of the
    // state: ghost cells that a step reads without rewriting (with weight 0
    // in an interpolation) hold its finite values, not the corrections staged
    // in the stage buffer or an earlier state's
    CK(mirror_state(ctx, true), "upload core");
    if (ctx->P) {
        const size_t np = (size_t)ctx->dims.nblocks * ctx->dims.ncell * ctx->elem;
        CK(cudaMemcpyAsync(ctx->P, ctx->P2, np, cudaMemcpyDeviceToDevice, ctx->st), "upload core");
        CK(launch_psi_ghost_mixed(ctx->dims, ctx->gl, (float*)ctx->P, ctx->st), "upload core");
        for (void* q : {ctx->Prk, ctx->P2}) CK(cudaMemcpyAsync(q, ctx->P, np, cudaMemcpyDeviceToDevice, ctx->st), "upload core");
    }
    CK(cudaStreamSynchronize(ctx->st), "upload core");
    return FALCON_OK;
}

int falcon_download_state_core(falcon_ctx* ctx, double* u) {
    int rc = need_device(ctx);
    if (rc) return rc;
    if (!u) return ctx->fail(FALCON_ERR_INVALID_ARG, "null state");
    double* dst = (double*)mapped_host(ctx, u, host_elems(ctx) * 8);
    if (!dst || ((uintptr_t)dst % 16) != 0) return falcon_download_state(ctx, u);
    // the core cells are current after a step (its last exchange and the
    // radial boundary copy cover them); only edge ghosts are left stale
    CK(launch_core_down(ctx->U, ctx->mixed() ? ctx->Ulo : nullptr, ctx->P, ctx->mixed(), dst, ctx->dims, ctx->st),
       "download core");
    CK(cudaStreamSynchronize(ctx->st), "download core");
    return FALCON_OK;
}

int falcon_pin_host(falcon_ctx* ctx, void* p, size_t bytes) {
    int rc = need_device(ctx);
    if (rc) return rc;
    if (!p || !bytes) return ctx->fail(FALCON_ERR_INVALID_ARG, "null buffer");
    CK(cudaHostRegister(p, bytes, cudaHostRegisterMapped), "cudaHostRegister");
    ctx->pinned.push_back({(uintptr_t)p, bytes});
    return FALCON_OK;
}

int falcon_unpin_host(falcon_ctx* ctx, void* p) {
    int rc = need_device(ctx);
    if (rc) return rc;
    CK(cudaHostUnregister(p), "cudaHostUnregister");
    for (size_t q = 0; q < ctx->pinned.size(); ++q)
        if (ctx->pinned[q].first == (uintptr_t)p) {
            ctx->pinned.erase(ctx->pinned.begin() + (long)q);
            break;
        }
    return FALCON_OK;
}

int falcon_init_synthetic(falcon_ctx* ctx, int32_t kind, uint64_t seed, double mach) {
    int rc = need_device(ctx);
    if (rc) return rc;
    if (kind < 0 || kind > 1) return ctx->fail(FALCON_ERR_INVALID_ARG, "unknown synthetic kind");
    std::string e = synth_initial_state(ctx->grid, ctx->geom(), ctx->U, ctx->mixed(), kind, seed, mach, ctx->st);
    if (!e.empty()) return ctx->fail(FALCON_ERR_CUDA, e);
    if (ctx->Ulo) CK(cudaMemsetAsync(ctx->Ulo, 0, lo_elems(ctx->dims), ctx->st), "init");
    CK(mirror_state(ctx, true), "init");
    ctx->stale_edges = false;
    CK(drop_pending_cfl(ctx), "init");
    CK(clear_step_flags(ctx), "init");
    CK(cudaStreamSynchronize(ctx->st), "init");
    return FALCON_OK;
}

int falcon_exchange(falcon_ctx* ctx) {
    int rc = need_device(ctx);
    if (rc) return rc;
    if (ctx->shard.on) {   // the entries within this rank; the others through falcon_shard_pack/unpack
        CK(launch_ghost_fp64(ctx->dims, ctx->shard.local, (double*)ctx->U, ctx->st), "ghost fill");
        ctx->shard.last_out = ctx->U;
        CK(cudaStreamSynchronize(ctx->st), "ghost fill");
        return FALCON_OK;
    }
    CK(ghost(ctx, ctx->U), "ghost fill");
    ctx->stale_edges = false;
    if (ctx->P)
        CK(ctx->mixed() ? launch_psi_ghost_mixed(ctx->dims, ctx->gl, (float*)ctx->P, ctx->st)
                        : launch_psi_ghost_fp64(ctx->dims, ctx->gl, (double*)ctx->P, ctx->st),
           "ghost fill");
    CK(cudaStreamSynchronize(ctx->st), "ghost fill");
    collect(ctx);
    return FALCON_OK;
}

int falcon_timestep(falcon_ctx* ctx, double* dt_out) {
    int rc = need_device(ctx);
    if (rc) return rc;
    CK(cfl(ctx), "cfl");
    double dt = 0;
    CK(cudaMemcpyAsync(&dt, &ctx->sc->dt, sizeof dt, cudaMemcpyDeviceToHost, ctx->st), "dt");
    CK(cudaStreamSynchronize(ctx->st), "dt");
    collect(ctx);
    if (dt_out) *dt_out = dt;
    return check_nan(ctx);
}

static int run(falcon_ctx* ctx, int32_t n) {
    int rc = autotune(ctx);
    if (rc) return rc;
    if (ctx->ktiming) {
        for (int32_t s = 0; s < n; ++s) {
            CK(enqueue_step(ctx), "step");
            end_step(ctx);
            ++ctx->steps_done;
        }
        return FALCON_OK;
    }
    if (ctx->step_mode == FALCON_STEP_PERSISTENT) {
        for (int32_t s = 0; s < n; ++s) {
            // the CFL minimum of u^n: formed by the previous step's diffusion
            // pass, else by k_cfl here (the persistent step starts at dt)
            if (!ctx->cfl_ready)
                CK(launch_cfl_mixed(ctx->dims, ctx->geom(), (const float*)ctx->U, ctx->sc, ctx->st), "cfl");
            CK(launch_step_persistent_mixed(ctx->dims, ctx->geom(), (float*)ctx->U, (float*)ctx->RK, (float*)ctx->R2,
                                            ctx->Ulo, ctx->push, ctx->gl_stage, ctx->gl_final, ctx->sc, ctx->gbar,
                                            ctx->st),
               "persistent step");
            end_step(ctx);
            ++ctx->steps_done;
        }
        return FALCON_OK;
    }
    for (int32_t s = 0; s < n; ++s) {
        cudaGraphExec_t& gx = ctx->graphs[ctx->U == ctx->bufA ? 0 : 1][ctx->cfl_ready ? 1 : 0];
        if (!gx) {
            cudaGraph_t gr;
            CK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal), "capture");
            cudaError_t e = enqueue_step(ctx);
            cudaError_t e2 = cudaStreamEndCapture(ctx->st, &gr);
            if (e != cudaSuccess) return ctx->cuda_fail(e, "capture step");
            if (e2 != cudaSuccess) return ctx->cuda_fail(e2, "end capture");
            CK(cudaGraphInstantiate(&gx, gr, 0), "instantiate");
            cudaGraphDestroy(gr);
        }
        CK(cudaGraphLaunch(gx, ctx->st), "graph launch");
        end_step(ctx);
        ++ctx->steps_done;
    }
    return FALCON_OK;
}

int falcon_step_rk4(falcon_ctx* ctx, double* dt_out) {
    int rc = need_device(ctx);
    if (rc) return rc;
    rc = run(ctx, 1);
    if (rc) return rc;
    if (dt_out) {
        CK(cudaMemcpyAsync(dt_out, &ctx->sc->dt, sizeof(double), cudaMemcpyDeviceToHost, ctx->st), "dt");
        CK(cudaStreamSynchronize(ctx->st), "dt");
        collect(ctx);
        return check_nan(ctx);
    }
    return FALCON_OK;
}

int falcon_run_steps(falcon_ctx* ctx, int32_t nsteps) {
    int rc = need_device(ctx);
    if (rc) return rc;
    if (nsteps < 0) return ctx->fail(FALCON_ERR_INVALID_ARG, "nsteps < 0");
    return run(ctx, nsteps);
}

// One phase over the owned blocks of a sharded context, then the exchange of
// the entries within the rank. Phase 0 only accumulates the owned blocks'
// CFL minimum (falcon_shard_min_ratio / falcon_shard_set_min_ratio finish dt
// after the MIN over ranks).
int shard_phase(falcon_ctx* ctx, int phase) {
    auto& S = ctx->shard;
    StepDims dl = ctx->dims;
    dl.nblocks = S.last - S.first;
    const Geometry gl = geom_from(ctx, S.first);
    const size_t off = (size_t)S.first * NV * ctx->dims.ncell;
    double* U = (double*)ctx->U;
    double* RK = (double*)ctx->RK;
    const DivBArgs none{nullptr, nullptr, nullptr, 0};
    cudaError_t e = cudaSuccess;
    if (phase == 0) {
        if (dl.nblocks > 0) e = launch_cfl_fp64(dl, gl, U + off, ctx->sc, ctx->st);
    } else if (phase <= 4) {
        const int s = phase;
        double* in = s == 1 ? U : RK;
        double* out = s < 4 ? RK : U;
        if (dl.nblocks > 0)
            e = launch_stage_fp64(dl, gl, in + off, U + off, out + off, none, s, 1, ctx->sc, 1, ctx->kpar_stage, ctx->st);
        if (e == cudaSuccess) e = launch_ghost_fp64(ctx->dims, S.local, out, ctx->st);
        S.last_out = out;
    } else {
        if (dl.nblocks > 0) e = launch_diffusion_fp64(dl, gl, U + off, ctx->sc, ctx->kpar_diff, ctx->st);
        if (e == cudaSuccess) e = launch_ghost_fp64(ctx->dims, S.local, U, ctx->st);
        S.last_out = U;
        ++ctx->steps_done;
    }
    if (e != cudaSuccess) return ctx->cuda_fail(e, "shard phase");
    CK(cudaStreamSynchronize(ctx->st), "shard phase");
    return FALCON_OK;
}

int falcon_step_phase(falcon_ctx* ctx, int32_t phase) {
    int rc = need_device(ctx);
    if (rc) return rc;
    if (phase < 0 || phase > 5) return ctx->fail(FALCON_ERR_INVALID_ARG, "phase must be 0..5");
    rc = autotune(ctx);
    if (rc) return rc;
    if (ctx->shard.on) return shard_phase(ctx, phase);
    CK(drop_pending_cfl(ctx), "phase");   // the phases change the state outside the fused step
    cudaError_t e = cudaSuccess;
    if (phase == 0) {
        e = cfl(ctx);
    } else if (phase <= 4) {
        const int s = phase;
        void* in = (s == 1) ? ctx->U : ctx->RK;
        void* out = (s < 4) ? ctx->RK : ctx->U;
        e = stage(ctx, s, in, out, PushTable{});
        if (e == cudaSuccess) e = ghost(ctx, out);
    } else {
        e = diffusion(ctx, ctx->U, PushTable{});
        if (e == cudaSuccess) e = ghost(ctx, ctx->U);
        if (e == cudaSuccess) {
            ++ctx->steps_done;
            ctx->stale_edges = false;
        }
    }
    if (e != cudaSuccess) return ctx->cuda_fail(e, "phase");
    CK(cudaStreamSynchronize(ctx->st), "phase");
    collect(ctx);
    return FALCON_OK;
}

int falcon_download_stage_state(falcon_ctx* ctx, double* u) {
    int rc = need_device(ctx);
    if (rc) return rc;
    if (!u) return ctx->fail(FALCON_ERR_INVALID_ARG, "null state");
    return get_state(ctx, ctx->RK, nullptr, ctx->Prk, u);
}

// ---- output and restart ----------------------------------------------------
namespace {
// Fortran ES16.8: d.ddddddddE+dd right-justified in 16 columns; with a
// three-digit exponent Fortran drops the E (d.dddddddd+ddd).
void es16_8(double x, char* o) {
    char buf[48];
    int n;
    if (std::isnan(x)) {
        n = snprintf(buf, sizeof buf, "NaN");
    } else if (std::isinf(x)) {
        n = snprintf(buf, sizeof buf, "%s", x > 0 ? "Infinity" : "-Infinity");
    } else {
        n = snprintf(buf, sizeof buf, "%.8E", x);
        char* e = std::strchr(buf, 'E');
        if (e && std::strlen(e + 2) == 3) {
            std::memmove(e, e + 1, std::strlen(e + 1) + 1);
            --n;
        }
    }
    if (n > 16) {
        std::memset(o, '*', 16);
        return;
    }
    std::memset(o, ' ', (size_t)(16 - n));
    std::memcpy(o + 16 - n, buf, (size_t)n);
}
// write(c,'(I8)') with the blanks turned into '0' (3_6/ModSavePlot.f90:536-539)
std::string i8_zero(long v) {
    char b[32];
    snprintf(b, sizeof b, "%8ld", v);
    for (char* c = b; *c; ++c)
        if (*c == ' ') *c = '0';
    return b;
}

struct RestartHeader {
    char magic[8];
    uint32_t version, precision;
    int32_t ni, nj, nk, ng, nblocks, divb_option;
    uint64_t grid_hash;
    int64_t steps_done;
    uint64_t bytes_state, bytes_lo, bytes_psi;
};
const char kRestartMagic[8] = {'F', 'A', 'L', 'C', 'R', 'S', 'T', '1'};

uint64_t grid_hash(const Grid& g) {   // FNV-1a over the block ranges and flags
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](const void* p, size_t n) {
        const unsigned char* c = (const unsigned char*)p;
        for (size_t q = 0; q < n; ++q) { h ^= c[q]; h *= 1099511628211ull; }
    };
    mix(g.ranges.data(), g.ranges.size() * sizeof(double));
    mix(g.flags.data(), g.flags.size() * sizeof(int32_t));
    return h;
}

RestartHeader restart_header(const falcon_ctx* ctx) {
    RestartHeader h{};
    std::memcpy(h.magic, kRestartMagic, 8);
    h.version = 2;   // 2: the u^n correction stored for interior cells only
    h.precision = (uint32_t)ctx->cfg.precision;
    h.ni = ctx->dims.ni; h.nj = ctx->dims.nj; h.nk = ctx->dims.nk; h.ng = ctx->grid.ng;
    h.nblocks = ctx->dims.nblocks;
    h.divb_option = ctx->cfg.phys.divb_option;
    h.grid_hash = grid_hash(ctx->grid);
    h.steps_done = ctx->steps_done;
    const size_t cells = (size_t)ctx->dims.nblocks * ctx->dims.ncell;
    h.bytes_state = cells * NV * ctx->elem;
    h.bytes_lo = ctx->Ulo ? lo_elems(ctx->dims) : 0;
    h.bytes_psi = ctx->P ? cells * ctx->elem : 0;
    return h;
}
constexpr size_t kIoChunk = 64u << 20;
}  // namespace

int falcon_save_allcells(falcon_ctx* ctx, const char* directory, int32_t step) {
    int rc = need_device(ctx);
    if (rc) return rc;
    if (!directory) return ctx->fail(FALCON_ERR_INVALID_ARG, "null directory");
    CK(fresh_state(ctx), "ghost fill");
    const Grid& g = ctx->grid;
    const StepDims& d = ctx->dims;
    const std::string dir = std::string(directory) + "/AllCells_" + i8_zero(step);
    std::error_code ec;
    std::filesystem::create_directories(dir, ec);
    if (ec) return ctx->fail(FALCON_ERR_INVALID_ARG, "cannot create " + dir + ": " + ec.message());
    {
        FILE* f = std::fopen((dir + "/info.dat").c_str(), "w");
        if (!f) return ctx->fail(FALCON_ERR_INVALID_ARG, "cannot write " + dir + "/info.dat");
        std::fprintf(f, "nBlocks = %d\nni = %d\nnj = %d\nnk = %d\nnVarsTotal = %d\n", g.nblocks, g.ni, g.nj, g.nk,
                     FALCON_NVAR + 3);
        std::fputs("VARIABLES = \"X [Rs]\", \"Y [Rs]\", \"Z [Rs]\", \"Rho1\", \"Vx\", \"Vy\", \"Vz\", "
                   "\"Bx\", \"By\", \"Bz\", \"S1\", \"PHI\"\n", f);
        if (std::fclose(f) != 0) return ctx->fail(FALCON_ERR_INVALID_ARG, "cannot write " + dir + "/info.dat");
    }
    // face coordinates (3_6/ModBlock.f90:320-322) and their sines and cosines
    const int nci = g.ni + 1, ncj = g.nj + 1, nck = g.nk + 1;
    const int ts = allcells_table_stride(d);
    std::vector<double> tab((size_t)g.nblocks * ts);
    for (int b = 0; b < g.nblocks; ++b) {
        const double* r = &g.ranges[(size_t)b * 6];
        double* t = &tab[(size_t)b * ts];
        for (int i = 1; i <= nci; ++i) t[i - 1] = (r[0] * (g.ni + 1 - i) + r[1] * (i - 1)) / g.ni;
        for (int j = 1; j <= ncj; ++j) {
            const double th = (r[2] * (g.nj + 1 - j) + r[3] * (j - 1)) / g.nj;
            t[nci + j - 1] = std::sin(th);
            t[nci + ncj + j - 1] = std::cos(th);
        }
        for (int k = 1; k <= nck; ++k) {
            const double ph = (r[4] * (g.nk + 1 - k) + r[5] * (k - 1)) / g.nk;
            t[nci + 2 * ncj + k - 1] = std::sin(ph);
            t[nci + 2 * ncj + nck + k - 1] = std::cos(ph);
        }
        t[nci + 2 * ncj + 2 * nck] = (g.flags[b] & 1) ? 1.0 : 0.0;
    }
    const size_t ncor = (size_t)nci * ncj * nck;
    const int batch = (int)std::max<size_t>(1, std::min<size_t>(g.nblocks, (64u << 20) / (ncor * 12 * 8)));
    double *dtab = nullptr, *dout = nullptr;
    auto release = [&] {
        if (dtab) cudaFree(dtab);
        if (dout) cudaFree(dout);
    };
    cudaError_t e = cudaMalloc((void**)&dtab, tab.size() * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void**)&dout, (size_t)batch * ncor * 12 * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpyAsync(dtab, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->st);
    if (e != cudaSuccess) {
        release();
        return ctx->cuda_fail(e, "allcells buffers");
    }
    std::vector<double> host((size_t)batch * ncor * 12);
    const size_t line = 12 * 16 + 1;
    int bad = -1;
    for (int b0 = 0; b0 < g.nblocks && bad < 0; b0 += batch) {
        const int nbb = std::min(batch, g.nblocks - b0);
        e = launch_allcells(d, ctx->U, ctx->Ulo, ctx->P, ctx->mixed(), dtab, b0, nbb, dout, ctx->st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(host.data(), dout, (size_t)nbb * ncor * 12 * sizeof(double), cudaMemcpyDeviceToHost,
                                ctx->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
        if (e != cudaSuccess) {
            release();
            return ctx->cuda_fail(e, "allcells");
        }
#pragma omp parallel for schedule(dynamic)
        for (int bb = 0; bb < nbb; ++bb) {
            std::string text(ncor * line, ' ');
            const double* v = &host[(size_t)bb * ncor * 12];
            for (size_t c = 0; c < ncor; ++c) {
                char* o = &text[c * line];
                for (int q = 0; q < 12; ++q) es16_8(v[c * 12 + q], o + 16 * q);
                o[line - 1] = '\n';
            }
            const std::string fn = dir + "/Block_" + i8_zero(b0 + bb + 1) + ".dat";
            FILE* f = std::fopen(fn.c_str(), "w");
            bool ok = f && std::fwrite(text.data(), 1, text.size(), f) == text.size();
            if (f) ok = (std::fclose(f) == 0) && ok;
            if (!ok) {
#pragma omp critical
                bad = b0 + bb;
            }
        }
    }
    release();
    if (bad >= 0) return ctx->fail(FALCON_ERR_INVALID_ARG, "cannot write the file of block " + std::to_string(bad + 1));
    return FALCON_OK;
}

int falcon_save_restart(falcon_ctx* ctx, const char* path) {
    int rc = need_device(ctx);
    if (rc) return rc;
    if (!path) return ctx->fail(FALCON_ERR_INVALID_ARG, "null path");
    CK(fresh_state(ctx), "ghost fill");
    CK(cudaStreamSynchronize(ctx->st), "restart");
    const RestartHeader h = restart_header(ctx);
    FILE* f = std::fopen(path, "wb");
    if (!f) return ctx->fail(FALCON_ERR_INVALID_ARG, std::string("cannot write ") + path);
    bool ok = std::fwrite(&h, sizeof h, 1, f) == 1;
    std::vector<unsigned char> buf(kIoChunk);
    const void* src[3] = {ctx->U, ctx->Ulo, ctx->P};
    const uint64_t len[3] = {h.bytes_state, h.bytes_lo, h.bytes_psi};
    cudaError_t e = cudaSuccess;
    for (int a = 0; a < 3 && ok; ++a)
        for (uint64_t off = 0; off < len[a] && ok; off += kIoChunk) {
            const size_t n = (size_t)std::min<uint64_t>(kIoChunk, len[a] - off);
            e = cudaMemcpy(buf.data(), (const unsigned char*)src[a] + off, n, cudaMemcpyDeviceToHost);
            ok = e == cudaSuccess && std::fwrite(buf.data(), 1, n, f) == n;
        }
    ok = (std::fclose(f) == 0) && ok;
    if (e != cudaSuccess) return ctx->cuda_fail(e, "restart");
    if (!ok) return ctx->fail(FALCON_ERR_INVALID_ARG, std::string("cannot write ") + path);
    return FALCON_OK;
}

int falcon_load_restart(falcon_ctx* ctx, const char* path) {
    int rc = need_device(ctx);
    if (rc) return rc;
    if (!path) return ctx->fail(FALCON_ERR_INVALID_ARG, "null path");
    FILE* f = std::fopen(path, "rb");
    if (!f) return ctx->fail(FALCON_ERR_INVALID_ARG, std::string("cannot read ") + path);
    RestartHeader h{};
    const RestartHeader want = restart_header(ctx);
    std::string why;
    if (std::fread(&h, sizeof h, 1, f) != 1 || std::memcmp(h.magic, kRestartMagic, 8) != 0 || h.version != 2)
        why = "not a restart file of this library";
    else if (h.precision != want.precision)
        why = "precision differs";
    else if (h.ni != want.ni || h.nj != want.nj || h.nk != want.nk || h.ng != want.ng || h.nblocks != want.nblocks ||
             h.grid_hash != want.grid_hash)
        why = "grid differs";
    else if (h.divb_option != want.divb_option)
        why = "divb_option differs";
    else if (h.bytes_state != want.bytes_state || h.bytes_lo != want.bytes_lo || h.bytes_psi != want.bytes_psi)
        why = "payload sizes differ";
    if (why.empty()) {   // the whole payload must be there before the state is touched
        const long here = std::ftell(f);
        std::fseek(f, 0, SEEK_END);
        const long end = std::ftell(f);
        std::fseek(f, here, SEEK_SET);
        if ((uint64_t)(end - here) != h.bytes_state + h.bytes_lo + h.bytes_psi) why = "file is truncated or too long";
    }
    if (!why.empty()) {
        std::fclose(f);
        return ctx->fail(FALCON_ERR_INVALID_ARG, std::string("restart ") + path + ": " + why);
    }
    CK(cudaStreamSynchronize(ctx->st), "restart");
    std::vector<unsigned char> buf(kIoChunk);
    void* dst[3] = {ctx->U, ctx->Ulo, ctx->P};
    const uint64_t len[3] = {h.bytes_state, h.bytes_lo, h.bytes_psi};
    cudaError_t e = cudaSuccess;
    bool ok = true;
    for (int a = 0; a < 3 && ok; ++a)
        for (uint64_t off = 0; off < len[a] && ok; off += kIoChunk) {
            const size_t n = (size_t)std::min<uint64_t>(kIoChunk, len[a] - off);
            ok = std::fread(buf.data(), 1, n, f) == n;
            if (ok) e = cudaMemcpy((unsigned char*)dst[a] + off, buf.data(), n, cudaMemcpyHostToDevice);
            ok = ok && e == cudaSuccess;
        }
    std::fclose(f);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "restart");
    if (!ok) return ctx->fail(FALCON_ERR_INVALID_ARG, std::string("restart ") + path + ": short read");
    // the stage arrays start equal to the state, as after falcon_upload_state
    CK(mirror_state(ctx, true), "restart");
    ctx->stale_edges = false;
    CK(drop_pending_cfl(ctx), "restart");
    CK(clear_step_flags(ctx), "restart");
    if (ctx->P)
        for (void* q : {ctx->Prk, ctx->P2})
            CK(cudaMemcpyAsync(q, ctx->P, h.bytes_psi, cudaMemcpyDeviceToDevice, ctx->st), "restart");
    CK(cudaStreamSynchronize(ctx->st), "restart");
    ctx->steps_done = h.steps_done;
    return FALCON_OK;
}

int falcon_shard_ranges(const falcon_ctx* ctx, int32_t nranks, int32_t* first) {
    if (!ctx || !first || nranks < 1 || nranks > ctx->grid.nblocks) return FALCON_ERR_INVALID_ARG;
    const std::vector<int> f = shard_ranges(ctx->grid.nblocks, nranks);
    for (int r = 0; r <= nranks; ++r) first[r] = f[r];
    return FALCON_OK;
}

int falcon_shard_plan(const falcon_ctx* ctx, int32_t nranks, int32_t rank, int32_t peer, int32_t dir, int64_t* entries,
                      int64_t cap, int64_t* n) {
    if (!ctx || !n || nranks < 1 || nranks > ctx->grid.nblocks || rank < 0 || rank >= nranks || peer < 0 ||
        peer >= nranks || (dir != FALCON_SHARD_SEND && dir != FALCON_SHARD_RECV))
        return FALCON_ERR_INVALID_ARG;
    const std::vector<int> f = shard_ranges(ctx->grid.nblocks, nranks);
    const std::vector<int64_t> v = dir == FALCON_SHARD_SEND ? shard_entries(ctx->grid, f, rank, peer)
                                                            : shard_entries(ctx->grid, f, peer, rank);
    *n = (int64_t)v.size();
    if (!entries) return FALCON_OK;
    if (cap < *n) return FALCON_ERR_BOUNDS;
    std::memcpy(entries, v.data(), v.size() * sizeof(int64_t));
    return FALCON_OK;
}

int falcon_set_shard(falcon_ctx* ctx, int32_t nranks, int32_t rank) {
    int rc = need_device(ctx);
    if (rc) return rc;
    if (ctx->shard.on) return ctx->fail(FALCON_ERR_INVALID_ARG, "falcon_set_shard: the context is already sharded");
    if (ctx->mixed() || ctx->cfg.phys.divb_option != 0)
        return ctx->fail(FALCON_ERR_INVALID_ARG, "falcon_set_shard: FP64 precision and divb_option 0 only");
    if (nranks < 1 || nranks > ctx->grid.nblocks || rank < 0 || rank >= nranks)
        return ctx->fail(FALCON_ERR_INVALID_ARG, "falcon_set_shard: bad rank count or rank");
    rc = autotune(ctx);
    if (rc) return rc;
    auto& S = ctx->shard;
    const std::vector<int> f = shard_ranges(ctx->grid.nblocks, nranks);
    S.nranks = nranks;
    S.rank = rank;
    S.first = f[rank];
    S.last = f[rank + 1];
    // entries within the rank: copies and interpolated/rotated entries as one list
    GhostInterpList loc{};
    CK(upload_interp_list(ctx, shard_entries(ctx->grid, f, rank, rank), loc, nullptr), "shard lists");
    S.local = GhostLists{GhostCopyList{0, nullptr, nullptr}, GhostLinList{0, nullptr, nullptr, nullptr, nullptr}, loc};
    S.send.assign(nranks, GhostInterpList{});
    S.recv_dst.assign(nranks, nullptr);
    S.nrecv.assign(nranks, 0);
    size_t most = 0;
    for (int p = 0; p < nranks; ++p) {
        if (p == rank) continue;
        CK(upload_interp_list(ctx, shard_entries(ctx->grid, f, rank, p), S.send[p], nullptr), "shard lists");
        GhostInterpList in{};
        CK(upload_interp_list(ctx, shard_entries(ctx->grid, f, p, rank), in, &S.recv_dst[p]), "shard lists");
        S.nrecv[p] = in.n;
        most = std::max(most, (size_t)std::max(S.send[p].n, in.n));
    }
    S.pack_elems = most * NV;
    CK(ctx->alloc(&S.pack, std::max<size_t>(S.pack_elems, 1) * sizeof(double)), "shard pack");
    S.last_out = ctx->U;
    S.on = true;
    CK(cudaStreamSynchronize(ctx->st), "shard");
    return FALCON_OK;
}

int falcon_shard_counts(const falcon_ctx* ctx, int32_t peer, int64_t* nsend, int64_t* nrecv) {
    if (!ctx || !ctx->shard.on || peer < 0 || peer >= ctx->shard.nranks || !nsend || !nrecv) return FALCON_ERR_INVALID_ARG;
    *nsend = peer == ctx->shard.rank ? 0 : ctx->shard.send[peer].n;
    *nrecv = peer == ctx->shard.rank ? 0 : ctx->shard.nrecv[peer];
    return FALCON_OK;
}

namespace {
bool is_device_ptr(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}
}  // namespace

int falcon_shard_pack(falcon_ctx* ctx, int32_t peer, double* buf) {
    int rc = need_device(ctx);
    if (rc) return rc;
    auto& S = ctx->shard;
    if (!S.on || peer < 0 || peer >= S.nranks || peer == S.rank || !buf)
        return ctx->fail(FALCON_ERR_INVALID_ARG, "falcon_shard_pack: not sharded, or bad peer or buffer");
    const GhostInterpList& L = S.send[peer];
    const bool dev = is_device_ptr(buf);
    double* out = dev ? buf : S.pack;
    CK(launch_shard_pack_fp64(ctx->dims, L, (const double*)S.last_out, out, ctx->st), "shard pack");
    if (!dev && L.n) CK(cudaMemcpyAsync(buf, S.pack, (size_t)L.n * NV * sizeof(double), cudaMemcpyDeviceToHost, ctx->st), "shard pack");
    CK(cudaStreamSynchronize(ctx->st), "shard pack");
    return FALCON_OK;
}

int falcon_shard_unpack(falcon_ctx* ctx, int32_t peer, const double* buf) {
    int rc = need_device(ctx);
    if (rc) return rc;
    auto& S = ctx->shard;
    if (!S.on || peer < 0 || peer >= S.nranks || peer == S.rank || !buf)
        return ctx->fail(FALCON_ERR_INVALID_ARG, "falcon_shard_unpack: not sharded, or bad peer or buffer");
    const int64_t n = S.nrecv[peer];
    const bool dev = is_device_ptr(buf);
    const double* in = buf;
    if (!dev && n) {
        CK(cudaMemcpyAsync(S.pack, buf, (size_t)n * NV * sizeof(double), cudaMemcpyHostToDevice, ctx->st), "shard unpack");
        in = S.pack;
    }
    CK(launch_shard_unpack_fp64(ctx->dims, S.recv_dst[peer], n, in, (double*)S.last_out, ctx->st), "shard unpack");
    CK(cudaStreamSynchronize(ctx->st), "shard unpack");
    return FALCON_OK;
}

int falcon_shard_min_ratio(falcon_ctx* ctx, double* local_min) {
    int rc = need_device(ctx);
    if (rc) return rc;
    if (!ctx->shard.on || !local_min) return ctx->fail(FALCON_ERR_INVALID_ARG, "falcon_shard_min_ratio: not sharded");
    unsigned long long bits = 0;
    CK(cudaMemcpyAsync(&bits, &ctx->sc->min_ratio_bits, sizeof bits, cudaMemcpyDeviceToHost, ctx->st), "min ratio");
    CK(cudaStreamSynchronize(ctx->st), "min ratio");
    std::memcpy(local_min, &bits, sizeof bits);
    return check_nan(ctx);
}

int falcon_shard_set_min_ratio(falcon_ctx* ctx, double global_min) {
    int rc = need_device(ctx);
    if (rc) return rc;
    if (!ctx->shard.on || !(global_min > 0.0)) return ctx->fail(FALCON_ERR_INVALID_ARG, "falcon_shard_set_min_ratio");
    unsigned long long bits;
    std::memcpy(&bits, &global_min, sizeof bits);
    CK(cudaMemcpyAsync(&ctx->sc->min_ratio_bits, &bits, sizeof bits, cudaMemcpyHostToDevice, ctx->st), "min ratio");
    CK(launch_finalize_dt(ctx->sc, ctx->st), "min ratio");
    CK(cudaStreamSynchronize(ctx->st), "min ratio");
    return FALCON_OK;
}

int falcon_set_wait_limit(falcon_ctx* ctx, int32_t polls) {
    int rc = need_device(ctx);
    if (rc) return rc;
    const int32_t v = polls < 0 ? kDefaultWaitPolls : polls;
    CK(cudaMemcpyAsync(&ctx->sc->wait_polls, &v, sizeof v, cudaMemcpyHostToDevice, ctx->st), "wait limit");
    CK(cudaStreamSynchronize(ctx->st), "wait limit");
    return FALCON_OK;
}

int falcon_synchronize(falcon_ctx* ctx) {
    int rc = need_device(ctx);
    if (rc) return rc;
    CK(cudaStreamSynchronize(ctx->st), "synchronize");
    collect(ctx);
    return check_nan(ctx);
}

int falcon_set_kernel_timing(falcon_ctx* ctx, int32_t on) {
    int rc = need_device(ctx);
    if (rc) return rc;
    ctx->ktiming = on != 0;
    return FALCON_OK;
}

int falcon_kernel_stats(falcon_ctx* ctx, char* names, size_t names_len, double* ms, int64_t* launches, int32_t cap,
                        int32_t* n) {
    if (!ctx || !n) return FALCON_ERR_INVALID_ARG;
    if (ctx->on_device) { cudaStreamSynchronize(ctx->st); collect(ctx); }
    *n = KN_COUNT;
    std::string all;
    for (int k = 0; k < KN_COUNT; ++k) {
        all += kKernelNames[k];
        all += "\n";
        if (k < cap) {
            if (ms) ms[k] = ctx->kms[k];
            if (launches) launches[k] = ctx->kcount[k];
        }
    }
    if (names && names_len) snprintf(names, names_len, "%s", all.c_str());
    return FALCON_OK;
}

int falcon_reset_kernel_stats(falcon_ctx* ctx) {
    if (!ctx) return FALCON_ERR_INVALID_ARG;
    if (ctx->on_device) { cudaStreamSynchronize(ctx->st); collect(ctx); }
    for (int k = 0; k < KN_COUNT; ++k) { ctx->kms[k] = 0; ctx->kcount[k] = 0; }
    return FALCON_OK;
}

int falcon_timer_start(falcon_ctx* ctx) {
    int rc = need_device(ctx);
    if (rc) return rc;
    CK(cudaEventRecord(ctx->t0, ctx->st), "timer");
    return FALCON_OK;
}

int falcon_timer_stop(falcon_ctx* ctx, double* ms) {
    int rc = need_device(ctx);
    if (rc) return rc;
    CK(cudaEventRecord(ctx->t1, ctx->st), "timer");
    CK(cudaEventSynchronize(ctx->t1), "timer");
    float f = 0.f;
    CK(cudaEventElapsedTime(&f, ctx->t0, ctx->t1), "timer");
    if (ms) *ms = f;
    collect(ctx);
    return FALCON_OK;
}

int falcon_tuning(falcon_ctx* ctx, int32_t* kpar_stage, int32_t* kpar_diffusion) {
    int rc = need_device(ctx);
    if (rc) return rc;
    rc = autotune(ctx);
    if (rc) return rc;
    if (kpar_stage) *kpar_stage = ctx->kpar_stage;
    if (kpar_diffusion) *kpar_diffusion = ctx->kpar_diff;
    return FALCON_OK;
}

int falcon_set_tuning(falcon_ctx* ctx, int32_t kpar_stage, int32_t kpar_diffusion) {
    int rc = need_device(ctx);
    if (rc) return rc;
    int cand[8];
    const int n = ctx->mixed() ? kpar_candidates_mixed(ctx->dims, cand) : kpar_candidates_fp64(ctx->dims, cand);
    bool ok_s = false, ok_d = false;
    for (int q = 0; q < n; ++q) {
        ok_s |= cand[q] == kpar_stage;
        ok_d |= cand[q] == kpar_diffusion;
    }
    if (!ok_s || !ok_d)
        return ctx->fail(FALCON_ERR_INVALID_ARG, "falcon_set_tuning: no compiled variant with k-chunk depths " +
                                                     std::to_string(kpar_stage) + ", " + std::to_string(kpar_diffusion));
    CK(cudaStreamSynchronize(ctx->st), "set tuning");
    for (auto& row : ctx->graphs)   // captured with the previous depths
        for (cudaGraphExec_t& gx : row)
            if (gx) {
                cudaGraphExecDestroy(gx);
                gx = nullptr;
            }
    ctx->kpar_stage = kpar_stage;
    ctx->kpar_diff = kpar_diffusion;
    return FALCON_OK;
}

int falcon_set_step_mode(falcon_ctx* ctx, int32_t mode) {
    int rc = need_device(ctx);
    if (rc) return rc;
    if (mode != FALCON_STEP_GRAPH && mode != FALCON_STEP_PERSISTENT)
        return ctx->fail(FALCON_ERR_INVALID_ARG, "falcon_set_step_mode: unknown mode");
    if (mode == FALCON_STEP_PERSISTENT) {
        if (!ctx->mixed() || !ctx->R2 || ctx->P || ctx->cfg.phys.divb_option != 0 || ctx->dims.ni != 16 ||
            ctx->dims.nj != 16 || ctx->dims.nk != 16)
            return ctx->fail(FALCON_ERR_INVALID_ARG,
                             "falcon_set_step_mode: the persistent step covers the mixed path with 16^3 blocks and "
                             "divb_option 0");
        if (!ctx->gbar) CK(ctx->alloc(&ctx->gbar, 8 * sizeof(unsigned int)), "alloc grid barrier");
        CK(cudaMemsetAsync(ctx->gbar, 0, 8 * sizeof(unsigned int), ctx->st), "grid barrier");
    }
    ctx->step_mode = mode;
    return FALCON_OK;
}

int falcon_exchange_stats(const falcon_ctx* ctx, int64_t* out) {
    if (!ctx || !out) return FALCON_ERR_INVALID_ARG;
    for (int q = 0; q < 3; ++q) out[q] = ctx->stage_counts[q];
    out[3] = ctx->pushed_faces;
    out[4] = ctx->pushed_cells;
    return FALCON_OK;
}

int falcon_ghost_list_sizes(const falcon_ctx* ctx, int64_t* counts) {
    if (!ctx || !counts) return FALCON_ERR_INVALID_ARG;
    for (int q = 0; q < 3; ++q) counts[q] = ctx->ghost_counts[q];
    return FALCON_OK;
}

int falcon_device_bytes(const falcon_ctx* ctx, int64_t* bytes) {
    if (!ctx || !bytes) return FALCON_ERR_INVALID_ARG;
    *bytes = ctx->dev_bytes;
    return FALCON_OK;
}

}  // extern "C"
