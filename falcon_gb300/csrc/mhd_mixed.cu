// mhd_mixed.cu -- mixed-precision instantiation of the step kernels: FP32
// state (u^n compensated by an 8-bit correction) and stencil RHS; p1 assembled
// in FP64; FP64 CFL reduction and dt.
#include "launch_impl.cuh"

namespace falcon {
cudaError_t launch_stage_mixed(const StepDims& d, const Geometry& g, const float* in, const float* un, float* out,
                               int8_t* lo, const PushTable& push, const DivBArgs& psi, int stage, int bcw, StepScalars* sc,
                               int heat, int kpar, cudaStream_t st) {
    return impl::stage_any<float>(d, g, in, un, out, lo, push, psi, stage, bcw, sc, heat, kpar, st);
}
cudaError_t launch_psi_diffusion_mixed(const StepDims& d, const Geometry& g, const float* u, const float* psi,
                                       float* psi_out, StepScalars* sc, cudaStream_t st) {
    return impl::psi_diffusion_any<float>(d, g, u, psi, psi_out, sc, st);
}
cudaError_t launch_psi_ghost_mixed(const StepDims& d, const GhostLists& gl, float* psi, cudaStream_t st) {
    return impl::psi_ghost_any<float>(d, gl, psi, st);
}
cudaError_t launch_diffusion_mixed(const StepDims& d, const Geometry& g, const float* u, float* out, int8_t* lo,
                                   const PushTable& push, StepScalars* sc, int kpar, cudaStream_t st, int cfl_next) {
    return impl::diff_any<float>(d, g, u, out, lo, push, sc, kpar, st, cfl_next);
}
cudaError_t launch_cfl_mixed(const StepDims& d, const Geometry& g, const float* u, StepScalars* sc, cudaStream_t st) {
    return impl::cfl_any<float>(d, g, u, sc, st);
}
cudaError_t launch_ghost_mixed(const StepDims& d, const GhostLists& gl, float* u, cudaStream_t st) {
    return impl::ghost_any<float>(d, gl, u, st);
}
int kpar_candidates_mixed(const StepDims& d, int* out) { return impl::candidates<float>(d, out); }
cudaError_t launch_clear_outside_core_mixed(const StepDims& d, float* u, int nvar, cudaStream_t st) {
    const int64_t nbv = (int64_t)d.nblocks * nvar;
    impl::k_clear_outside_core<float><<<(unsigned)(nbv < 65535 * 4 ? nbv : 65535 * 4), 256, 0, st>>>(u, nbv, d);
    return cudaGetLastError();
}
cudaError_t launch_push_state_mixed(const StepDims& d, const Geometry& g, float* u, const PushTable& push,
                                    StepScalars* sc, cudaStream_t st) {
    if (d.ni == 16 && d.nj == 16 && d.nk == 16) impl::k_push_state<16, 16, 16><<<d.nblocks, 256, 0, st>>>(u, push, g, sc);
    else if (d.ni == 8 && d.nj == 8 && d.nk == 8) impl::k_push_state<8, 8, 8><<<d.nblocks, 64, 0, st>>>(u, push, g, sc);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}


cudaError_t launch_step_persistent_mixed(const StepDims& d, const Geometry& g, float* U, float* RK, float* R2,
                                         int8_t* lo, const PushTable& push, const GhostLists& gl_stage,
                                         const GhostLists& gl_final, StepScalars* sc, unsigned int* bar,
                                         cudaStream_t st) {
    if (d.ni != 16 || d.nj != 16 || d.nk != 16 || !bar) return cudaErrorInvalidValue;
    using SS = impl::Shape<float, 16, 16, 16, 2>;
    using SD = impl::MShape<16, 16, 16, 2>;
    constexpr size_t smem = SS::smem_stage > SD::smem ? SS::smem_stage : SD::smem;
    // two CTAs of 512 threads per SM, as the separate stage and diffusion
    // launches run (228 KB per SM, 1 KB of it reserved per CTA, and about
    // 0.5 KB of static shared memory in the bodies)
    static_assert(2 * (smem + 512 + 1024) <= 233472, "two CTAs per SM");
    auto kern = impl::k_step_persistent<16>;
    static int grid_cap = 0, dev_cached = -1;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev != dev_cached) {
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int per_sm = 0, nsm = 0;
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 512, smem);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) return cudaErrorLaunchOutOfResources;
        grid_cap = per_sm * nsm;   // every CTA resident at once: the grid barrier needs it
        dev_cached = dev;
    }
    const unsigned grid = (unsigned)(d.nblocks < grid_cap ? d.nblocks : grid_cap);
    e = cudaMemsetAsync(bar, 0, 8 * sizeof(unsigned int), st);   // arrival counter, generation, block tickets
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(512);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, impl::StepBuffers{U, RK, R2, lo}, push, g, sc, gl_stage, gl_final, d,
                              impl::GridBarrier{bar, bar + 1, bar + 2});
}

}  // namespace falcon
