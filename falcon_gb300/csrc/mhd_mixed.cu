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

}  // namespace falcon
