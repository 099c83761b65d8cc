// mhd_mixed.cu -- mixed-precision instantiation of the step kernels: FP32
// state and stencil RHS; p1 assembled in FP64; FP64 CFL reduction and dt.
#include "launch_impl.cuh"

namespace falcon {
cudaError_t launch_stage_mixed(const StepDims& d, const Geometry& g, const float* in, const float* un, float* out,
                               int stage, int bcw, const StepScalars* sc, int heat, cudaStream_t st) {
    return impl::stage_any<float>(d, g, in, un, out, stage, bcw, sc, heat, st);
}
cudaError_t launch_diffusion_mixed(const StepDims& d, const Geometry& g, float* u, const StepScalars* sc,
                                   cudaStream_t st) {
    return impl::diff_any<float>(d, g, u, sc, st);
}
cudaError_t launch_cfl_mixed(const StepDims& d, const Geometry& g, const float* u, StepScalars* sc, cudaStream_t st) {
    return impl::cfl_any<float>(d, g, u, sc, st);
}
cudaError_t launch_ghost_mixed(const StepDims& d, const GhostCopyList& cp, const GhostInterpList& ip, float* u,
                               cudaStream_t st) {
    return impl::ghost_any<float>(d, cp, ip, u, st);
}
}  // namespace falcon
