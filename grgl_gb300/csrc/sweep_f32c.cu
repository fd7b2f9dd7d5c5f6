// Sweep kernel instances for the AddF32C accumulation operator.
#include "sweep_inst.cuh"

namespace grgx {
void launch_sweep_f32c(const SweepParams<float>& p, int vw, int g, int variant, dim3 grid, int sms,
                       cudaStream_t s) {
    GRGX_SWEEP_DISPATCH4(AddF32C)
    GRGX_SWEEP_DEEP4(AddF32C)
    GRGX_SWEEP_UNSUPPORTED
}
void launch_sweep_staged_f32c(const SweepParams<float>& p, dim3 grid, cudaStream_t s) GRGX_SWEEP_STAGED(AddF32C)
}  // namespace grgx
