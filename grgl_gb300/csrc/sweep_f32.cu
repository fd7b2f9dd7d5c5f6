// Sweep kernel instances for the AddF32 accumulation operator.
#include "sweep_inst.cuh"

namespace grgx {
void launch_sweep_f32(const SweepParams<float>& p, int vw, int g, int variant, dim3 grid, int sms,
                      cudaStream_t s) {
    GRGX_SWEEP_DISPATCH4(AddF32)
    GRGX_SWEEP_DEEP4(AddF32)
    GRGX_SWEEP_UNSUPPORTED
}
void launch_sweep_staged_f32(const SweepParams<float>& p, dim3 grid, cudaStream_t s) GRGX_SWEEP_STAGED(AddF32)
}  // namespace grgx
