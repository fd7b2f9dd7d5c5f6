// Sweep kernel instances for the AddU32 accumulation operator.
#include "sweep_inst.cuh"

namespace grgx {
void launch_sweep_u32(const SweepParams<uint32_t>& p, int vw, int g, int variant, dim3 grid, int sms,
                      cudaStream_t s) {
    GRGX_SWEEP_DISPATCH4(AddU32)
    GRGX_SWEEP_DEEP4(AddU32)
    GRGX_SWEEP_UNSUPPORTED
}
void launch_sweep_staged_u32(const SweepParams<uint32_t>& p, dim3 grid, cudaStream_t s) GRGX_SWEEP_STAGED(AddU32)
}  // namespace grgx
