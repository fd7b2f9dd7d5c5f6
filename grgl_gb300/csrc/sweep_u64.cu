// Sweep kernel instances for the AddU64 accumulation operator.
#include "sweep_inst.cuh"

namespace grgx {
void launch_sweep_u64(const SweepParams<unsigned long long>& p, int vw, int g, int variant, dim3 grid, int sms,
                      cudaStream_t s) {
    GRGX_SWEEP_DISPATCH8(AddU64)
    GRGX_SWEEP_UNSUPPORTED
}
}  // namespace grgx
