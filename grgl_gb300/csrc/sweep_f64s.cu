// Sweep kernel instances for the AddF64S (float64 as scaled float pairs) operator.
#include "sweep_inst.cuh"

namespace grgx {
void launch_sweep_f64s(const SweepParams<DF>& p, int vw, int g, int variant, dim3 grid, int sms,
                       cudaStream_t s) {
    GRGX_SWEEP_DISPATCH8(AddF64S)
    GRGX_SWEEP_DEEP8(AddF64S)
    GRGX_SWEEP_UNSUPPORTED
}
}  // namespace grgx
