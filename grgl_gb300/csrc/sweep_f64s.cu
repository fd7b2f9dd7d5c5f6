// Sweep kernel instances for the AddF64S (float64 as scaled float pairs) operator.
#include "sweep_inst.cuh"

namespace grgx {
void launch_sweep_f64s(const SweepParams<DF>& p, int vw, int g, dim3 grid, int sms, cudaStream_t s) {
    GRGX_SWEEP_DISPATCH8(AddF64S)
}
}  // namespace grgx
