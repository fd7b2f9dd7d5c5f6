// Sweep kernel instances for the AddF64 accumulation operator.
#include "sweep_inst.cuh"

namespace grgx {
void launch_sweep_f64(const SweepParams<double>& p, int vw, int g, int variant, dim3 grid, int sms,
                      cudaStream_t s) {
    GRGX_SWEEP_DISPATCH8(AddF64)
    GRGX_SWEEP_UNSUPPORTED
}
}  // namespace grgx
