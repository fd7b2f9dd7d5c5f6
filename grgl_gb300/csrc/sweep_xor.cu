// Sweep kernel instances for the XorU32 accumulation operator.
#include "sweep_inst.cuh"

namespace grgx {
void launch_sweep_xor(const SweepParams<uint32_t>& p, int vw, int g, int variant, dim3 grid, int sms,
                      cudaStream_t s) {
    GRGX_SWEEP_DISPATCH4(XorU32)
    GRGX_SWEEP_UNSUPPORTED
}
void launch_sweep_staged_xor(const SweepParams<uint32_t>& p, dim3 grid, cudaStream_t s) GRGX_SWEEP_STAGED(XorU32)
}  // namespace grgx
