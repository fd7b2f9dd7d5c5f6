// Instantiation helper: a dispatcher from a runtime (VW, G, depth variant) to the sweep_kernel
// template.
#pragma once
#include <stdexcept>

#include "launch.h"

// Persistent grid: at most as many blocks as can be resident at once.  The 16-bit-id instance
// (split block passes) and the 32-bit one are separate kernels.
#define GRGX_SWEEP_CASE(OP, VWV, GV, DV)                                              \
    if (vw == VWV && g == GV && variant == DV - 1) {                                  \
        static int perSm = 0;                                                         \
        if (perSm == 0) {                                                             \
            int nb = 0;                                                               \
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, sweep_kernel<OP, VWV, GV, DV, false>, 256, 0); \
            perSm = nb > 0 ? nb : 1;                                                  \
        }                                                                             \
        const unsigned cap = (unsigned)(perSm * sms);                                 \
        if (grid.x > cap) grid.x = cap;                                               \
        if (p.id16)                                                                   \
            sweep_kernel<OP, VWV, GV, DV, true><<<grid, 256, 0, s>>>(p);              \
        else                                                                          \
            sweep_kernel<OP, VWV, GV, DV, false><<<grid, 256, 0, s>>>(p);             \
        return;                                                                       \
    }

// 4-byte storage: (1,1), (2,1), (4, 1..32)
#define GRGX_SWEEP_DISPATCH4(OP)                                                      \
    GRGX_SWEEP_CASE(OP, 1, 1, 1)                                                      \
    GRGX_SWEEP_CASE(OP, 2, 1, 1)                                                      \
    GRGX_SWEEP_CASE(OP, 4, 1, 1)                                                      \
    GRGX_SWEEP_CASE(OP, 4, 2, 1)                                                      \
    GRGX_SWEEP_CASE(OP, 4, 4, 1)                                                      \
    GRGX_SWEEP_CASE(OP, 4, 8, 1)                                                      \
    GRGX_SWEEP_CASE(OP, 4, 16, 1)                                                     \
    GRGX_SWEEP_CASE(OP, 4, 32, 1)

// the deep variants of the 16-byte-vector shapes
#define GRGX_SWEEP_DEEP4(OP)                                                          \
    GRGX_SWEEP_CASE(OP, 4, 1, 2)                                                      \
    GRGX_SWEEP_CASE(OP, 4, 2, 2)                                                      \
    GRGX_SWEEP_CASE(OP, 4, 4, 2)                                                      \
    GRGX_SWEEP_CASE(OP, 4, 8, 2)                                                      \
    GRGX_SWEEP_CASE(OP, 4, 16, 2)                                                     \
    GRGX_SWEEP_CASE(OP, 4, 32, 2)

// 8-byte storage: (1,1), (2, 1..32)
#define GRGX_SWEEP_DISPATCH8(OP)                                                      \
    GRGX_SWEEP_CASE(OP, 1, 1, 1)                                                      \
    GRGX_SWEEP_CASE(OP, 2, 1, 1)                                                      \
    GRGX_SWEEP_CASE(OP, 2, 2, 1)                                                      \
    GRGX_SWEEP_CASE(OP, 2, 4, 1)                                                      \
    GRGX_SWEEP_CASE(OP, 2, 8, 1)                                                      \
    GRGX_SWEEP_CASE(OP, 2, 16, 1)                                                     \
    GRGX_SWEEP_CASE(OP, 2, 32, 1)

#define GRGX_SWEEP_DEEP8(OP)                                                          \
    GRGX_SWEEP_CASE(OP, 2, 1, 2)                                                      \
    GRGX_SWEEP_CASE(OP, 2, 2, 2)                                                      \
    GRGX_SWEEP_CASE(OP, 2, 4, 2)                                                      \
    GRGX_SWEEP_CASE(OP, 2, 8, 2)                                                      \
    GRGX_SWEEP_CASE(OP, 2, 16, 2)                                                     \
    GRGX_SWEEP_CASE(OP, 2, 32, 2)

#define GRGX_SWEEP_UNSUPPORTED throw std::runtime_error("unsupported sweep shape");

// The staged kernel with the block's source values as dynamic shared memory (opted in above the
// default 48 KB on the current device on every launch: the call is cheap and per device).
#define GRGX_SWEEP_STAGED(OP)                                                                      \
    {                                                                                             \
        const int bytes = kStagedBytes<typename OP::S>;                                            \
        cudaFuncSetAttribute(sweep_kernel_staged<OP>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes); \
        sweep_kernel_staged<OP><<<grid, kStagedThreads, bytes, s>>>(p);                            \
    }
