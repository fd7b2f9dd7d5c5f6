// Instantiation helper: a dispatcher from runtime (VW, G) to the sweep_kernel template.
#pragma once
#include <stdexcept>

#include "launch.h"

// Persistent grid: at most as many blocks as can be resident at once.
#define GRGX_SWEEP_CASE(OP, VWV, GV)                                                  \
    if (vw == VWV && g == GV) {                                                       \
        static int perSm = 0;                                                         \
        if (perSm == 0) {                                                             \
            int nb = 0;                                                               \
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, sweep_kernel<OP, VWV, GV>, 256, 0); \
            perSm = nb > 0 ? nb : 1;                                                  \
        }                                                                             \
        const unsigned cap = (unsigned)(perSm * sms);                                 \
        if (grid.x > cap) grid.x = cap;                                               \
        sweep_kernel<OP, VWV, GV><<<grid, 256, 0, s>>>(p);                            \
        return;                                                                       \
    }

// 4-byte storage: (1,1), (2,1), (4, 1..32)
#define GRGX_SWEEP_DISPATCH4(OP)                                                      \
    GRGX_SWEEP_CASE(OP, 1, 1)                                                         \
    GRGX_SWEEP_CASE(OP, 2, 1)                                                         \
    GRGX_SWEEP_CASE(OP, 4, 1)                                                         \
    GRGX_SWEEP_CASE(OP, 4, 2)                                                         \
    GRGX_SWEEP_CASE(OP, 4, 4)                                                         \
    GRGX_SWEEP_CASE(OP, 4, 8)                                                         \
    GRGX_SWEEP_CASE(OP, 4, 16)                                                        \
    GRGX_SWEEP_CASE(OP, 4, 32)                                                        \
    throw std::runtime_error("unsupported sweep shape");

// 8-byte storage: (1,1), (2, 1..32)
#define GRGX_SWEEP_DISPATCH8(OP)                                                      \
    GRGX_SWEEP_CASE(OP, 1, 1)                                                         \
    GRGX_SWEEP_CASE(OP, 2, 1)                                                         \
    GRGX_SWEEP_CASE(OP, 2, 2)                                                         \
    GRGX_SWEEP_CASE(OP, 2, 4)                                                         \
    GRGX_SWEEP_CASE(OP, 2, 8)                                                         \
    GRGX_SWEEP_CASE(OP, 2, 16)                                                        \
    GRGX_SWEEP_CASE(OP, 2, 32)                                                        \
    throw std::runtime_error("unsupported sweep shape");
