"""grgl_gb300 -- GB300-native GRG matrix multiplication (drop-in for pygrgl.matmul).

    import grgl_gb300 as pygrgl
    grg = pygrgl.load_immutable_grg("data.grg")
    counts = pygrgl.matmul(grg, numpy.ones((1, grg.num_samples), dtype=numpy.int32), pygrgl.TraversalDirection.UP)

The compute runs in libgrgx.so (hand-written sm_103a CUDA kernels behind a C ABI,
include/grgx.h); there is no CPU implementation in this package.
"""
from .api import (COAL_COUNT_NOT_SET, DOWN, GRG, INVALID_NODE, UP, Server, TraversalDirection, autotune,
                  autotune_clear, autotune_load, autotune_table, collect_timings, dot_product, from_csr, from_pygrgl, last_timing,
                  PendingMatmul, host_empty, load_immutable_grg, matmul, matmul_async, matmul_batch, matmul_gram,
                  matmul_standardized, measure_l2_bandwidth, pool_usage, set_graph_replay, set_timing,
                  window_tree_grg)

__all__ = [
    "COAL_COUNT_NOT_SET", "DOWN", "GRG", "INVALID_NODE", "UP", "TraversalDirection", "dot_product", "from_csr",
    "from_pygrgl", "last_timing", "load_immutable_grg", "matmul", "matmul_batch", "set_timing", "window_tree_grg",
    "Server", "matmul_standardized", "measure_l2_bandwidth", "set_graph_replay", "autotune", "autotune_table",
    "autotune_load", "autotune_clear", "matmul_gram", "collect_timings", "matmul_async", "PendingMatmul", "host_empty",
    "pool_usage",
]
