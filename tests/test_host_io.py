"""Host results in pinned pooled memory: values and numpy behaviour match the device path."""
import ctypes

import numpy as np
import pytest

DOWN, UP = 1, 2


def test_host_free_ignores_foreign_pointers(lib_built):
    from grgl_gb300 import _lib

    buf = ctypes.create_string_buffer(64)
    _lib.lib().grgx_host_free(ctypes.addressof(buf))  # not from the pool: ignored
    _lib.lib().grgx_host_free(None)


@pytest.mark.gpu
def test_pinned_results_match_device_path(cuda_ok):
    import torch

    import grgl_gb300 as gx

    g = gx.window_tree_grg(4000, 30000, seed=71)
    rng = np.random.default_rng(0)
    for dt in (np.float64, np.int32):
        V = (rng.standard_normal((40, g.num_samples)) if dt == np.float64
             else rng.integers(0, 2, size=(40, g.num_samples))).astype(dt)
        outs = []
        for _ in range(3):  # later calls reuse freed blocks
            out = gx.matmul(g, V, UP)
            assert out.nbytes >= 4 << 20 and out.flags.c_contiguous and out.flags.writeable
            outs.append(out.copy())
            del out
        dev = gx.matmul(g, torch.from_numpy(V).cuda(), UP).cpu().numpy()
        for o in outs:
            assert np.array_equal(o, dev)
        out = gx.matmul(g, V, UP)
        out[...] = 0  # an ordinary writable array
        assert not out.any()
