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


@pytest.mark.gpu
@pytest.mark.parametrize("replay", [False, True])
def test_matmul_async_matches_matmul(cuda_ok, replay):
    """Host-buffer products queued on two streams (GRGX_FLAG_ASYNC) give the arrays the
    synchronous call gives, through the direct path and through graph replay, and keep the
    buffers they were given alive until result()."""
    import gc

    import torch

    import grgl_gb300 as gx
    from tests.conftest import GOLDEN

    gx.set_graph_replay(replay)
    try:
        g = gx.window_tree_grg(3000, 20000, seed=13)
        rng = np.random.default_rng(5)
        streams = [torch.cuda.Stream(), torch.cuda.Stream()]
        calls = []
        for dt, K in ((np.float64, 3), (np.float32, 40), (np.int32, 64), (np.int64, 8), (np.uint8, 5)):
            for d in (UP, DOWN):
                cols = g.num_samples if d == UP else g.num_mutations
                V = (rng.standard_normal((K, cols)) if np.dtype(dt).kind == "f"
                     else rng.integers(0, 100, size=(K, cols))).astype(dt)
                calls.append((V, d))
        pend = []
        for i, (V, d) in enumerate(calls):
            P = gx.host_empty(V.shape, V.dtype)
            P[...] = V
            # the pending call holds the only reference to its pinned input
            pend.append(gx.matmul_async(g, P, d, stream=streams[i % 2]))
            del P
        gc.collect()
        for (V, d), p in zip(calls, pend):
            got = p.result()
            assert p.done()
            assert np.array_equal(got, gx.matmul(g, V, d))
        # UP writes `miss` in place; the async form does so by result()
        gm = gx.load_immutable_grg(str(GOLDEN / "t200miss.grg"))
        V = rng.standard_normal((4, gm.num_samples))
        m_sync = rng.standard_normal((4, gm.num_mutations))
        m_async = m_sync.copy()
        ref = gx.matmul(gm, V, UP, miss=m_sync)
        got = gx.matmul_async(gm, V, UP, miss=m_async, stream=streams[0]).result()
        assert np.array_equal(got, ref) and np.array_equal(m_async, m_sync)
        # misuse is reported at the call, before anything is queued
        with pytest.raises(RuntimeError, match="non-zero dimensions"):
            gx.matmul_async(g, np.zeros((0, g.num_samples)), UP)
    finally:
        gx.set_graph_replay(True)
