"""grgx_matmul_noalloc: the entry point for callers that cannot allocate device memory while
they run (a host that hands out a fixed device budget at start-up and forbids allocation
afterwards).  Called through the C ABI with device buffers the test owns, it must give what
grgx_matmul gives -- bit-exact for integers, within the float tolerances of the other GPU tests
-- on two calls in a row that share its static scratch; one call per dtype is also checked
against the oracle, and a call after the first must leave the device's free memory and the
library's memory pool exactly as they were.  Collected last on purpose, so a failure here comes
after every other test has run."""
import numpy as np
import pytest

from tests.conftest import assert_matches, assert_matches_oracle, oracle_graph_of

pytestmark = pytest.mark.gpu
DOWN, UP = 1, 2
DTYPE_CODES = {np.dtype(np.float64): 0, np.dtype(np.float32): 1, np.dtype(np.int64): 2, np.dtype(np.int32): 3}


@pytest.fixture(scope="module")
def env(cuda_ok):
    import torch

    import grgl_gb300 as gx
    from grgl_gb300 import _lib

    g = gx.window_tree_grg(2000, 20000, seed=21).upload()
    return torch, gx, _lib, g


def _noalloc_dev(torch, _lib, g, x, direction, out):
    """One call on device tensors the caller allocated beforehand."""
    st = _lib.lib().grgx_matmul_noalloc(g._h, DTYPE_CODES[np.dtype(str(x.dtype).split(".")[-1])], x.data_ptr(),
                                       x.shape[1], x.shape[0], direction, out.data_ptr(), out.numel(),
                                       torch.cuda.current_stream().cuda_stream)
    _lib.check(st)


def _noalloc(torch, _lib, g, V, direction, out_cols):
    x = torch.from_numpy(V).cuda()
    out = torch.empty((V.shape[0], out_cols), dtype=x.dtype, device="cuda")
    _noalloc_dev(torch, _lib, g, x, direction, out)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("dtype", [np.int32, np.int64, np.float32, np.float64])
def test_noalloc_matches_matmul_twice(env, dtype):
    torch, gx, _lib, g = env
    og = oracle_graph_of(g)
    rng = np.random.default_rng(5)
    for direction, cols, out_cols in ((UP, g.num_samples, g.num_mutations), (DOWN, g.num_mutations, g.num_samples)):
        for call in range(2):  # two calls in a row share (and reuse) the static scratch
            K = 8 + 5 * call
            if np.dtype(dtype).kind == "f":
                V = rng.standard_normal((K, cols)).astype(dtype)
            else:
                V = rng.integers(-500, 500, size=(K, cols)).astype(dtype)
            got = _noalloc(torch, _lib, g, V, direction, out_cols)
            ref = gx.matmul(g, V, direction)
            scale = np.abs(gx.matmul(g, np.abs(V).astype(np.float64), direction)) if np.dtype(dtype).kind == "f" else None
            rtol = 1e-6 if np.dtype(dtype) == np.float32 else None
            assert_matches(got, ref, None if scale is None else scale.astype(ref.dtype), rtol=rtol)
            if call == 1:
                assert_matches_oracle(og, V, direction, got)


def test_noalloc_second_call_allocates_nothing(env):
    """After a first call, a call changes neither the device's free memory (cudaMemGetInfo) nor
    what the library's pool holds or hands out."""
    torch, gx, _lib, g = env
    rng = np.random.default_rng(9)
    for direction, cols, out_cols in ((DOWN, g.num_mutations, g.num_samples), (UP, g.num_samples, g.num_mutations)):
        x = torch.from_numpy(rng.standard_normal((16, cols))).cuda()
        out = torch.empty((16, out_cols), dtype=x.dtype, device="cuda")
        _noalloc_dev(torch, _lib, g, x, direction, out)  # the first call on this device may look up the scratch
        torch.cuda.synchronize()
        dev = torch.cuda.current_device()
        free0, pool0 = torch.cuda.mem_get_info(dev)[0], gx.pool_usage(dev)
        _noalloc_dev(torch, _lib, g, x, direction, out)
        torch.cuda.synchronize()
        free1, pool1 = torch.cuda.mem_get_info(dev)[0], gx.pool_usage(dev)
        assert free1 == free0, (free0, free1)
        assert pool1 == pool0, (pool0, pool1)


def test_noalloc_rejects_oversized_products(env):
    torch, gx, _lib, g = env
    K = 2000  # 2000 x nodes x 8 bytes of node values is far beyond the 64 MiB static scratch
    V = np.zeros((K, g.num_samples), dtype=np.float64)
    with pytest.raises(RuntimeError, match="static scratch"):
        _noalloc(torch, _lib, g, V, UP, g.num_mutations)


def test_noalloc_needs_resident_graph(env):
    torch, gx, _lib, _ = env
    g2 = gx.window_tree_grg(100, 300, seed=1)  # never uploaded
    V = np.ones((1, 100), dtype=np.int32)
    with pytest.raises(RuntimeError, match="grgx_graph_upload"):
        _noalloc(torch, _lib, g2, V, UP, g2.num_mutations)
