"""Standardized-genotype products Z = (X - mu)/sigma on the GPU against a float64 dense oracle."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
DOWN, UP = 1, 2


@pytest.fixture(scope="module")
def env(cuda_ok):
    import grgl_gb300 as gx

    g = gx.window_tree_grg(600, 4000, seed=41)
    a = g.export_arrays()
    og = oracle.OracleGraph(num_samples=600, ploidy=2, down_off=a["down_off"], down_adj=a["down_adj"],
                            mut_node=a["mut_node"])
    return gx, g, og


@pytest.mark.parametrize("dtype,rtol", [(np.float64, 1e-12), (np.float32, 1e-6)])
def test_standardized_matches_dense(env, dtype, rtol):
    gx, g, og = env
    rng = np.random.default_rng(2)
    for direction, cols in ((UP, g.num_samples), (DOWN, g.num_mutations)):
        for K in (1, 7, 64):
            V = rng.standard_normal((K, cols)).astype(dtype)
            got = gx.matmul_standardized(g, V, direction)
            ref, scale = oracle.standardized(og, V, direction, return_scale=True)
            err = np.abs(got.astype(np.float64) - ref)
            assert np.all(err <= rtol * scale + 1e-300), (direction, K, float(np.max(err / np.maximum(scale, 1e-300))))


def test_standardized_device_and_masked_columns(env):
    import torch

    gx, g, og = env
    V = np.random.default_rng(3).standard_normal((4, g.num_mutations))
    host = gx.matmul_standardized(g, V, DOWN)
    dev = gx.matmul_standardized(g, torch.from_numpy(V).cuda(), DOWN)
    torch.cuda.synchronize()
    assert np.array_equal(dev.cpu().numpy(), host)
    # a graph with a mutation carried by every sample (sigma = 0): its column is masked to zero
    N = 4
    down_off = np.array([0, 0, 0, 0, 0, 4], dtype=np.uint64)
    arrs = dict(num_samples=N, ploidy=2, down_off=down_off, down_adj=np.arange(4, dtype=np.uint32),
                mut_node=np.array([4, 0], dtype=np.uint32))
    gm = gx.from_csr(**arrs)
    out = gx.matmul_standardized(gm, np.ones((1, N)), UP)
    ref = oracle.standardized(oracle.OracleGraph(**arrs), np.ones((1, N)), UP)
    assert out[0, 0] == 0.0 and np.allclose(out, ref, rtol=0, atol=1e-12)


def test_standardized_rejects_integer_input(env):
    gx, g, _ = env
    with pytest.raises(RuntimeError, match="float32 or float64"):
        gx.matmul_standardized(g, np.ones((1, g.num_samples), dtype=np.int32), UP)
