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


def test_standardized_requests_batched_and_served(env):
    """Standardized requests stacked beside plain ones (one traversal) and through the server
    give the standardized product; the plain requests beside them are unaffected."""
    import torch

    gx, g, og = env
    rng = np.random.default_rng(4)
    reqs = []
    for i in range(12):
        d = UP if i % 2 else DOWN
        dt = np.float32 if i % 3 else np.float64
        V = rng.standard_normal((int(rng.integers(1, 9)), g.num_samples if d == UP else g.num_mutations)).astype(dt)
        reqs.append((V, d, i % 4 != 0))
    for outs in (gx.matmul_batch(g, reqs),
                 [o.cpu().numpy() for o in gx.matmul_batch(g, [(torch.from_numpy(V).cuda(), d, st)
                                                               for V, d, st in reqs])]):
        for (V, d, st), got in zip(reqs, outs):
            rtol = 1e-6 if V.dtype == np.float32 else 1e-12
            if st:
                ref, scale = oracle.standardized(og, V, d, return_scale=True)
            else:
                ref = oracle.matmul(og, V.astype(np.float64), d)
                scale = oracle.matmul(og, np.abs(V).astype(np.float64), d)
            err = np.abs(got.astype(np.float64) - ref)
            assert np.all(err <= rtol * scale + 1e-300), (d, st, V.dtype)
    with gx.Server(workers=2) as srv:
        gid = srv.add_graph(g)
        tickets = [srv.submit(gid, V, d, standardized=st) for V, d, st in reqs]
        for (V, d, st), t in zip(reqs, tickets):
            got, _ = srv.result(t, timeout=120)
            if st:
                ref, scale = oracle.standardized(og, V, d, return_scale=True)
                rtol = 1e-6 if V.dtype == np.float32 else 1e-12
                assert np.all(np.abs(got.astype(np.float64) - ref) <= rtol * scale + 1e-300)
    with pytest.raises(RuntimeError, match="float32 or float64"):
        gx.matmul_batch(g, [(np.ones((1, g.num_samples), dtype=np.int32), UP, True)])


@pytest.mark.parametrize("standardized", [False, True])
def test_gram_products_match_dense(env, standardized):
    """V X X^T / V X^T X (and with Z) from two chained device traversals against dense float64."""
    import torch

    gx, g, og = env
    X = og.dense_X().astype(np.float64)
    N = X.shape[0]
    if standardized:
        mu = X.sum(axis=0) / N
        var = mu * (1 - mu)
        inv = np.where(var > 0, 1 / np.sqrt(np.where(var > 0, var, 1.0)), 0.0)
        X = (X - mu[None, :]) * inv[None, :]
    rng = np.random.default_rng(5)
    for first, cols in ((UP, g.num_samples), (DOWN, g.num_mutations)):
        V = rng.standard_normal((3, cols))
        ref = V @ X @ X.T if first == UP else V @ X.T @ X
        scale = np.abs(V) @ np.abs(X) @ np.abs(X).T if first == UP else np.abs(V) @ np.abs(X).T @ np.abs(X)
        got = gx.matmul_gram(g, V, first, standardized=standardized)
        assert np.all(np.abs(got - ref) <= 1e-11 * scale + 1e-300)
        dev = gx.matmul_gram(g, torch.from_numpy(V).cuda(), first, standardized=standardized)
        torch.cuda.synchronize()
        assert np.array_equal(dev.cpu().numpy(), got)
    Vi = rng.integers(-3, 4, size=(2, g.num_samples)).astype(np.int64)
    if not standardized:
        assert np.array_equal(gx.matmul_gram(g, Vi, UP), Vi @ og.dense_X().astype(np.int64) @ og.dense_X().T)
