"""Parity at the benchmark's full sizes, against the oracle (the reference algorithm restated in C,
run on all host cores with the reference's range-split pattern, test/endtoend/test_matmul.py:264-325).
The reference itself checks its GPU path against its CPU path on a large user-supplied graph
(test/unit/test_cuda_matmul.cpp:179-299); these are the same checks on the benchmark graphs:

* the window-tree GRG with N=200,000 haplotypes and M=1,000,000 variants (seed 42, ~2e9 edges):
  int32 K=1 and K=8 both directions bit-exact; float64 K=8 within 1e-12 and compensated float32
  K=8 within 1e-6 of the sum of |terms| per output (float32 against the oracle's float64 product
  of the same inputs); plus identities that need no oracle (ones totals, 0/1 inputs give exact
  integer sums through float64 and float32, integer linearity);
* the large graph: tests/test_full_size_large.py.
"""
import numpy as np
import pytest

from tests.conftest import assert_matches

pytestmark = pytest.mark.gpu
DOWN, UP = 1, 2


def oracle_setup(g):
    import oracle

    a = g.export_arrays()
    og = oracle.OracleGraph(num_samples=g.num_samples, ploidy=g.ploidy, down_off=a["down_off"],
                            down_adj=a["down_adj"], mut_node=a["mut_node"])
    return og, oracle.Shards(og, oracle.host_threads(), align=100)


def check_vs_oracle(gx, torch, g, sh, rng, dtype, K, direction):
    dtype = np.dtype(dtype)
    cols = g.num_samples if direction == UP else g.num_mutations
    if dtype.kind == "f":
        V = rng.standard_normal((K, cols)).astype(dtype)
    else:
        V = rng.integers(0, 2, size=(K, cols)).astype(dtype)
        V[0] = 1
    got = gx.matmul(g, torch.from_numpy(V).cuda(), direction)
    torch.cuda.synchronize()
    got = got.cpu().numpy()
    if dtype.kind != "f":
        assert_matches(got, sh.matmul(V, direction))
        return
    V64 = V.astype(np.float64)
    ref = sh.matmul(V64, direction)
    scale = sh.matmul(np.abs(V64), direction)
    assert_matches(got.astype(np.float64), ref, scale, rtol=1e-6 if dtype == np.float32 else 1e-12)


@pytest.fixture(scope="module")
def bench_graph(cuda_ok):
    import torch

    import grgl_gb300 as gx

    g = gx.window_tree_grg(200_000, 1_000_000, seed=42).upload()
    og, sh = oracle_setup(g)
    yield gx, torch, g, og, sh
    del sh, og, g
    torch.cuda.empty_cache()


@pytest.mark.parametrize("dtype,K,direction", [(np.int32, 1, UP), (np.int32, 1, DOWN), (np.int32, 8, UP),
                                               (np.int32, 8, DOWN), (np.float64, 8, UP), (np.float64, 8, DOWN),
                                               (np.float32, 8, UP), (np.float32, 8, DOWN)])
def test_benchmark_graph_vs_oracle(bench_graph, dtype, K, direction):
    gx, torch, g, og, sh = bench_graph
    assert g.num_edges > 1_900_000_000
    check_vs_oracle(gx, torch, g, sh, np.random.default_rng(100 + K + direction), dtype, K, direction)


def test_benchmark_graph_properties(bench_graph):
    """Checks that need no oracle: UP and DOWN ones totals agree (= nnz of X); 0/1 genotype inputs
    give integer sums that float64 (float pairs; UP in split form at K=64) and compensated float32
    reproduce exactly; integer linearity."""
    gx, torch, g, og, sh = bench_graph
    N, M = g.num_samples, g.num_mutations
    rng = np.random.default_rng(8)
    up1 = gx.matmul(g, torch.ones((1, N), dtype=torch.int64, device="cuda"), UP)
    down1 = gx.matmul(g, torch.ones((1, M), dtype=torch.int64, device="cuda"), DOWN)
    assert int(up1.sum()) == int(down1.sum()) > 0
    for d, cols in ((UP, N), (DOWN, M)):
        X = torch.from_numpy(rng.integers(0, 2, size=(64, cols)).astype(np.int64)).cuda()
        exact = gx.matmul(g, X, d)
        assert torch.equal(gx.matmul(g, X.double(), d), exact.double())
        assert torch.equal(gx.matmul(g, X[:16].float(), d), exact[:16].float())
        a = torch.from_numpy(rng.integers(-50, 50, size=(2, cols)).astype(np.int32)).cuda()
        b = torch.from_numpy(rng.integers(-50, 50, size=(2, cols)).astype(np.int32)).cuda()
        assert torch.equal(gx.matmul(g, 3 * a - 7 * b, d), 3 * gx.matmul(g, a, d) - 7 * gx.matmul(g, b, d))
