"""Parity on the large window-tree graph against the oracle: N=1,000,000 haplotypes and the first
300,000 variants (seed 42, ~3e9 edges: above 2^31, so 64-bit edge offsets; UP runs in split
form), float32 (compensated) and float64 K=16 in both directions, within 1e-6 / 1e-12 of the sum
of |terms| per output.  A module of its own so that the benchmark graph of test_full_size.py is
freed before this one is built."""
import numpy as np
import pytest

from tests.test_full_size import check_vs_oracle, oracle_setup

pytestmark = pytest.mark.gpu
DOWN, UP = 1, 2


@pytest.fixture(scope="module")
def large_graph(cuda_ok):
    import torch

    import grgl_gb300 as gx

    g = gx.window_tree_grg(1_000_000, 300_000, seed=42).upload()
    og, sh = oracle_setup(g)
    yield gx, torch, g, og, sh
    del sh, og, g
    torch.cuda.empty_cache()


@pytest.mark.parametrize("dtype,direction", [(np.float32, UP), (np.float32, DOWN), (np.float64, UP),
                                             (np.float64, DOWN)])
def test_large_graph_vs_oracle(large_graph, dtype, direction):
    gx, torch, g, og, sh = large_graph
    assert g.num_edges > 2 ** 31
    check_vs_oracle(gx, torch, g, sh, np.random.default_rng(200 + direction), dtype, 16, direction)
