"""The reference's end-to-end matmul tests, restated against grgl_gb300 on the GPU.

Each test below makes the checks of the reference test it names, on the graphs the reference
constructor built from the same inputs (`t200.grg` from test-200-samples.vcf.gz, `t200miss.grg`
from test-200-samples.miss.igd; tests/golden/make_golden.py):
  test/endtoend/test_matmul.py   different_methods, diploid, xtx_init, vector_init, matrix_init,
                                 init_failures, parallel (range shards instead of `grg split`)
  test/endtoend/test_missing.py  muts, mult
The dense genotype matrices are built here from the down edges (test_matmul.py:21-38 and
testing_utils.py grg2X / allele_frequencies), independently of the oracle.
"""
import concurrent.futures

import numpy as np
import pytest

from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu
INVALID = 0x7FFFFFFF


@pytest.fixture(scope="module")
def gx(cuda_ok):
    import grgl_gb300

    return grgl_gb300


class Dense:
    """Samples below each node, with path multiplicity, from the down edges."""

    def __init__(self, g):
        a = g.export_arrays()
        self.g, self.a = g, a
        self.n, self.N, self.M = g.num_nodes, g.num_samples, g.num_mutations
        off, adj = a["down_off"].astype(np.int64), a["down_adj"].astype(np.int64)
        self.children = [adj[off[v]:off[v + 1]] for v in range(self.n)]
        below = np.zeros((self.n, self.N), dtype=np.int64)
        for v in self._children_first():
            if v < self.N:
                below[v, v] += 1
            for c in self.children[v]:
                below[v] += below[c]
        self.below = below
        self.parents = [[] for _ in range(self.n)]
        for v in range(self.n):
            for c in self.children[v]:
                self.parents[c].append(v)

    def _children_first(self):
        seen, order = np.zeros(self.n, dtype=bool), []
        for root in range(self.n):
            stack = [(root, False)]
            while stack:
                v, done = stack.pop()
                if done:
                    order.append(v)
                    continue
                if seen[v]:
                    continue
                seen[v] = True
                stack.append((v, True))
                stack.extend((int(c), False) for c in self.children[v] if not seen[c])
        return order

    def X(self, individual=False):
        """N x M (or individuals x M) genotype matrix, path multiplicities (test_matmul.py:21-38)."""
        out = np.zeros((self.N, self.M))
        for m, node in enumerate(self.a["mut_node"]):
            if node != INVALID:
                out[:, m] += self.below[node]
        if individual:
            out = out.reshape(self.N // self.g.ploidy, self.g.ploidy, self.M).sum(axis=1)
        return out


@pytest.fixture(scope="module")
def t200(gx):
    g = gx.load_immutable_grg(str(GOLDEN / "t200.grg"))
    return g, Dense(g)


def test_different_methods(gx, t200):
    g, dense = t200
    rng = np.random.default_rng(42)
    X = dense.X()
    for direction, size, ref in ((gx.UP, g.num_samples, lambda V: V @ X),
                                 (gx.DOWN, g.num_mutations, lambda V: V @ X.T)):
        vects = rng.random((100, size))
        dots = np.array([gx.dot_product(g, v, direction) for v in vects])
        assert np.allclose(dots, ref(vects))
        assert np.allclose(dots, gx.matmul(g, vects, direction))


def test_diploid(gx, t200):
    g, dense = t200
    rng = np.random.default_rng(43)
    Xi = dense.X(individual=True)
    V = rng.random((10, g.num_individuals))
    assert np.allclose(gx.matmul(g, V, gx.UP, by_individual=True), V @ Xi)
    V = rng.random((10, g.num_mutations))
    assert np.allclose(gx.matmul(g, V, gx.DOWN, by_individual=True), V @ Xi.T)


def test_xtx_init(gx, t200):
    g, dense = t200
    coals = dense.a["coals"]
    if len(coals) == 0 or np.any(coals == gx.COAL_COUNT_NOT_SET):
        pytest.skip("graph without individual coalescence counts")
    assert g.ploidy == 2 and np.all(coals <= g.num_samples // 2)
    xx = np.zeros(dense.n, dtype=np.int64)
    for v in dense._children_first():
        xx[v] = 1 if v < dense.N else int(xx[dense.children[v]].sum()) + 2 * int(coals[v - dense.N])
    got = gx.matmul(g, np.ones((2, g.num_samples), dtype=np.int32), gx.UP, init="xtx")
    for m, node in enumerate(dense.a["mut_node"]):
        if node != INVALID:
            assert got[0, m] == xx[node] and got[1, m] == xx[node]


def test_vector_init(gx, t200):
    g, _ = t200
    K = 10
    ones = np.ones((K, g.num_samples))
    without = gx.matmul(g, ones, gx.UP)
    with_init = gx.matmul(g, ones, gx.UP, init=np.full(K, 2.0))
    assert without.shape == with_init.shape and np.all(with_init >= 2 * without)


def test_matrix_init(gx, t200):
    g, dense = t200
    K = 10
    ones = np.ones((K, g.num_samples), dtype=np.int64)
    init = np.zeros((K, g.num_nodes), dtype=np.int64)
    without = gx.matmul(g, ones, gx.UP)
    assert np.array_equal(gx.matmul(g, ones, gx.UP, init=init), without)
    tweak = int(np.random.default_rng(44).integers(g.num_samples, g.num_nodes - 100))
    # the mutations on the tweaked node and on every node above it
    above, stack, seen = set(), [tweak], set()
    while stack:
        v = stack.pop()
        if v in seen:
            continue
        seen.add(v)
        above.update(np.flatnonzero(dense.a["mut_node"] == v).tolist())
        stack.extend(dense.parents[v])
    init[4, tweak] = 100
    got = gx.matmul(g, ones, gx.UP, init=init)
    rows = np.arange(K) != 4
    assert np.array_equal(got[rows], without[rows])
    hit = np.zeros(g.num_mutations, dtype=bool)
    hit[list(above)] = True
    assert np.array_equal(got[4, ~hit], without[4, ~hit]) and np.all(got[4, hit] > without[4, hit])


def test_init_failures(gx, t200):
    g, _ = t200
    N = g.num_samples
    bad = [
        (np.ones((1, N)), dict(init=np.ones((1, 200000)))),               # init matrix of the wrong shape
        (np.ones((1, N)), dict(init=np.ones((2, N)))),                    # init matrix of the wrong shape
        (np.ones((1, N), dtype=np.int32), dict(init=np.ones((1, N)))),    # init dtype differs
        (np.ones((1, N), dtype=np.int32), dict(init="test")),             # unknown init string
        (np.ones((9, N)), dict(init=np.ones(10))),                        # init vector too long
    ]
    for V, kw in bad:
        with pytest.raises(RuntimeError):
            gx.matmul(g, V, gx.UP, **kw)


def test_parallel(gx, t200):
    """Range shards multiplied from four threads at once sum to the whole graph's DOWN product.
    Each round takes fresh shards, so the threads' first calls -- device plans built on the
    legacy stream, CUDA graphs captured on others -- overlap every time."""
    from grgl_gb300.shard import split_by_mutations

    g, _ = t200
    for rnd in range(5):
        V = np.random.default_rng(45 + rnd).standard_normal((10, g.num_mutations))
        full = gx.matmul(g, V, gx.DOWN)
        ranges, shards = split_by_mutations(g, 4)
        assert sum(s.num_mutations for s in shards) == g.num_mutations
        with concurrent.futures.ThreadPoolExecutor(max_workers=4) as ex:
            futures = [ex.submit(gx.matmul, s, V[:, r.start:r.stop], gx.DOWN) for s, r in zip(shards, ranges)]
            parts = [f.result() for f in futures]
        np.testing.assert_allclose(full, np.sum(parts, axis=0))


# ---- test/endtoend/test_missing.py -------------------------------------------------------------

MISSING_INDIVS = 21
MISSING_SAMPLES = 25


@pytest.fixture(scope="module")
def t200miss(gx):
    g = gx.load_immutable_grg(str(GOLDEN / "t200miss.grg"))
    return g, Dense(g)


def test_missing_muts(gx, t200miss):
    g, dense = t200miss
    total, total_indiv = 0, 0
    for m, (node, miss) in enumerate(zip(dense.a["mut_node"], dense.a["miss_node"])):
        if node != INVALID and miss != INVALID:
            assert dense.below[node].max() <= 1 and dense.below[miss].max() <= 1  # no sample twice
            ms = np.flatnonzero(dense.below[miss])
            total += len(ms)
            total_indiv += len(set((ms // 2).tolist()))
    assert total == MISSING_SAMPLES and total_indiv == MISSING_INDIVS


def allele_frequencies(gx, g):
    """testing_utils.allele_frequencies: counts / (N - missing), 0 where nothing is called."""
    miss = np.zeros((1, g.num_mutations), dtype=np.int32)
    counts = gx.matmul(g, np.ones((1, g.num_samples), dtype=np.int32), gx.UP, miss=miss)[0]
    denom = g.num_samples - miss[0]
    return np.divide(counts, denom, out=np.zeros(counts.shape), where=denom != 0)


def test_missing_mult(gx, t200miss):
    g, dense = t200miss
    freqs = allele_frequencies(gx, g)
    # diploid X with the allele frequency in every missing call
    X = dense.X(individual=True)
    for m, miss in enumerate(dense.a["miss_node"]):
        if miss != INVALID:
            per_indiv = dense.below[miss].reshape(-1, g.ploidy).sum(axis=1)
            X[:, m] += per_indiv * freqs[m]
    assert len(np.where((X > 0) & (X != 1) & (X != 2))[0]) == MISSING_INDIVS
    rng = np.random.default_rng(46)
    K = 7
    # UP: the missingness product lands in M; adding M * freqs gives the mean-imputed product
    rv = rng.standard_normal((K, g.num_individuals))
    M = np.zeros((K, g.num_mutations))
    got = gx.matmul(g, rv, gx.UP, by_individual=True, miss=M)
    np.testing.assert_allclose(rv @ X, got + M * freqs)
    # DOWN: missingness input freqs * rv weights the missing calls
    rv = rng.standard_normal((K, g.num_mutations))
    got = gx.matmul(g, rv, gx.DOWN, by_individual=True, miss=np.array([freqs]) * rv)
    np.testing.assert_allclose(rv @ X.T, got)
