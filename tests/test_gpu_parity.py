"""GPU parity: the sm_103a kernels (through the C ABI) against the reference's golden outputs and
the CPU oracle.  Integers and bool are bit-exact; float64 is within 1e-12 and compensated float32
within 1e-6 of the float64 result, both relative to the per-output sum of |terms|."""
import numpy as np
import pytest

import oracle
from tests.conftest import GOLDEN, abs_scale, assert_matches, kat_graph_arrays, load_golden, sample8_arrays
from tests.golden.cases import cases_for

pytestmark = pytest.mark.gpu
DOWN, UP = 1, 2


@pytest.fixture(scope="module")
def gx(cuda_ok):
    import grgl_gb300

    return grgl_gb300


def _run_both(gx, g, og, V, direction, **kw):
    kw = dict(kw)
    miss = kw.pop("miss", None)
    m_gpu = None if miss is None else miss.copy()
    m_ref = None if miss is None else miss.copy()
    got = gx.matmul(g, V, direction, miss=m_gpu, **kw)
    ref = oracle.matmul(og, V, direction, miss=m_ref, **kw)
    return got, ref, m_gpu, m_ref


def test_kats_on_gpu(gx):
    g = gx.from_csr(**kat_graph_arrays((1, 5, 6)))
    assert gx.matmul(g, np.array([[1.0, 2.0, 1.0]]), DOWN).tolist() == [[1.0, 2.0, 3.0, 3.0]]
    assert gx.matmul(g, np.ones((1, 4)), UP).tolist() == [[1.0, 2.0, 4.0]]
    V = np.array([[1.0, 2.0, 1.0], [0.0, 1.0, 1.0]])
    assert gx.matmul(g, V, DOWN).ravel().tolist() == [1, 2, 3, 3, 1, 1, 2, 2]
    assert gx.dot_product(g, np.ones(4), UP).tolist() == [1.0, 2.0, 4.0]
    g2 = gx.from_csr(**kat_graph_arrays((6, 5, 4)), coals=np.array([1, 1, 0], dtype=np.uint32))
    assert gx.matmul(g2, np.ones((1, 4), dtype=np.int64), UP, init="xtx").tolist() == [[8, 4, 4]]
    assert gx.matmul(g2, np.array([[11, 41, 37, 73]], dtype=np.int64), UP).tolist() == [[162, 110, 52]]
    # unordered node ids (a parent below its children): still {162, 110, 52}
    g3 = gx.from_csr(num_samples=4, ploidy=2, down_off=np.array([0, 0, 0, 0, 0, 2, 4, 6], dtype=np.uint64),
                     down_adj=np.array([6, 5, 2, 3, 0, 1], dtype=np.uint32), mut_node=np.array([4, 5, 6]))
    assert gx.matmul(g3, np.array([[11, 41, 37, 73]], dtype=np.int64), UP).tolist() == [[162, 110, 52]]
    g8 = gx.from_csr(**sample8_arrays())
    og8 = oracle.OracleGraph(**sample8_arrays())
    assert np.array_equal(gx.matmul(g8, np.eye(8, dtype=np.int64), UP), og8.dense_X())


@pytest.mark.parametrize("fixture", ["t200", "t200miss", "wt_n1000_m10000"])
def test_reference_golden_outputs(gx, fixture):
    z, meta = load_golden(fixture)
    g = gx.load_immutable_grg(str(GOLDEN / f"{fixture}.grg"))
    og = oracle.read_grg(GOLDEN / f"{fixture}.grg")
    for name, (V, direction, kw) in cases_for(og.num_samples, og.num_mutations, og.num_nodes, og.ploidy,
                                              has_miss=bool(meta.get("miss")), profile=meta["profile"]):
        kw = dict(kw)
        miss = kw.pop("miss", None)
        m_gpu = None if miss is None else miss.copy()
        got = gx.matmul(g, V, direction, miss=m_gpu, **kw)
        scale = abs_scale(og, V, direction, dict(kw, miss=miss))
        if V.dtype == np.float32:
            # compensated float32 against the float64 product of the same inputs
            kw64 = {k: (v.astype(np.float64) if isinstance(v, np.ndarray) else v) for k, v in kw.items()}
            ref64 = oracle.matmul(og, V.astype(np.float64), direction, **kw64)
            assert_matches(got.astype(np.float64), ref64, scale.astype(np.float64), rtol=1e-6)
            assert_matches(got, z[name], scale, rtol=1e-5)
        else:
            assert_matches(got, z[name], scale)
        if miss is not None and direction == UP:
            mscale = None
            if V.dtype.kind == "f":
                mscale = np.abs(miss) + abs_scale(og, V, direction, dict(kw, miss=np.zeros_like(miss)))
            assert_matches(m_gpu, z[name + "__miss"], mscale)


KS = [1, 2, 3, 4, 5, 8, 16, 31, 32, 33, 64, 65, 128, 129, 257]


@pytest.fixture(scope="module")
def wt(gx):
    g = gx.window_tree_grg(2000, 20000, seed=5)
    a = g.export_arrays()
    og = oracle.OracleGraph(num_samples=2000, ploidy=2, down_off=a["down_off"], down_adj=a["down_adj"],
                            mut_node=a["mut_node"])
    return g, og


@pytest.mark.parametrize("K", KS)
@pytest.mark.parametrize("dtype", [np.int32, np.float64, np.float32, np.int64])
def test_window_tree_vs_oracle(gx, wt, K, dtype):
    g, og = wt
    rng = np.random.default_rng(K)
    for direction, cols in ((UP, og.num_samples), (DOWN, og.num_mutations)):
        if np.dtype(dtype).kind == "f":
            V = rng.standard_normal((K, cols)).astype(dtype)
        else:
            V = rng.integers(-1000, 1000, size=(K, cols)).astype(dtype)
        got = gx.matmul(g, V, direction)
        if np.dtype(dtype) == np.float32:
            ref = oracle.matmul(og, V.astype(np.float64), direction)
            scale = oracle.matmul(og, np.abs(V).astype(np.float64), direction)
            assert_matches(got.astype(np.float64), ref, scale, rtol=1e-6)
        else:
            ref = oracle.matmul(og, V, direction)
            scale = oracle.matmul(og, np.abs(V), direction) if np.dtype(dtype).kind == "f" else None
            assert_matches(got, ref, scale)


def test_plain_f32_option(gx, wt):
    g, og = wt
    V = np.random.default_rng(0).standard_normal((8, og.num_samples)).astype(np.float32)
    got = gx.matmul(g, V, UP, f32_compensated=False)
    ref = oracle.matmul(og, V.astype(np.float64), UP)
    scale = oracle.matmul(og, np.abs(V).astype(np.float64), UP)
    assert_matches(got.astype(np.float64), ref, scale, rtol=2e-5)


def test_bool_many_words(gx, wt):
    g, og = wt
    rng = np.random.default_rng(1)
    for K in (1, 31, 32, 33, 100, 200):
        for direction, cols in ((UP, og.num_samples), (DOWN, og.num_mutations)):
            V = rng.random((K, cols)) < 0.3
            assert_matches(gx.matmul(g, V, direction), oracle.matmul(og, V, direction))


def _star_graph(N, extra_parents=0):
    """One node over every sample (a heavy row in UP) plus `extra_parents` nodes over sample 0
    (a heavy row in DOWN)."""
    off = [0] * (N + 1)
    adj = list(range(N))
    off.append(len(adj))
    for _ in range(extra_parents):
        adj.append(0)
        off.append(len(adj))
    n = len(off) - 1
    mut = np.arange(N, n, dtype=np.uint32)
    return dict(num_samples=N, ploidy=2, down_off=np.array(off, dtype=np.uint64),
                down_adj=np.array(adj, dtype=np.uint32), mut_node=mut)


@pytest.mark.parametrize("dtype", [np.int32, np.float64, np.float32])
def test_heavy_rows(gx, dtype):
    arrs = _star_graph(300000, extra_parents=50000)
    g = gx.from_csr(**arrs)
    og = oracle.OracleGraph(**arrs)
    rng = np.random.default_rng(2)
    for K in (1, 4, 40, 136):  # 136: a narrow last column tile, launched on its own
        for direction, cols in ((UP, og.num_samples), (DOWN, og.num_mutations)):
            V = (rng.standard_normal((K, cols)) if np.dtype(dtype).kind == "f"
                 else rng.integers(-9, 9, size=(K, cols))).astype(dtype)
            got = gx.matmul(g, V, direction)
            if np.dtype(dtype) == np.float32:
                ref = oracle.matmul(og, V.astype(np.float64), direction)
                scale = oracle.matmul(og, np.abs(V).astype(np.float64), direction)
                assert_matches(got.astype(np.float64), ref, scale, rtol=1e-6)
            else:
                scale = oracle.matmul(og, np.abs(V), direction) if np.dtype(dtype).kind == "f" else None
                assert_matches(got, oracle.matmul(og, V, direction), scale)
            # deterministic: a second run is bitwise identical
            assert np.array_equal(got, gx.matmul(g, V, direction))


def test_edge_cases(gx):
    # no edges at all, some mutations unmapped
    arrs = dict(num_samples=6, ploidy=2, down_off=np.zeros(7, dtype=np.uint64), down_adj=np.zeros(0, np.uint32),
                mut_node=np.array([0, oracle.INVALID_NODE, 5], dtype=np.uint32))
    g = gx.from_csr(**arrs)
    og = oracle.OracleGraph(**arrs)
    for direction, cols in ((UP, 6), (DOWN, 3)):
        V = np.arange(2 * cols, dtype=np.int32).reshape(2, cols) + 1
        assert_matches(gx.matmul(g, V, direction), oracle.matmul(og, V, direction))
        assert_matches(gx.matmul(g, V, direction, emit_all_nodes=True),
                       oracle.matmul(og, V, direction, emit_all_nodes=True))
    # a single sample, a single mutation on it
    arrs = dict(num_samples=1, ploidy=1, down_off=np.zeros(2, dtype=np.uint64), down_adj=np.zeros(0, np.uint32),
                mut_node=np.array([0], dtype=np.uint32))
    g = gx.from_csr(**arrs)
    assert gx.matmul(g, np.array([[7.5]]), UP).tolist() == [[7.5]]
    assert gx.matmul(g, np.array([[7.5]]), DOWN).tolist() == [[7.5]]


def test_integer_wraparound(gx, wt):
    g, og = wt
    V = np.full((2, og.num_samples), 2 ** 30, dtype=np.int32)
    assert_matches(gx.matmul(g, V, UP), oracle.matmul(og, V, UP))
    V8 = np.full((3, og.num_mutations), 100, dtype=np.int8)
    assert_matches(gx.matmul(g, V8, DOWN), oracle.matmul(og, V8, DOWN))


def test_device_tensors_match_host(gx, wt):
    import torch

    g, og = wt
    rng = np.random.default_rng(9)
    for dtype in (np.float64, np.int32, np.float32):
        V = (rng.standard_normal((16, og.num_mutations)) * 10).astype(dtype)
        host = gx.matmul(g, V, DOWN)
        dev = gx.matmul(g, torch.from_numpy(V).cuda(), DOWN)
        torch.cuda.synchronize()
        assert dev.is_cuda and np.array_equal(dev.cpu().numpy(), host)


def test_large_window_tree_properties(gx):
    """Size-independent checks at a larger size: UP ones total == DOWN ones total (= nnz of X),
    and exact integer linearity."""
    N, M = 20000, 200000
    g = gx.window_tree_grg(N, M, seed=42)
    up = gx.matmul(g, np.ones((1, N), dtype=np.int64), UP)
    down = gx.matmul(g, np.ones((1, M), dtype=np.int64), DOWN)
    assert up.sum() == down.sum() > 0
    rng = np.random.default_rng(4)
    a = rng.integers(-100, 100, size=(3, N)).astype(np.int64)
    b = rng.integers(-100, 100, size=(3, N)).astype(np.int64)
    assert np.array_equal(gx.matmul(g, 3 * a - 7 * b, UP), 3 * gx.matmul(g, a, UP) - 7 * gx.matmul(g, b, UP))
    # DOWN(1) per sample is the number of mutations carried; UP(1) per mutation its count
    assert up.min() >= 1 and down.max() <= M


def test_f64_extreme_magnitudes_and_native(gx, wt):
    """float64 rows are scaled by powers of two before the float-pair sweep: rows of 1e300,
    1e-300 and mixed magnitudes keep 1e-12 accuracy; the FP64-pipe variant agrees too."""
    g, og = wt
    rng = np.random.default_rng(12)
    for direction, cols in ((UP, og.num_samples), (DOWN, og.num_mutations)):
        V = rng.standard_normal((4, cols))
        V[0] *= 1e300
        V[1] *= 1e-300
        V[2, ::7] *= 1e200
        V[3] *= 1e-310  # subnormal row
        ref = oracle.matmul(og, V, direction)
        scale = oracle.matmul(og, np.abs(V), direction)
        assert_matches(gx.matmul(g, V, direction), ref, scale)
        assert_matches(gx.matmul(g, V, direction, f64_native=True), ref, scale)


def test_f64_nonfinite_propagates_like_reference(gx, wt):
    g, og = wt
    rng = np.random.default_rng(13)
    for direction, cols in ((UP, og.num_samples), (DOWN, og.num_mutations)):
        V = rng.standard_normal((3, cols))
        V[0, 5] = np.inf
        V[1, 9] = np.nan
        V[2, 3], V[2, 4] = np.inf, -np.inf
        with np.errstate(invalid="ignore"):
            ref = oracle.matmul(og, V, direction)
            got = gx.matmul(g, V, direction)
        assert np.array_equal(np.isnan(got), np.isnan(ref))
        assert np.array_equal(np.isposinf(got), np.isposinf(ref))
        assert np.array_equal(np.isneginf(got), np.isneginf(ref))
        fin = np.isfinite(ref)
        with np.errstate(invalid="ignore"):
            scale = oracle.matmul(og, np.where(np.isfinite(V), np.abs(V), 0.0), direction)
        assert np.all(np.abs(got[fin] - ref[fin]) <= 1e-12 * scale[fin] + 1e-300)


def test_graph_replay_matches_direct(gx):
    """Small-graph calls replay a captured CUDA graph: same kernels, so bitwise the same results
    as the direct path, on repeated calls, several shapes and concurrent threads."""
    import threading
    import time

    g = gx.load_immutable_grg(str(GOLDEN / "t200.grg"))
    rng = np.random.default_rng(8)
    cases = [(rng.standard_normal((k, g.num_samples)).astype(dt), UP) for k, dt in ((1, np.float64), (5, np.float32))]
    cases += [(rng.integers(-9, 9, size=(3, g.num_mutations)).astype(np.int32), DOWN)]
    try:
        gx.set_graph_replay(False)
        direct = [gx.matmul(g, V, d) for V, d in cases]
        t0 = time.perf_counter()
        for _ in range(20):
            gx.matmul(g, cases[0][0], UP)
        t_direct = time.perf_counter() - t0
    finally:
        gx.set_graph_replay(True)
    for _ in range(3):
        for (V, d), ref in zip(cases, direct):
            assert np.array_equal(gx.matmul(g, V, d), ref)
    t0 = time.perf_counter()
    for _ in range(20):
        gx.matmul(g, cases[0][0], UP)
    t_graph = time.perf_counter() - t0
    print(f"t200 K=1 f64 UP per call: direct {1e3 * t_direct / 20:.3f} ms, graph replay {1e3 * t_graph / 20:.3f} ms")
    errors = []

    def worker(i):
        V, d = cases[i % len(cases)]
        for _ in range(10):
            if not np.array_equal(gx.matmul(g, V, d), direct[i % len(cases)]):
                errors.append(i)

    th = [threading.Thread(target=worker, args=(i,)) for i in range(6)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors


def test_deferred_timing(gx, wt):
    """Deferred timing records every call without synchronising; collection returns them in order."""
    import torch

    g, og = wt
    V = torch.ones((4, og.num_samples), dtype=torch.float32, device="cuda")
    gx.set_timing("deferred")
    try:
        for _ in range(3):
            gx.matmul(g, V, UP)
        ts = gx.collect_timings()
    finally:
        gx.set_timing(False)
    assert len(ts) == 3 and all(t["total_ms"] >= t["sweep_ms"] > 0 and t["launches"] > 0 for t in ts)
    assert gx.collect_timings() == []
