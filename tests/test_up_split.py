"""UP in split form (edges to height-0 children taken first, in passes over blocks of height-0
ids, each node's sum kept in accumulator form; the other edges level by level) gives the oracle's
results: integers bit-exact, floats within the usual tolerances, with every option of the UP
direction."""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
DOWN, UP = 1, 2
DEFAULT_BLOCK, DEFAULT_THRESHOLD = 32768, 64 << 20


def _split_knobs(block, threshold):
    from grgl_gb300 import _lib

    fn = _lib.lib().grgx_debug_up_split
    fn.restype = None
    fn.argtypes = [ctypes.c_longlong, ctypes.c_ulonglong]
    fn(block, threshold)


@pytest.fixture(scope="module")
def env(cuda_ok):
    import grgl_gb300 as gx

    _split_knobs(256, 0)  # split copies built now cut every 256 height-0 ids; every UP call runs split
    try:
        g = gx.window_tree_grg(3000, 20000, seed=91).upload()
        a = g.export_arrays()
        og = oracle.OracleGraph(num_samples=3000, ploidy=2, down_off=a["down_off"], down_adj=a["down_adj"],
                                mut_node=a["mut_node"])
        yield gx, g, og
    finally:
        _split_knobs(DEFAULT_BLOCK, DEFAULT_THRESHOLD)


def _check(got, ref, scale, dt):
    if np.dtype(dt).kind == "f":
        rtol = 1e-6 if dt == np.float32 else 1e-12
        assert np.all(np.abs(got.astype(np.float64) - ref) <= rtol * scale + 1e-300)
    else:
        assert np.array_equal(got, ref)


@pytest.mark.parametrize("dt", [np.int32, np.int64, np.uint16, np.float32, np.float64])
@pytest.mark.parametrize("K", [1, 7, 64, 200])
def test_split_up_matches_oracle(env, dt, K):
    gx, g, og = env
    rng = np.random.default_rng(K)
    V = (rng.standard_normal((K, g.num_samples)) if np.dtype(dt).kind == "f"
         else rng.integers(0, 50, size=(K, g.num_samples))).astype(dt)
    got = gx.matmul(g, V, UP)
    if np.dtype(dt).kind == "f":
        ref = oracle.matmul(og, V.astype(np.float64), UP)
        scale = oracle.matmul(og, np.abs(V).astype(np.float64), UP)
    else:
        ref, scale = oracle.matmul(og, V, UP), None
    _check(got, ref, scale, dt)


def test_split_up_options(env):
    gx, g, og = env
    rng = np.random.default_rng(3)
    V = rng.standard_normal((5, g.num_samples))
    init = rng.standard_normal(5)
    got = gx.matmul(g, V, UP, emit_all_nodes=True, init=init)
    ref = oracle.matmul(og, V, UP, emit_all_nodes=True, init=init)
    scale = oracle.matmul(og, np.abs(V), UP, emit_all_nodes=True, init=np.abs(init))
    _check(got, ref, scale, np.float64)
    Vb = rng.integers(0, 2, size=(40, g.num_samples)).astype(bool)
    assert np.array_equal(gx.matmul(g, Vb, UP), oracle.matmul(og, Vb, UP))
    Vi = rng.integers(0, 9, size=(3, g.num_individuals)).astype(np.int32)
    assert np.array_equal(gx.matmul(g, Vi, UP, by_individual=True), oracle.matmul(og, Vi, UP, by_individual=True))


def test_split_f64_extremes_take_native_path(env):
    gx, g, og = env
    V = np.random.default_rng(4).standard_normal((2, g.num_samples))
    V[0, :7] *= 1e200
    V[1, 3] = np.inf
    got = gx.matmul(g, V, UP)
    ref = oracle.matmul(og, V, UP)
    finite = np.isfinite(ref)
    assert np.array_equal(np.isfinite(got), finite)
    scale = oracle.matmul(og, np.where(np.isfinite(V), np.abs(V), 0.0), UP)
    assert np.all(np.abs(got[finite] - ref[finite]) <= 1e-12 * scale[finite] + 1e-300)


def test_split_equals_unsplit_for_integers(env):
    gx, g, og = env
    V = np.random.default_rng(5).integers(-9, 9, size=(33, g.num_samples)).astype(np.int32)
    blocked = gx.matmul(g, V, UP)
    _split_knobs(0, 1 << 62)  # same plan, every call on the unsplit UP CSR
    try:
        plain = gx.matmul(g, V, UP)
    finally:
        _split_knobs(0, 0)
    assert np.array_equal(blocked, plain)


def test_split_built_lazily_under_concurrent_calls(cuda_ok):
    """Threads that all make the graph's first UP call at once share one split copy and get the
    single-threaded results."""
    import threading

    import torch

    import grgl_gb300 as gx

    _split_knobs(256, 0)
    try:
        g = gx.window_tree_grg(2500, 9000, seed=93).upload()
        rng = np.random.default_rng(6)
        Vs = [rng.integers(-20, 20, size=(5, g.num_samples)).astype(np.int32) for _ in range(6)]
        outs = [None] * 6
        errs = []

        def work(i):
            try:
                outs[i] = gx.matmul(g, torch.from_numpy(Vs[i]).cuda(), UP).cpu().numpy()
            except Exception as e:  # reported below
                errs.append(e)

        th = [threading.Thread(target=work, args=(i,)) for i in range(6)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        assert not errs, errs
        a = g.export_arrays()
        og = oracle.OracleGraph(num_samples=2500, ploidy=2, down_off=a["down_off"], down_adj=a["down_adj"],
                                mut_node=a["mut_node"])
        for V, out in zip(Vs, outs):
            assert np.array_equal(out, oracle.matmul(og, V, UP))
    finally:
        _split_knobs(DEFAULT_BLOCK, DEFAULT_THRESHOLD)
