"""DOWN in split form (the height-0 rows' parents taken in blocks of parent ids, each row's sum
kept in accumulator form, then the rows written onto their seed values), the 16-bit block-relative
edge ids of both split copies, and the single-column passes that stage a block's source values in
shared memory: every combination gives the oracle's results -- integers bit-exact, floats within
the usual tolerances -- with the DOWN options (by_individual, emit_all_nodes, init, miss)."""
import ctypes

import numpy as np
import pytest

import oracle
from tests.conftest import GOLDEN, abs_scale, assert_matches

pytestmark = pytest.mark.gpu
DOWN, UP = 1, 2
DEFAULT_BLOCK, DEFAULT_THRESHOLD = 32768, 64 << 20


def _knobs(block=None, threshold=None, down_mode=None, staged=None):
    from grgl_gb300 import _lib

    lib = _lib.lib()
    if block is not None:
        fn = lib.grgx_debug_up_split
        fn.restype = None
        fn.argtypes = [ctypes.c_longlong, ctypes.c_ulonglong]
        fn(block, threshold)
    if down_mode is not None:
        fn = lib.grgx_debug_split_forms
        fn.restype = None
        fn.argtypes = [ctypes.c_int, ctypes.c_int]
        fn(down_mode, int(staged))


def _restore():
    _knobs(DEFAULT_BLOCK, DEFAULT_THRESHOLD, 0, True)


@pytest.fixture(scope="module")
def env(cuda_ok):
    import grgl_gb300 as gx

    _knobs(256, 0, 1, True)  # copies built now cut every 256 ids; UP and DOWN run split; staging on
    gx.set_graph_replay(False)  # every call runs the forms the knobs select (no replayed capture)
    try:
        g = gx.window_tree_grg(3000, 20000, seed=97).upload()
        a = g.export_arrays()
        og = oracle.OracleGraph(num_samples=3000, ploidy=2, down_off=a["down_off"], down_adj=a["down_adj"],
                                mut_node=a["mut_node"])
        yield gx, g, og
    finally:
        gx.set_graph_replay(True)
        _restore()


def _rand(rng, dt, shape):
    if np.dtype(dt).kind == "f":
        return rng.standard_normal(shape).astype(dt)
    if np.dtype(dt) == np.bool_:
        return rng.integers(0, 2, size=shape).astype(bool)
    return rng.integers(0, 50, size=shape).astype(dt)


def _check(og, V, direction, got, **kw):
    if V.dtype == np.float32:  # compensated float32 against the float64 product of the same inputs
        V = V.astype(np.float64)
        kw = {k: (v.astype(np.float64) if isinstance(v, np.ndarray) else v) for k, v in kw.items()}
        got = got.astype(np.float64)
        rtol = 1e-6
    else:
        rtol = 1e-12
    ref = oracle.matmul(og, V, direction, **{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in kw.items()})
    if V.dtype.kind == "f":
        scale = abs_scale(og, V, direction, kw)
        assert_matches(got.astype(np.float64), ref, scale, rtol=rtol)
    else:
        assert_matches(got, ref)


@pytest.mark.parametrize("staged", [True, False])
@pytest.mark.parametrize("dt", [np.int32, np.int64, np.uint16, np.float32, np.float64, np.bool_])
@pytest.mark.parametrize("K", [1, 7, 64])
def test_split_down_matches_oracle(env, staged, dt, K):
    gx, g, og = env
    _knobs(down_mode=1, staged=staged)
    try:
        V = _rand(np.random.default_rng(K + 7), dt, (K, g.num_mutations))
        _check(og, V, DOWN, gx.matmul(g, V, DOWN))
    finally:
        _knobs(down_mode=1, staged=True)


@pytest.mark.parametrize("staged", [True, False])
@pytest.mark.parametrize("dt", [np.int32, np.float32, np.bool_])
def test_split_up_single_column(env, staged, dt):
    """K=1 (and bool up to 32 columns): the staged block passes of the UP split form."""
    gx, g, og = env
    _knobs(down_mode=1, staged=staged)
    try:
        for K in ((1, 32) if dt == np.bool_ else (1,)):
            V = _rand(np.random.default_rng(K), dt, (K, g.num_samples))
            _check(og, V, UP, gx.matmul(g, V, UP))
    finally:
        _knobs(down_mode=1, staged=True)


def test_split_down_options(env):
    gx, g, og = env
    rng = np.random.default_rng(3)
    V = rng.standard_normal((5, g.num_mutations))
    init = rng.standard_normal(5)
    _check(og, V, DOWN, gx.matmul(g, V, DOWN, emit_all_nodes=True, init=init), emit_all_nodes=True, init=init)
    Vi = rng.integers(0, 9, size=(3, g.num_mutations)).astype(np.int32)
    _check(og, Vi, DOWN, gx.matmul(g, Vi, DOWN, by_individual=True), by_individual=True)
    V1 = rng.standard_normal((1, g.num_mutations)).astype(np.float32)
    initm = rng.standard_normal((1, g.num_nodes)).astype(np.float32)
    _check(og, V1, DOWN, gx.matmul(g, V1, DOWN, init=initm), init=initm)


def test_split_down_equals_unsplit_for_integers(env):
    gx, g, og = env
    V = np.random.default_rng(5).integers(-9, 9, size=(33, g.num_mutations)).astype(np.int32)
    gx.set_timing(True)
    try:
        blocked = gx.matmul(g, V, DOWN)
        n_blocked = gx.last_timing()["launches"]
        _knobs(down_mode=2, staged=True)  # same plan, the height-0 level on the unsplit DOWN CSR
        try:
            plain = gx.matmul(g, V, DOWN)
            n_plain = gx.last_timing()["launches"]
        finally:
            _knobs(down_mode=1, staged=True)
    finally:
        gx.set_timing(False)
    assert np.array_equal(blocked, plain)
    assert n_blocked > n_plain  # the split form ran: one launch per parent block plus the finish
    V1 = np.random.default_rng(6).integers(-9, 9, size=(1, g.num_mutations)).astype(np.int32)
    staged = gx.matmul(g, V1, DOWN)
    _knobs(down_mode=1, staged=False)
    try:
        unstaged = gx.matmul(g, V1, DOWN)
    finally:
        _knobs(down_mode=1, staged=True)
    assert np.array_equal(staged, unstaged)


def test_autotune_records_down_form(env):
    gx, g, og = env
    _knobs(down_mode=0, staged=True)
    try:
        rep = gx.autotune(g, np.int32, 1, DOWN)
        assert "DOWN runs" in rep
        V = np.random.default_rng(8).integers(0, 5, size=(1, g.num_mutations)).astype(np.int32)
        _check(og, V, DOWN, gx.matmul(g, V, DOWN))
    finally:
        gx.autotune_clear()
        _knobs(down_mode=1, staged=True)


def test_split_down_missingness_golden(cuda_ok):
    """The reference-built graph with missingness nodes, DOWN with `miss`, split into blocks of 64
    parent ids, against the oracle."""
    import grgl_gb300 as gx

    _knobs(64, 0, 1, True)
    gx.set_graph_replay(False)
    try:
        g = gx.load_immutable_grg(str(GOLDEN / "t200miss.grg")).upload()
        og = oracle.read_grg(GOLDEN / "t200miss.grg")
        rng = np.random.default_rng(11)
        for dt in (np.int32, np.float64):
            V = _rand(rng, dt, (3, g.num_mutations))
            miss = _rand(rng, dt, (3, g.num_mutations))
            got = gx.matmul(g, V, DOWN, miss=miss)
            _check(og, V, DOWN, got, miss=miss)
    finally:
        gx.set_graph_replay(True)
        _restore()
