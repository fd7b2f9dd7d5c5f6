"""The device plan builder (heights, renumbering, UP adjacency and parent counts on the GPU)
lays out exactly the plan of the host builder: every product, floats included, is bit-identical
between graphs uploaded either way."""
import ctypes

import numpy as np
import pytest

import oracle
from tests.conftest import kat_graph_arrays

pytestmark = pytest.mark.gpu
DOWN, UP = 1, 2


@pytest.fixture(scope="module")
def gx(cuda_ok):
    import grgl_gb300

    return grgl_gb300


def _host_planned(gx, make):
    from grgl_gb300 import _lib

    g = make()
    fn = _lib.lib().grgx_graph_upload_host_plan
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p]
    _lib.check(fn(g._h))
    return g


def _same_products(gx, a, b, rng):
    for dt in (np.float32, np.float64, np.int32):
        for K in (1, 5, 64):
            for d, cols in ((UP, a.num_samples), (DOWN, a.num_mutations)):
                V = (rng.standard_normal((K, cols)) if dt != np.int32
                     else rng.integers(-9, 9, size=(K, cols))).astype(dt)
                assert np.array_equal(gx.matmul(a, V, d), gx.matmul(b, V, d)), (dt, K, d)


@pytest.mark.parametrize("N,M,seed", [(3000, 20000, 81), (500, 900, 82)])
def test_device_plan_equals_host_plan(gx, N, M, seed):
    dev = gx.window_tree_grg(N, M, seed=seed).upload()
    host = _host_planned(gx, lambda: gx.window_tree_grg(N, M, seed=seed))
    assert dev.info()["num_levels"] == host.info()["num_levels"]
    assert dev.info()["device_bytes"] == host.info()["device_bytes"]
    _same_products(gx, dev, host, np.random.default_rng(seed))


def test_device_plan_unordered_ids(gx):
    """Node ids that are not topologically ordered (a parent before its child)."""
    # samples 0..3; node 4 is a parent of node 6, node 6 of samples 0, 1; node 5 of 2, 3
    arrs = dict(num_samples=4, ploidy=2, down_off=np.array([0, 0, 0, 0, 0, 2, 4, 6], dtype=np.uint64),
                down_adj=np.array([6, 3, 2, 3, 0, 1], dtype=np.uint32), mut_node=np.array([4, 5, 6], dtype=np.uint32))
    dev = gx.from_csr(**arrs).upload()
    host = _host_planned(gx, lambda: gx.from_csr(**arrs))
    og = oracle.OracleGraph(**arrs)
    V = np.arange(12, dtype=np.float64).reshape(3, 4)
    assert np.array_equal(gx.matmul(dev, V, UP), oracle.matmul(og, V, UP))
    _same_products(gx, dev, host, np.random.default_rng(1))


def test_cycle_reported(gx):
    arrs = dict(num_samples=2, ploidy=2, down_off=np.array([0, 0, 0, 2, 3], dtype=np.uint64),
                down_adj=np.array([0, 3, 2], dtype=np.uint32), mut_node=np.array([2], dtype=np.uint32))
    g = gx.from_csr(**arrs)
    with pytest.raises(RuntimeError, match="GRG contains a cycle"):
        g.upload()


def test_kat_graph_device_plan(gx):
    a = kat_graph_arrays()
    g = gx.from_csr(**a).upload()
    og = oracle.OracleGraph(**a)
    V = np.ones((1, og.num_samples), dtype=np.int64)
    assert np.array_equal(gx.matmul(g, V, UP), oracle.matmul(og, V, UP))


@pytest.mark.parametrize("fixture", ["t200", "t200miss", "wt_n1000_m10000"])
def test_grg_decoded_on_device(gx, fixture):
    """A .grg's buckets decoded on the GPU give the plan (and every product) of the same file
    decoded on the host."""
    from tests.conftest import GOLDEN

    path = str(GOLDEN / f"{fixture}.grg")
    dev = gx.load_immutable_grg(path).upload()
    host = _host_planned(gx, lambda: gx.load_immutable_grg(path))
    assert dev.info()["device_bytes"] == host.info()["device_bytes"]
    _same_products(gx, dev, host, np.random.default_rng(7))
    o = oracle.read_grg(GOLDEN / f"{fixture}.grg")
    V = np.ones((1, o.num_samples), dtype=np.int32)
    assert np.array_equal(gx.matmul(dev, V, UP), oracle.matmul(o, V, UP))
    # the host copy is still there for host consumers after a device decode
    a = dev.export_arrays()
    assert np.array_equal(a["down_adj"], o.down_adj)


def test_corrupt_bucket_reported_on_device(gx, tmp_path):
    from tests.conftest import GOLDEN

    raw = bytearray((GOLDEN / "t200.grg").read_bytes())
    raw[136:142] = b"\xff" * 6
    bad = tmp_path / "badbucket.grg"
    bad.write_bytes(bytes(raw))
    g = gx.load_immutable_grg(str(bad))
    with pytest.raises(RuntimeError, match="Malformed GRG file"):
        g.upload()
