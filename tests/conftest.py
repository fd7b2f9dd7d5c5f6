"""Shared fixtures.  Tests marked `gpu` need a CUDA device; everything else runs on CPU."""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a build)")


@pytest.fixture(scope="session")
def lib_built():
    from grgl_gb300 import build

    build.build()
    import oracle

    oracle.build()
    return True


@pytest.fixture(scope="session")
def cuda_ok(lib_built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return True


def kat_graph_arrays(mut_nodes=(1, 5, 6)):
    """depth3BinTree (test/unit/common_grgs.h:13-27): 4 samples, pn4->(s0,s1), pn5->(s2,s3), pn6->(pn4,pn5)."""
    down_off = np.array([0, 0, 0, 0, 0, 2, 4, 6], dtype=np.uint64)
    down_adj = np.array([0, 1, 2, 3, 4, 5], dtype=np.uint32)
    return dict(num_samples=4, ploidy=2, down_off=down_off, down_adj=down_adj,
                mut_node=np.array(mut_nodes, dtype=np.uint32))


def sample8_arrays(mut_nodes=(8, 9, 10, 11, 12, 13)):
    """sample8Grg (test/unit/common_grgs.h:29-57)."""
    children = {8: [0, 1], 9: [2, 8], 10: [3, 4, 7], 11: [6, 8, 10], 12: [5, 10], 13: [9, 12]}
    off, adj = [0], []
    for v in range(14):
        adj += children.get(v, [])
        off.append(len(adj))
    return dict(num_samples=8, ploidy=2, down_off=np.array(off, dtype=np.uint64),
                down_adj=np.array(adj, dtype=np.uint32), mut_node=np.array(mut_nodes, dtype=np.uint32))


def load_golden(name):
    import json

    z = np.load(GOLDEN / f"{name}.npz")
    meta = json.loads(bytes(z["__meta__"]).decode())
    return z, meta


def abs_scale(og, V, direction, kw):
    """Per-output sum of |terms| (the oracle on |inputs|): the scale FP tolerances are relative to."""
    import oracle

    kw = dict(kw)
    if V.dtype.kind != "f":
        return None
    for key in ("init", "miss"):
        if isinstance(kw.get(key), np.ndarray):
            kw[key] = np.abs(kw[key])
    miss = kw.pop("miss", None)
    return oracle.matmul(og, np.abs(V), direction, miss=miss, **kw)


def assert_matches(got, ref, scale=None, rtol=None):
    """Integer/bool: bit-exact.  Float: |got-ref| <= rtol * scale (+ tiny)."""
    assert got.shape == ref.shape and got.dtype == ref.dtype, (got.shape, ref.shape, got.dtype, ref.dtype)
    if ref.dtype.kind != "f":
        mism = np.flatnonzero(got.ravel() != ref.ravel())
        assert mism.size == 0, f"{mism.size} mismatches, first at {mism[:5]}: {got.ravel()[mism[:5]]} vs {ref.ravel()[mism[:5]]}"
        return
    if rtol is None:
        rtol = 1e-12 if ref.dtype == np.float64 else 1e-6
    if scale is None:
        scale = np.abs(ref)
    err = np.abs(got.astype(np.float64) - ref.astype(np.float64))
    bound = rtol * scale.astype(np.float64) + 1e-300
    bad = np.flatnonzero(err.ravel() > bound.ravel())
    assert bad.size == 0, f"{bad.size} outputs beyond rtol={rtol}: max err/scale {np.max(err / np.maximum(scale, 1e-300))}"


def oracle_graph_of(g):
    """The oracle's view of a grgl_gb300 graph (its exported CSR arrays)."""
    import oracle

    a = g.export_arrays()
    return oracle.OracleGraph(num_samples=g.num_samples, ploidy=g.ploidy, down_off=a["down_off"],
                              down_adj=a["down_adj"], mut_node=a["mut_node"])


def assert_matches_oracle(og, V, direction, got, by_individual=False):
    """`got` against the oracle on the same input: integers bit-exact; float64 within 1e-12 and
    (compensated) float32 within 1e-6 of the sum of |terms| per output, float32 against the
    oracle's float64 product of the same inputs."""
    import oracle

    V = np.asarray(V)
    got = np.asarray(got)
    if V.dtype.kind != "f":
        assert_matches(got, oracle.matmul(og, V, direction, by_individual=by_individual))
        return
    V64 = V.astype(np.float64)
    ref = oracle.matmul(og, V64, direction, by_individual=by_individual)
    scale = oracle.matmul(og, np.abs(V64), direction, by_individual=by_individual)
    assert_matches(got.astype(np.float64), ref, scale, rtol=1e-6 if V.dtype == np.float32 else 1e-12)
