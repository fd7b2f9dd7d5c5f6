"""Launch-shape autotuner: the table's text round trip (host only), and on the GPU that tuning
records one entry per level and that every shape it may choose gives the oracle's results
(bit-exact for integers, the float tolerances otherwise)."""
import numpy as np
import pytest

import oracle

DOWN, UP = 1, 2


@pytest.fixture()
def gx(lib_built):
    import grgl_gb300

    grgl_gb300.autotune_clear()
    yield grgl_gb300
    grgl_gb300.autotune_clear()


def test_table_text_round_trip(gx):
    text = "3 64 17 11 4 4 1\n0 1 12 3 1 1 0\n"
    gx.autotune_load(text)
    got = gx.autotune_table()
    assert sorted(got.strip().splitlines()) == sorted(text.strip().splitlines())
    gx.autotune_clear()
    assert gx.autotune_table() == ""
    with pytest.raises(RuntimeError, match="malformed autotune table line"):
        gx.autotune_load("3 64 17\n")
    with pytest.raises(RuntimeError, match="invalid autotune table entry"):
        gx.autotune_load("3 64 17 11 3 4 1\n")  # G must be a power of two


def _oracle_graph(g):
    a = g.export_arrays()
    return oracle.OracleGraph(num_samples=g.num_samples, ploidy=2, down_off=a["down_off"], down_adj=a["down_adj"],
                              mut_node=a["mut_node"])


@pytest.mark.gpu
def test_autotune_records_levels_and_results_hold(gx, cuda_ok):
    g = gx.window_tree_grg(3000, 12000, seed=61)
    og = _oracle_graph(g)
    rng = np.random.default_rng(0)
    cases = [(np.int32, 64, UP), (np.int32, 8, DOWN), (np.float32, 32, UP), (np.float64, 64, DOWN)]
    for dt, K, d in cases:
        report = gx.autotune(g, dt, K, d)
        assert "sweep" in report and "level" in report
    table = gx.autotune_table().strip().splitlines()
    assert table
    # every entry the tuner may pick, forced on every level: G halved twice and the deep variant
    forced = []
    for line in table:
        kind, stride, rl, dl, g_, t_, v_ = (int(x) for x in line.split())
        forced.append((kind, stride, rl, dl))
    for shrink, variant in ((1, 1), (2, 0), (4, 1)):
        gx.autotune_clear()
        lines = []
        for kind, stride, rl, dl in forced:
            vw = 4 if kind in (0, 3, 4, 5) else 2  # 4-byte kinds: 4 per vector; 8-byte: 2
            vecs = max(1, stride // vw)
            g0 = min(32, 1 << (vecs - 1).bit_length())
            gg = max(1, g0 // shrink)
            lines.append(f"{kind} {stride} {rl} {dl} {gg} {-(-vecs // gg)} {variant}")
        gx.autotune_load("\n".join(lines) + "\n")
        for dt, K, d in cases:
            cols = g.num_samples if d == UP else g.num_mutations
            if np.dtype(dt).kind == "f":
                V = rng.standard_normal((K, cols)).astype(dt)
            else:
                V = rng.integers(-50, 50, size=(K, cols)).astype(dt)
            got = gx.matmul(g, V, d)
            if np.dtype(dt).kind == "f":
                ref = oracle.matmul(og, V.astype(np.float64), d)
                scale = oracle.matmul(og, np.abs(V).astype(np.float64), d)
                rtol = 1e-6 if dt == np.float32 else 1e-12
                assert np.all(np.abs(got - ref) <= rtol * scale + 1e-300), (dt, K, d, shrink, variant)
            else:
                assert np.array_equal(got, oracle.matmul(og, V, d)), (dt, K, d, shrink, variant)
