"""Host-side tests of libgrgx (no GPU): the C ABI exports, the .grg loader, argument validation
with the reference's messages, and the synthetic window-tree generator."""
import ctypes
import re

import numpy as np
import pytest

import oracle
from tests.conftest import GOLDEN, ROOT, kat_graph_arrays

DOWN, UP = 1, 2


@pytest.fixture(scope="module")
def gx(lib_built):
    import grgl_gb300

    return grgl_gb300


def test_exports_every_declared_symbol(lib_built):
    from grgl_gb300 import _lib

    header = (ROOT / "include" / "grgx.h").read_text()
    declared = set(re.findall(r"\b(grgx_[a-z0-9_]+)\s*\(", header))
    assert declared, "no declarations found"
    handle = ctypes.CDLL(str(_lib.LIB_PATH))
    missing = [s for s in sorted(declared) if not hasattr(handle, s)]
    assert not missing, missing
    assert declared == set(_lib.SIGNATURES), declared ^ set(_lib.SIGNATURES)


@pytest.mark.parametrize("fixture", ["t200", "t200miss", "wt_n1000_m10000"])
def test_loader_matches_independent_reader(gx, fixture):
    g = gx.load_immutable_grg(str(GOLDEN / f"{fixture}.grg"))
    o = oracle.read_grg(GOLDEN / f"{fixture}.grg")
    a = g.export_arrays()
    assert g.num_nodes == o.num_nodes and g.num_edges == o.num_edges
    assert g.num_samples == o.num_samples and g.num_mutations == o.num_mutations and g.ploidy == o.ploidy
    for key in ("down_off", "down_adj", "mut_node", "coals"):
        assert np.array_equal(a[key], getattr(o, key)), key
    if o.miss_node is not None:
        assert g.has_missing_data and np.array_equal(a["miss_node"], o.miss_node)


def test_loader_rejects_bad_files(gx, tmp_path, capsys):
    bad = tmp_path / "bad.grg"
    bad.write_bytes(b"\0" * 200)
    assert gx.load_immutable_grg(str(bad)) is None
    assert "Invalid file header" in capsys.readouterr().err
    assert gx.load_immutable_grg(str(tmp_path / "missing.grg")) is None
    trunc = tmp_path / "trunc.grg"
    trunc.write_bytes((GOLDEN / "t200.grg").read_bytes()[:5000])
    assert gx.load_immutable_grg(str(trunc)) is None
    assert "Malformed GRG file" in capsys.readouterr().err


def test_validation_messages_match_reference(gx):
    """Misuse is reported before any device work, with the reference's messages
    (internal_mult.h:130-158, _grgl.cpp:100-241)."""
    g = gx.from_csr(**kat_graph_arrays((1, 5, 6)))
    cases = [
        (lambda: gx.matmul(g, np.zeros((1, 4)), DOWN), "Input vector is not size M (numMutations)"),
        (lambda: gx.matmul(g, np.zeros((1, 3)), UP),
         "Input vector is not size N (numSamples, or numIndividuals depending on flags)"),
        (lambda: gx.matmul(g, np.zeros((1, 4)), UP, by_individual=True),
         "Input vector is not size N (numSamples, or numIndividuals depending on flags)"),
        (lambda: gx.matmul(g, np.zeros(4), UP), "matmul() only support two dimensional numpy arrays as input."),
        (lambda: gx.matmul(g, np.zeros((0, 4)), UP), "matmul() requires non-zero dimensions."),
        (lambda: gx.matmul(g, [[1.0, 2.0, 3.0, 4.0]], UP), "Unsupported numpy dtype: float64"),
        (lambda: gx.matmul(g, np.zeros((1, 4), dtype=np.float16), UP), "Unsupported numpy dtype: float16"),
        (lambda: gx.matmul(g, np.zeros((1, 4)), UP, init="abc"), "Unexpected init value: abc"),
        (lambda: gx.matmul(g, np.zeros((1, 4)), UP, init=np.zeros(1, dtype=np.float32)),
         "The init matrix must match the dtype of the input matrix. Got: float32"),
        (lambda: gx.matmul(g, np.zeros((2, 4)), UP, init=np.zeros(3)),
         "If init has a single dimension, it must match the number of rows in the input matrix"),
        (lambda: gx.matmul(g, np.zeros((2, 4)), UP, init=np.zeros((2, 3))),
         "If init is a matrix, it must match the dimensions ROW x NODES"),
        (lambda: gx.matmul(g, np.zeros((1, 4), dtype=bool), UP, init="xtx"),
         "init=... is not supported with boolean dtype"),
        (lambda: gx.matmul(g, np.zeros((1, 4)), UP, init="xtx"),
         "Coalescent counts not available for this GRG (init=XTX won't work)"),
        (lambda: gx.matmul(g, np.zeros((1, 4)), UP, emit_all_nodes=True, miss=np.zeros((1, 7))),
         'The "miss" parameter cannot be mixed with the "emit_all_nodes" parameter'),
        (lambda: gx.matmul(g, np.zeros((1, 4)), UP, miss=np.zeros((1, 3), dtype=np.int32)),
         'The "miss" input must be a matrix with dtype matching the input matrix. Got: int32'),
        (lambda: gx.matmul(g, np.zeros((1, 4)), UP, miss=np.zeros(3)),
         '"miss" must be a two-dimension numpy array (matrix). ndim=1'),
        (lambda: gx.matmul(g, np.zeros((1, 4)), UP, miss=np.zeros((2, 3))),
         '"miss" has 2 rows, but must match the input and output matrices (1)'),
        (lambda: gx.matmul(g, np.zeros((1, 3)), DOWN, miss=np.zeros((1, 4))),
         'The "miss" matrix must match the number of columns in the input matrix. Got: 4'),
        (lambda: gx.matmul(g, np.zeros((1, 4)), UP, miss=np.zeros((1, 4))),
         'The "miss" matrix must match the number of columns in the output matrix. Got: 4'),
        (lambda: gx.dot_product(g, np.zeros((1, 4)), UP),
         "dot_product() only support one-dimensional numpy arrays as input."),
        (lambda: gx.dot_product(g, np.zeros(0), UP), "dot_product() requires non-empty array input."),
        (lambda: gx.dot_product(g, np.zeros(4, dtype=np.int8), UP), "Unsupported numpy dtype: int8"),
    ]
    for fn, msg in cases:
        with pytest.raises(RuntimeError) as ei:
            fn()
        assert str(ei.value) == msg


def test_from_csr_rejects_malformed(gx):
    a = kat_graph_arrays()
    bad = dict(a, down_adj=np.array([0, 1, 2, 3, 4, 9], dtype=np.uint32))
    with pytest.raises(RuntimeError, match="edge target out of range"):
        gx.from_csr(**bad)
    bad = dict(a, mut_node=np.array([1, 99], dtype=np.uint32))
    with pytest.raises(RuntimeError, match="mutation node out of range"):
        gx.from_csr(**bad)


def test_window_tree_generator_deterministic(gx):
    a = gx.window_tree_grg(500, 2000, seed=7).export_arrays()
    b = gx.window_tree_grg(500, 2000, seed=7, threads=1).export_arrays()
    c = gx.window_tree_grg(500, 2000, seed=8).export_arrays()
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert not np.array_equal(a["down_adj"], c["down_adj"])


def test_window_tree_generator_structure(gx):
    N, M = 400, 1000
    g = gx.window_tree_grg(N, M, seed=42)
    a = g.export_arrays()
    off, adj, mut = a["down_off"], a["down_adj"], a["mut_node"]
    n = g.num_nodes
    # topologically ordered, sorted child lists, every mutation mapped
    for v in range(n):
        ch = adj[off[v]:off[v + 1]]
        assert np.all(ch < v) and np.all(np.diff(ch.astype(np.int64)) > 0)
    assert np.all(mut != oracle.INVALID_NODE)
    og = oracle.OracleGraph(num_samples=N, ploidy=2, down_off=off, down_adj=adj, mut_node=mut)
    X = og.dense_X()
    assert X.max() == 1  # trees: every sample is below a mutation node at most once
    freq = X.sum(axis=0)
    assert freq.min() >= 1 and freq.max() <= N - 1
    # ~1/f spectrum: singletons are the most common class
    hist = np.bincount(freq)
    assert hist[1] == hist[1:].max()


def test_window_tree_equals_reference_construction(gx):
    """The directly emitted graph and the reference constructor's graph for the same genotypes
    (tests/golden/wt_n1000_m10000.grg, built from the generator's VCF) give identical integer products."""
    direct = gx.window_tree_grg(1000, 10000, seed=42).export_arrays()
    og = oracle.OracleGraph(num_samples=1000, ploidy=2, down_off=direct["down_off"], down_adj=direct["down_adj"],
                            mut_node=direct["mut_node"])
    ref = oracle.read_grg(GOLDEN / "wt_n1000_m10000.grg")
    rng = np.random.default_rng(11)
    for direction, cols in ((UP, 1000), (DOWN, 10000)):
        V = rng.integers(-1000, 1000, size=(2, cols)).astype(np.int64)
        assert np.array_equal(oracle.matmul(og, V, direction), oracle.matmul(ref, V, direction))


def test_loader_keeps_buckets_encoded_until_needed(gx, tmp_path):
    """A loaded graph reports its sizes from the header; a corrupt bucket surfaces, with the
    loader's message, when the edges are first decoded (here on the host, by an export)."""
    raw = bytearray((GOLDEN / "t200.grg").read_bytes())
    g = gx.load_immutable_grg(str(GOLDEN / "t200.grg"))
    o = oracle.read_grg(GOLDEN / "t200.grg")
    assert g.num_edges == o.num_edges and g.num_nodes == o.num_nodes
    raw[136:142] = b"\xff" * 6  # the first bucket's count: a varint longer than five bytes
    bad = tmp_path / "badbucket.grg"
    bad.write_bytes(bytes(raw))
    gb = gx.load_immutable_grg(str(bad))
    assert gb is not None and gb.num_edges == o.num_edges
    with pytest.raises(RuntimeError, match="Malformed GRG file"):
        gb.export_arrays()


def test_save_round_trip(gx, tmp_path):
    """A saved graph reads back with the same arrays (and, where the reference build exists in
    this checkout, the reference reads it to the same products as the oracle)."""
    g = gx.window_tree_grg(600, 5000, seed=13)
    path = tmp_path / "wt.grg"
    g.save(str(path))
    back = gx.load_immutable_grg(str(path))
    a, b = g.export_arrays(), back.export_arrays()
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    o = oracle.read_grg(path)
    assert np.array_equal(o.down_adj, a["down_adj"]) and np.array_equal(o.mut_node, a["mut_node"])
    bad = gx.from_csr(num_samples=2, ploidy=2, down_off=np.array([0, 0, 0, 2], dtype=np.uint64),
                      down_adj=np.array([1, 0], dtype=np.uint32), mut_node=np.array([2], dtype=np.uint32))
    with pytest.raises(RuntimeError, match="ascending"):
        bad.save(str(tmp_path / "bad.grg"))


def test_saved_file_reads_in_the_reference(gx, tmp_path):
    import sys

    ref = ROOT / "oracle" / "_ref"
    if not (ref / "pygrgl").is_dir():
        pytest.skip("reference build not present (oracle/build_ref.sh)")
    sys.path[:0] = [str(ref)]
    try:
        pygrgl = pytest.importorskip("pygrgl")
    finally:
        del sys.path[:1]
    g = gx.window_tree_grg(500, 3000, seed=5)
    path = str(tmp_path / "wt.grg")
    g.save(path)
    r = pygrgl.load_immutable_grg(path)
    a = g.export_arrays()
    og = oracle.OracleGraph(num_samples=500, ploidy=2, down_off=a["down_off"], down_adj=a["down_adj"],
                            mut_node=a["mut_node"])
    rng = np.random.default_rng(0)
    V, W = rng.standard_normal((3, 500)), rng.standard_normal((2, 3000))
    assert np.array_equal(pygrgl.matmul(r, V, pygrgl.TraversalDirection.UP), oracle.matmul(og, V, UP))
    assert np.array_equal(pygrgl.matmul(r, W, pygrgl.TraversalDirection.DOWN), oracle.matmul(og, W, DOWN))


def test_header_is_plain_c(tmp_path):
    """include/grgx.h is a C header (C99, no C++ or CUDA types): a C program that includes it
    and names every entry point compiles."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    header = (ROOT / "include" / "grgx.h").read_text()
    names = sorted(set(re.findall(r"\b(grgx_[a-z0-9_]+)\s*\(", header)))
    src = tmp_path / "abi.c"
    src.write_text('#include "grgx.h"\ntypedef void (*entry)(void);\nentry table[] = {' +
                   ", ".join(f"(entry){n}" for n in names) + "};\n")
    res = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-pedantic", "-fsyntax-only",
                          f"-I{ROOT / 'include'}", str(src)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr


def test_c_program_links_and_runs(lib_built, tmp_path):
    """A C program linked against libgrgx.so alone (no Python) loads a reference-written .grg,
    reads its sizes, writes it back, reloads the copy, subsets it and reports a bad path with
    a status and a message -- the host side of the boundary a C or C++ caller drives."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = ROOT / "grgl_gb300" / "libgrgx.so"
    src = tmp_path / "host_abi.c"
    src.write_text(r'''
#include <stdio.h>
#include <string.h>
#include "grgx.h"
#define CHECK(x) do { if ((x) != GRGX_OK) { fprintf(stderr, "%s: %s\n", #x, grgx_last_error()); return 1; } } while (0)
int main(int argc, char** argv) {
    grgx_graph *g = NULL, *h = NULL, *s = NULL;
    grgx_graph_info a, b, c;
    CHECK(grgx_graph_load(argv[1], &g));
    CHECK(grgx_graph_info_get(g, &a));
    CHECK(grgx_graph_save(g, argv[2]));
    CHECK(grgx_graph_load(argv[2], &h));
    CHECK(grgx_graph_info_get(h, &b));
    if (a.num_nodes != b.num_nodes || a.num_edges != b.num_edges || a.num_samples != b.num_samples ||
        a.num_mutations != b.num_mutations || a.ploidy != b.ploidy) return 2;
    const uint32_t muts[3] = {0, 1, 2};
    CHECK(grgx_graph_subset(g, muts, 3, &s));
    CHECK(grgx_graph_info_get(s, &c));
    if (c.num_mutations != 3 || c.num_samples != a.num_samples) return 3;
    grgx_graph* bad = NULL;
    if (grgx_graph_load(argv[3], &bad) == GRGX_OK || strlen(grgx_last_error()) == 0) return 4;
    printf("%llu %llu %llu %llu\n", (unsigned long long)a.num_nodes, (unsigned long long)a.num_edges,
           (unsigned long long)a.num_samples, (unsigned long long)a.num_mutations);
    grgx_graph_destroy(s);
    grgx_graph_destroy(h);
    grgx_graph_destroy(g);
    return 0;
}
''')
    exe = tmp_path / "host_abi"
    res = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(src), "-o", str(exe),
                          str(lib), f"-Wl,-rpath,{lib.parent}"], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    run = subprocess.run([str(exe), str(GOLDEN / "t200.grg"), str(tmp_path / "copy.grg"),
                          str(tmp_path / "missing.grg")], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, (run.returncode, run.stderr)
    og = oracle.read_grg(GOLDEN / "t200.grg")
    assert run.stdout.split() == [str(og.num_nodes), str(og.num_edges), str(og.num_samples), str(og.num_mutations)]
