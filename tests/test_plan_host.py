"""The level plan laid out on the host (plan.cpp), checked on the CPU against a restatement of
what the sweep needs from it: heights and the height-major renumbering, the UP rows and their
children, the DOWN rows and their parent counts, the seed rows, and chunks that cover every
edge of a level exactly once (whole rows, or the pieces of one heavy row).  The device builder
shares the row and chunk stages and is compared with this builder product by product on the
GPU (test_plan_device.py)."""
import ctypes

import numpy as np
import pytest

from tests.conftest import GOLDEN

HEAD = np.uint32(0x80000000)
INVALID = 0x7FFFFFFF
CHUNK = np.dtype([("e0", "<i8"), ("r0", "<i4"), ("heavy", "<i4")])
HEAVY = np.dtype([("first_chunk", "<i4"), ("n_pieces", "<i4"), ("slot_base", "<i8")])
TYPES = {"level_begin": np.uint64, "old2new": np.uint32, "new2old": np.uint32, "mut_new": np.uint32,
         "miss_new": np.uint32, "down_row_of": np.int32, "rows": np.int32, "off": np.int64, "adj": np.uint32,
         "chunks": CHUNK, "heavy": HEAVY, "level_chunk_begin": np.int32, "level_chunk_end": np.int32}


def plan_array(g, name):
    from grgl_gb300 import _lib

    fn = _lib.lib().grgx_debug_host_plan
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p),
                   ctypes.POINTER(ctypes.c_uint64)]
    data, nbytes = ctypes.c_void_p(), ctypes.c_uint64()
    _lib.check(fn(g._h, name.encode(), ctypes.byref(data), ctypes.byref(nbytes)))
    dt = np.dtype(TYPES[name.split(".")[-1]])
    if nbytes.value == 0:
        return np.zeros(0, dtype=dt)
    buf = (ctypes.c_char * nbytes.value).from_address(data.value)
    return np.frombuffer(bytes(buf), dtype=dt)


def heights(n, off, adj):
    """Height of every node (0 without children, else 1 + the children's maximum)."""
    h = np.zeros(n, dtype=np.int64)
    src = np.repeat(np.arange(n), np.diff(off).astype(np.int64))
    for _ in range(n + 1):
        nh = np.zeros(n, dtype=np.int64)
        np.maximum.at(nh, src, h[adj.astype(np.int64)] + 1)
        if np.array_equal(nh, h):
            return h
        h = nh
    raise AssertionError("heights did not settle")


def check_chunks(csr, off, level_rows):
    """Chunks of each level cover its edges once: whole rows, or consecutive pieces of one row."""
    chunks, heavy = csr["chunks"], csr["heavy"]
    lb, le = csr["level_chunk_begin"], csr["level_chunk_end"]
    E, R = int(off[-1]), len(off) - 1
    assert chunks[-1]["e0"] == E and chunks[-1]["r0"] == R and chunks[-1]["heavy"] == -1
    assert np.all(np.diff(chunks["e0"]) >= 0)
    assert len(lb) == len(le) == len(level_rows)
    pos = 0
    for (b, e), (rb, re) in zip(zip(lb, le), level_rows):
        assert b == pos and e >= b
        pos = e
        if re == rb:
            continue
        # the level's edge span, from its first to its last row
        assert chunks[b]["e0"] == off[rb] and chunks[e]["e0"] == off[re]
        for c in range(b, e):
            ch, nxt = chunks[c], chunks[c + 1]
            r0 = int(ch["r0"])
            assert rb <= r0 < re
            if ch["heavy"] < 0:
                assert ch["e0"] == off[r0]  # whole rows: starts on a row boundary
                assert nxt["e0"] > ch["e0"] or off[r0 + 1] == off[r0]
            else:
                hr = heavy[ch["heavy"]]
                piece = c - int(hr["first_chunk"])
                assert 0 <= piece < hr["n_pieces"] and off[r0] <= ch["e0"] < off[r0 + 1]
                assert (piece == 0) == (ch["e0"] == off[r0])
                if piece == hr["n_pieces"] - 1:
                    assert nxt["e0"] == off[r0 + 1]
                else:
                    assert nxt["r0"] == r0 and nxt["heavy"] == ch["heavy"] and nxt["e0"] > ch["e0"]
    assert pos == len(chunks) - 1
    assert np.array_equal(heavy["slot_base"], np.concatenate([[0], np.cumsum(heavy["n_pieces"])[:-1]])
                          if len(heavy) else heavy["slot_base"])


def check_fine(fine, coarse, off, level_rows):
    """The finer chunking of the same rows: the same levels, every edge once, and at least as many
    chunks per level as the coarse chunking."""
    check_chunks(fine, off, level_rows)
    for l, (rb, re) in enumerate(level_rows):
        nc = coarse["level_chunk_end"][l] - coarse["level_chunk_begin"][l]
        nf = fine["level_chunk_end"][l] - fine["level_chunk_begin"][l]
        assert nf >= nc
    assert len(fine["chunks"]) >= len(coarse["chunks"])


def check_plan(g):
    a = g.export_arrays()
    n, N = g.num_nodes, g.num_samples
    off, adj = a["down_off"].astype(np.int64), a["down_adj"]
    h = heights(n, off, adj)
    L = int(h.max()) + 1 if n else 0
    P = {k: plan_array(g, k) for k in ("level_begin", "old2new", "new2old", "mut_new", "miss_new", "down_row_of")}
    for c in ("up", "down", "seed", "miss"):
        P[c] = {f: plan_array(g, f"{c}.{f}") for f in ("rows", "off", "adj", "chunks", "heavy",
                                                       "level_chunk_begin", "level_chunk_end")}
    for c in ("up_fine", "down_fine"):
        P[c] = {f: plan_array(g, f"{c}.{f}") for f in ("chunks", "heavy", "level_chunk_begin", "level_chunk_end")}
    lb = P["level_begin"].astype(np.int64)
    assert len(lb) == L + 1 and np.array_equal(np.diff(lb), np.bincount(h, minlength=L))
    o2n, n2o = P["old2new"].astype(np.int64), P["new2old"].astype(np.int64)
    assert np.array_equal(n2o[o2n], np.arange(n))
    # height-major, the original order kept inside a height (samples stay 0..N-1)
    order = np.lexsort((np.arange(n), h))
    assert np.array_equal(o2n[order], np.arange(n))
    assert np.all(h[:N] == 0) and np.array_equal(o2n[:N], np.arange(N))

    # UP: every node of height >= 1, ascending new id; its children (as new ids) in the graph's
    # own edge order, the order the reference adds them in (grg.h:1324-1334)
    up = P["up"]
    r0 = lb[1] if L > 1 else n
    assert np.array_equal(up["rows"], np.arange(r0, n))
    deg = np.diff(off)[n2o[r0:]]
    assert np.array_equal(np.diff(up["off"]), deg) and up["off"][0] == 0
    ua = up["adj"]
    heads = np.flatnonzero(ua & HEAD)
    assert np.array_equal(heads, up["off"][:-1][deg > 0])
    kids = (ua & ~HEAD).astype(np.int64)
    for i in range(len(up["rows"])):
        s, e = up["off"][i], up["off"][i + 1]
        old = n2o[up["rows"][i]]
        assert np.array_equal(kids[s:e], o2n[adj[off[old]:off[old + 1]].astype(np.int64)])
    check_chunks(up, up["off"], [(lb[k] - r0, lb[k + 1] - r0) for k in range(1, L)])
    check_fine(P["up_fine"], up, up["off"], [(lb[k] - r0, lb[k + 1] - r0) for k in range(1, L)])

    # DOWN: nodes with parents, heights descending, ids ascending inside a height
    dn = P["down"]
    pdeg_new = np.bincount(o2n[adj.astype(np.int64)], minlength=n)
    want = np.concatenate([np.arange(lb[k], lb[k + 1])[pdeg_new[lb[k]:lb[k + 1]] > 0] for k in range(L - 1, -1, -1)]) \
        if L else np.zeros(0, np.int64)
    assert np.array_equal(dn["rows"], want)
    assert np.array_equal(np.diff(dn["off"]), pdeg_new[want])
    row_of = np.full(n, -1)
    row_of[want] = np.arange(len(want))
    assert np.array_equal(P["down_row_of"], row_of)
    levels, pos = [], 0
    for k in range(L - 1, -1, -1):
        cnt = int(np.count_nonzero(pdeg_new[lb[k]:lb[k + 1]]))
        levels.append((pos, pos + cnt))
        pos += cnt
    check_chunks(dn, dn["off"], levels)
    check_fine(P["down_fine"], dn, dn["off"], levels)

    # seeds: mutation -> new node, rows = mapped nodes ascending, mutation ids ascending per row
    mut = a["mut_node"].astype(np.int64)
    mapped = mut != INVALID
    assert np.array_equal(P["mut_new"][mapped], o2n[mut[mapped]]) and np.all(P["mut_new"][~mapped] == INVALID)
    sd = P["seed"]
    sa = sd["adj"]
    starts = np.flatnonzero(sa & HEAD)
    soff = np.append(starts, len(sa))
    assert np.array_equal(sd["rows"], np.unique(o2n[mut[mapped]]))
    for i, node in enumerate(sd["rows"]):
        ms = (sa[soff[i]:soff[i + 1]] & ~HEAD).astype(np.int64)
        assert np.array_equal(ms, np.flatnonzero(P["mut_new"] == node))
    return P


@pytest.mark.parametrize("fixture", ["t200", "t200miss", "wt_n1000_m10000"])
def test_host_plan_of_reference_graphs(lib_built, fixture):
    import grgl_gb300 as gx

    P = check_plan(gx.load_immutable_grg(str(GOLDEN / f"{fixture}.grg")))
    if fixture == "t200miss":
        assert len(P["miss"]["rows"]) > 0


def test_host_plan_heavy_rows(lib_built):
    """Rows far longer than a level's chunk size are cut into pieces with partial slots."""
    import grgl_gb300 as gx

    N = 50_000
    children = [np.arange(N), np.arange(0, N, 2), np.array([N, N + 1] + list(range(5)))]
    off = np.concatenate([np.zeros(N + 1, np.uint64), np.cumsum([len(c) for c in children]).astype(np.uint64)])
    adj = np.concatenate(children).astype(np.uint32)
    g = gx.from_csr(num_samples=N, ploidy=2, down_off=off, down_adj=adj,
                    mut_node=np.array([N, N + 1, N + 2, N + 2, INVALID], dtype=np.uint32))
    P = check_plan(g)
    assert len(P["up"]["heavy"]) >= 2 and P["up"]["heavy"]["n_pieces"].min() > 1


def test_host_plan_of_window_tree(lib_built):
    import grgl_gb300 as gx

    check_plan(gx.window_tree_grg(3000, 20000, seed=13))


def test_host_plan_fine_chunks(lib_built):
    """A level with millions of edges: the fine chunking cuts it into several times the coarse
    chunking's chunks (heavy rows into more pieces), and both cover every edge once."""
    import grgl_gb300 as gx

    N, rows, deg = 40_000, 100, 40_000
    rng = np.random.default_rng(4)
    children = [np.sort(rng.choice(N, size=deg, replace=False)) for _ in range(rows)]
    off = np.concatenate([np.zeros(N + 1, np.uint64), np.cumsum([len(c) for c in children]).astype(np.uint64)])
    adj = np.concatenate(children).astype(np.uint32)
    g = gx.from_csr(num_samples=N, ploidy=2, down_off=off, down_adj=adj,
                    mut_node=np.arange(N, N + rows, dtype=np.uint32))
    up = {f: plan_array(g, f"up.{f}") for f in ("rows", "off", "chunks", "heavy", "level_chunk_begin",
                                                 "level_chunk_end")}
    fine = {f: plan_array(g, f"up_fine.{f}") for f in ("chunks", "heavy", "level_chunk_begin", "level_chunk_end")}
    levels = [(0, rows)]
    check_chunks(up, up["off"], levels)
    check_fine(fine, up, up["off"], levels)
    assert len(fine["chunks"]) > 2 * len(up["chunks"])
    assert fine["heavy"]["n_pieces"].sum() > 2 * up["heavy"]["n_pieces"].sum()
