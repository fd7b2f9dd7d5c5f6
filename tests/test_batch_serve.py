"""Batched traversals and the serving loop: every request's result equals its own single
matmul (bit-exact for integers, float tolerances as elsewhere), alone and in the mix."""
import threading

import numpy as np
import pytest

from tests.conftest import assert_matches, assert_matches_oracle, oracle_graph_of

pytestmark = pytest.mark.gpu
DOWN, UP = 1, 2


@pytest.fixture(scope="module")
def gx(cuda_ok):
    import grgl_gb300

    return grgl_gb300


@pytest.fixture(scope="module")
def graphs(gx):
    return gx.window_tree_grg(2000, 20000, seed=31).upload(), gx.window_tree_grg(500, 3000, seed=32).upload()


@pytest.fixture(scope="module")
def oracles(graphs):
    return [oracle_graph_of(g) for g in graphs]


def _rand(rng, dtype, shape):
    if np.dtype(dtype).kind == "f":
        return rng.standard_normal(shape).astype(dtype)
    return rng.integers(-300, 300, size=shape).astype(dtype)


def _check_same(gx, g, V, d, got):
    ref = gx.matmul(g, V, d)
    if V.dtype.kind == "f":
        scale = np.abs(gx.matmul(g, np.abs(V).astype(np.float64), d))
        assert_matches(got.astype(np.float64), ref.astype(np.float64), scale,
                       rtol=1e-6 if V.dtype == np.float32 else 1e-12)
    else:
        assert_matches(got, ref)


def test_matmul_batch_matches_single(gx, graphs, oracles):
    g = graphs[0]
    rng = np.random.default_rng(0)
    reqs = []
    for i in range(24):
        d = UP if i % 2 else DOWN
        dt = [np.int32, np.float32, np.float64, np.int64][i % 4]
        K = [1, 3, 8, 20, 5, 64][i % 6]
        reqs.append((_rand(rng, dt, (K, g.num_samples if d == UP else g.num_mutations)), d))
    outs = gx.matmul_batch(g, reqs)
    for (V, d), out in zip(reqs, outs):
        _check_same(gx, g, V, d, out)
    # one request per dtype and direction against the oracle as well
    seen = set()
    for (V, d), out in zip(reqs, outs):
        if (V.dtype, d) not in seen:
            seen.add((V.dtype, d))
            assert_matches_oracle(oracles[0], V, d, out)
    # a tiny stacking width forces many traversals; device tensors take the device path
    import torch

    outs = gx.matmul_batch(g, [(torch.from_numpy(V).cuda(), d) for V, d in reqs], max_cols=9)
    torch.cuda.synchronize()
    for (V, d), out in zip(reqs, outs):
        _check_same(gx, g, V, d, out.cpu().numpy())


def test_matmul_batch_splits_rows_across_stacks(gx, graphs, oracles):
    """Requests whose rows are cut across stacks (narrow stacking widths), and a group whose last
    stack would end in a nearly empty column tile (136 four-byte rows: stacks of 128 and 8), give
    each request's own product."""
    g = graphs[0]
    rng = np.random.default_rng(4)
    reqs = [(_rand(rng, np.float32, (8, g.num_samples)), UP) for _ in range(17)]
    reqs += [(_rand(rng, np.int64, (3, g.num_mutations)), DOWN) for _ in range(5)]
    reqs += [(_rand(rng, np.int32, (70, g.num_mutations)), DOWN)]
    for width in (0, 5, 64):
        outs = gx.matmul_batch(g, reqs, max_cols=width)
        for (V, d), out in zip(reqs, outs):
            _check_same(gx, g, V, d, out)
    assert_matches_oracle(oracles[0], reqs[0][0], UP, outs[0])
    assert_matches_oracle(oracles[0], reqs[-1][0], DOWN, outs[-1])


def test_server_results_alone_and_in_the_mix(gx, graphs, oracles):
    rng = np.random.default_rng(1)
    reqs = []
    for i in range(40):
        gid = i % 2
        g = graphs[gid]
        d = UP if (i // 2) % 2 else DOWN
        dt = [np.int32, np.float32, np.float64][i % 3]
        K = int(rng.integers(1, 40))
        reqs.append((gid, _rand(rng, dt, (K, g.num_samples if d == UP else g.num_mutations)), d))
    with gx.Server(workers=3) as srv:
        ids = [srv.add_graph(g) for g in graphs]
        # alone: one at a time
        for gid, V, d in reqs[:6]:
            out, st = srv.result(srv.submit(ids[gid], V, d), timeout=60)
            assert st["batch_requests"] == 1
            _check_same(gx, graphs[gid], V, d, out)
        # in the mix: submitted from 4 threads at once
        tickets = [None] * len(reqs)

        def submit(lo):
            for i in range(lo, len(reqs), 4):
                gid, V, d = reqs[i]
                tickets[i] = srv.submit(ids[gid], V, d)

        th = [threading.Thread(target=submit, args=(k,)) for k in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        batched = 0
        seen = set()
        for i, (gid, V, d) in enumerate(reqs):
            out, st = srv.result(tickets[i], timeout=120)
            batched += st["batch_requests"] > 1
            assert st["done_s"] >= st["start_s"] >= st["submit_s"]
            _check_same(gx, graphs[gid], V, d, out)
            if (gid, V.dtype) not in seen:  # one served result per graph and dtype vs the oracle
                seen.add((gid, V.dtype))
                assert_matches_oracle(oracles[gid], V, d, out)
        assert batched > 0  # queued requests were coalesced


def test_server_memory_admission(gx, graphs):
    g = graphs[1]
    small = np.ones((1, g.num_samples), dtype=np.int32)
    budget = 2 * 1024 * 1024  # room for narrow requests only
    with gx.Server(workers=2, memory_budget=budget) as srv:
        gid = srv.add_graph(g)
        huge = np.ones((4000, g.num_samples), dtype=np.int32)
        t_big = srv.submit(gid, huge, UP)
        ts = [srv.submit(gid, small, UP) for _ in range(5)]
        with pytest.raises((MemoryError, RuntimeError), match="memory budget"):
            srv.result(t_big, timeout=60)
        for t in ts:
            out, _ = srv.result(t, timeout=60)
            assert np.array_equal(out, gx.matmul(g, small, UP))


def test_by_individual_requests_batched_and_served(gx, graphs):
    """Requests folded by individual share traversals with each other (never with per-haplotype
    ones) and equal matmul(..., by_individual=True)."""
    g = graphs[0]
    rng = np.random.default_rng(12)
    reqs = []
    for i in range(10):
        d = UP if i % 2 else DOWN
        byi = i % 3 != 0
        dt = [np.int32, np.float64][i % 2]
        cols = (g.num_individuals if byi else g.num_samples) if d == UP else g.num_mutations
        reqs.append((_rand(rng, dt, (int(rng.integers(1, 7)), cols)), d, False, byi))
    outs = gx.matmul_batch(g, reqs)
    for (V, d, _, byi), out in zip(reqs, outs):
        ref = gx.matmul(g, V, d, by_individual=byi)
        if V.dtype.kind == "f":
            scale = np.abs(gx.matmul(g, np.abs(V), d, by_individual=byi))
            assert_matches(out, ref, scale, rtol=1e-12)
        else:
            assert_matches(out, ref)
    with gx.Server(workers=2) as srv:
        gid = srv.add_graph(g)
        ts = [srv.submit(gid, V, d, by_individual=byi) for V, d, _, byi in reqs]
        for (V, d, _, byi), t in zip(reqs, ts):
            out, _ = srv.result(t, timeout=120)
            if V.dtype.kind != "f":
                assert np.array_equal(out, gx.matmul(g, V, d, by_individual=byi))
    with pytest.raises(RuntimeError, match="per haplotype"):
        gx.matmul_batch(g, [(np.ones((1, g.num_samples), dtype=np.float32), UP, True, True)])
