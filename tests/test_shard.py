"""Range sharding (CPU): graph subsets by mutation range reproduce the full product (UP
column blocks concatenate, DOWN partials add), and the multi-rank combine works over gloo with
the oracle as the per-shard product.  The GPU variant (co-resident shards) is marked gpu."""
import os
import socket

import numpy as np
import pytest

import oracle

DOWN, UP = 1, 2


def _og(g):
    a = g.export_arrays()
    miss = a["miss_node"] if g.has_missing_data else None
    return oracle.OracleGraph(num_samples=g.num_samples, ploidy=g.ploidy, down_off=a["down_off"],
                              down_adj=a["down_adj"], mut_node=a["mut_node"], miss_node=miss, coals=a["coals"])


def _oracle_fn(shard, V, direction):
    return oracle.matmul(_og(shard), V, int(direction))


@pytest.fixture(scope="module")
def graph(lib_built):
    import grgl_gb300 as gx

    return gx.window_tree_grg(800, 5000, seed=17)


def test_subsets_reproduce_full_product(graph):
    from grgl_gb300 import shard

    full = _og(graph)
    ranges, shards = shard.split_by_mutations(graph, 5)
    assert ranges[0].start == 0 and ranges[-1].stop == graph.num_mutations
    assert all(a.stop == b.start for a, b in zip(ranges, ranges[1:]))
    rng = np.random.default_rng(0)
    Vu = rng.integers(-50, 50, size=(3, graph.num_samples)).astype(np.int64)
    Vd = rng.integers(-50, 50, size=(3, graph.num_mutations)).astype(np.int64)
    up = np.concatenate([_oracle_fn(s, Vu, UP) for s in shards], axis=1)
    assert np.array_equal(up, oracle.matmul(full, Vu, UP))
    down = sum(_oracle_fn(s, np.ascontiguousarray(Vd[:, r.start:r.stop]), DOWN) for r, s in zip(ranges, shards))
    assert np.array_equal(down, oracle.matmul(full, Vd, DOWN))
    # shards stay small: window-tree ranges share only the samples and the windows cut at a boundary
    inner = sum(s.num_nodes - s.num_samples for s in shards)
    assert graph.num_nodes - graph.num_samples <= inner < 1.1 * (graph.num_nodes - graph.num_samples)


def test_subset_of_reference_graph_with_missingness(lib_built):
    import grgl_gb300 as gx
    from tests.conftest import GOLDEN

    g = gx.load_immutable_grg(str(GOLDEN / "t200miss.grg"))
    ids = np.arange(100, 900, dtype=np.uint32)
    sub = g.subset_mutations(ids)
    assert sub.num_mutations == 800 and sub.has_missing_data
    V = np.random.default_rng(1).integers(-5, 5, size=(2, g.num_samples)).astype(np.int32)
    assert np.array_equal(oracle.matmul(_og(sub), V, UP), oracle.matmul(_og(g), V, UP)[:, 100:900])


def test_subset_rejects_bad_ids(graph):
    with pytest.raises(RuntimeError, match="Invalid MutationID"):
        graph.subset_mutations([graph.num_mutations])


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, result_dir):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import grgl_gb300 as gx
    from grgl_gb300 import shard

    g = gx.window_tree_grg(600, 3000, seed=23)
    ranges, shards = shard.split_by_mutations(g, 4)
    owned = [i for i in range(len(shards)) if i % world == rank]
    rng = np.random.default_rng(5)
    Vu = rng.integers(-20, 20, size=(2, g.num_samples)).astype(np.int32)
    Vd = rng.standard_normal((2, g.num_mutations))
    up = shard.distributed_matmul(shards, ranges, owned, Vu, UP, g.num_samples, g.num_mutations, _oracle_fn)
    down = shard.distributed_matmul(shards, ranges, owned, Vd, DOWN, g.num_samples, g.num_mutations, _oracle_fn)
    np.save(os.path.join(result_dir, f"up{rank}.npy"), up)
    np.save(os.path.join(result_dir, f"down{rank}.npy"), down)
    # the device-tensor form (the one nccl runs), here on host tensors under gloo
    import torch

    def tensor_fn(s, X, d):
        return torch.from_numpy(_oracle_fn(s, X.numpy(), d))

    downt = shard.distributed_matmul(shards, ranges, owned, torch.from_numpy(Vd), DOWN, g.num_samples,
                                     g.num_mutations, tensor_fn)
    assert isinstance(downt, torch.Tensor)
    np.save(os.path.join(result_dir, f"downt{rank}.npy"), downt.numpy())
    # GF(2): partials from different ranks combine by XOR, not OR
    Vb = rng.integers(0, 2, size=(3, g.num_mutations)).astype(bool)
    bd = shard.distributed_matmul(shards, ranges, owned, Vb, DOWN, g.num_samples, g.num_mutations, _oracle_fn)
    np.save(os.path.join(result_dir, f"bool{rank}.npy"), bd)
    # one range per rank, combined by combine_rank_output (the benchmark's multi-GPU step)
    r2 = shard.mutation_ranges(g, world, align=100)
    mine = g.subset_mutations(np.arange(r2[rank].start, r2[rank].stop, dtype=np.uint32))
    upr = shard.combine_rank_output(torch.from_numpy(_oracle_fn(mine, Vu, UP)), UP, r2)
    dnr = shard.combine_rank_output(
        torch.from_numpy(_oracle_fn(mine, np.ascontiguousarray(Vd[:, r2[rank].start:r2[rank].stop]), DOWN)), DOWN, r2)
    np.save(os.path.join(result_dir, f"upr{rank}.npy"), upr.numpy())
    np.save(os.path.join(result_dir, f"dnr{rank}.npy"), dnr.numpy())
    dist.destroy_process_group()


def test_distributed_combine_gloo(graph, tmp_path):
    import torch.multiprocessing as mp

    import grgl_gb300 as gx

    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    g = gx.window_tree_grg(600, 3000, seed=23)
    full = _og(g)
    rng = np.random.default_rng(5)
    Vu = rng.integers(-20, 20, size=(2, g.num_samples)).astype(np.int32)
    Vd = rng.standard_normal((2, g.num_mutations))
    ref_up, ref_down = oracle.matmul(full, Vu, UP), oracle.matmul(full, Vd, DOWN)
    scale = oracle.matmul(full, np.abs(Vd), DOWN)
    Vb = np.random.default_rng(5)
    Vb.integers(-20, 20, size=(2, g.num_samples))
    Vb.standard_normal((2, g.num_mutations))
    Vb = Vb.integers(0, 2, size=(3, g.num_mutations)).astype(bool)
    ref_bool = oracle.matmul(full, Vb, DOWN)
    for r in range(world):
        assert np.array_equal(np.load(tmp_path / f"up{r}.npy"), ref_up)
        assert np.all(np.abs(np.load(tmp_path / f"down{r}.npy") - ref_down) <= 1e-12 * scale)
        assert np.all(np.abs(np.load(tmp_path / f"downt{r}.npy") - ref_down) <= 1e-12 * scale)
        assert np.array_equal(np.load(tmp_path / f"bool{r}.npy"), ref_bool)
        assert np.array_equal(np.load(tmp_path / f"upr{r}.npy"), ref_up)
        assert np.all(np.abs(np.load(tmp_path / f"dnr{r}.npy") - ref_down) <= 1e-12 * scale)


@pytest.mark.gpu
def test_sharded_grg_on_one_gpu(cuda_ok):
    import grgl_gb300 as gx
    from grgl_gb300 import shard

    g = gx.window_tree_grg(2000, 20000, seed=29)
    sg = shard.ShardedGRG(g, 4)
    rng = np.random.default_rng(3)
    Vu = rng.integers(-100, 100, size=(8, g.num_samples)).astype(np.int32)
    Vd = rng.integers(-100, 100, size=(8, g.num_mutations)).astype(np.int32)
    assert np.array_equal(sg.matmul(Vu, UP), gx.matmul(g, Vu, UP))
    assert np.array_equal(sg.matmul(Vd, DOWN), gx.matmul(g, Vd, DOWN))
