"""Range-sharded GRG matmul: the reference's split-by-range pattern (test/endtoend/test_matmul.py:264-325)
done on resident shards.

A graph is split into contiguous mutation ranges (balanced by the number of edges below each
range).  UP products of the shards are disjoint column blocks of the full product and
concatenate; DOWN products are partial sums over the shards' mutations and add up.

* On one GPU, `ShardedGRG` keeps every shard resident and runs them back to back on one stream;
  the DOWN partials accumulate into one output buffer through the C ABI's add-to-output
  semantics, so the reduction happens inside the gather kernel.
* Across ranks (torch.distributed), `distributed_matmul` gives each rank a subset of the
  shards; UP column blocks are all-gathered and DOWN partials all-reduced.  `matmul_fn` is the
  per-shard product (the GPU matmul by default; the CPU tests pass the oracle).
"""
from __future__ import annotations

from typing import Callable, List, Sequence

import numpy as np

from .api import DOWN, GRG, UP, TraversalDirection, matmul

MatmulFn = Callable[..., np.ndarray]


def mutation_ranges(grg: GRG, nshards: int, align: int = 1) -> List[range]:
    """Contiguous mutation id ranges with about the same number of edges below each.  With
    `align` > 1 every boundary is rounded to a multiple of it (e.g. the window of a window-tree
    graph, so that no two ranges share a node with children)."""
    a = grg.export_arrays()
    off, mut = a["down_off"], a["mut_node"]
    deg = np.diff(off.astype(np.int64))
    valid = mut != 0x7FFFFFFF
    w = np.ones(len(mut), dtype=np.float64)
    w[valid] += deg[mut[valid]]
    cum = np.concatenate([[0.0], np.cumsum(w)])
    bounds = [0]
    for s in range(1, nshards):
        b = int(np.searchsorted(cum, cum[-1] * s / nshards))
        if align > 1:
            b = min(len(mut), (b + align // 2) // align * align)
        bounds.append(b)
    bounds.append(len(mut))
    bounds = sorted(set(bounds))
    return [range(bounds[i], bounds[i + 1]) for i in range(len(bounds) - 1)]


def split_by_mutations(grg: GRG, nshards: int):
    """(ranges, shard graphs) for `nshards` contiguous mutation ranges."""
    ranges = mutation_ranges(grg, nshards)
    return ranges, [grg.subset_mutations(np.arange(r.start, r.stop, dtype=np.uint32)) for r in ranges]


class ShardedGRG:
    """All shards of one graph resident on the current device."""

    def __init__(self, grg: GRG, nshards: int):
        self.num_samples = grg.num_samples
        self.num_mutations = grg.num_mutations
        self.ranges, self.shards = split_by_mutations(grg, nshards)
        for s in self.shards:
            s.upload()

    def matmul(self, input, direction):
        direction = TraversalDirection(int(direction))
        import torch

        x = input if isinstance(input, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(input)).cuda()
        host = not isinstance(input, torch.Tensor)
        if direction == UP:
            out = torch.cat([matmul(s, x, UP) for s in self.shards], dim=1)
        else:
            out = torch.zeros((x.shape[0], self.num_samples), dtype=x.dtype, device=x.device)
            from . import _lib
            from .api import _DTYPE_CODES, _torch_dtype_to_np

            code = _DTYPE_CODES[np.dtype(_torch_dtype_to_np(x.dtype))]
            stream = torch.cuda.current_stream(x.device).cuda_stream
            for r, s in zip(self.ranges, self.shards):
                part = x[:, r.start:r.stop].contiguous()
                # no OVERWRITE flag: each shard adds its partial sum into `out`
                _lib.check(_lib.lib().grgx_matmul(s._h, code, part.data_ptr(), part.shape[1], part.shape[0],
                                                  int(DOWN), out.data_ptr(), out.numel(), 0, 0, None, 0, None,
                                                  _lib.FLAG_DEVICE_POINTERS, stream))
        return out.cpu().numpy() if host else out


def distributed_matmul(shards: Sequence[GRG], ranges: Sequence[range], owned: Sequence[int], V,
                       direction, num_samples: int, num_mutations: int, matmul_fn: MatmulFn = matmul):
    """Product over shards spread across torch.distributed ranks.

    Every rank passes the full input `V`, the shard list and `owned`, the indices of the shards it
    computes.  UP: each rank fills its shards' column blocks, the blocks are summed across ranks
    (disjoint, so the sum is an all-gather); DOWN: per-rank partial sums are all-reduced.  `V`
    may be a numpy array (host tensors: the gloo backend) or a CUDA tensor (the partial outputs
    stay on the device and are reduced there: the nccl backend); the result has V's kind.  bool
    inputs combine in GF(2): partials are added as bytes and reduced mod 2.
    """
    import torch
    import torch.distributed as dist

    direction = TraversalDirection(int(direction))
    is_tensor = isinstance(V, torch.Tensor)
    X = V if is_tensor else torch.from_numpy(np.ascontiguousarray(V))
    gf2 = X.dtype == torch.bool
    acc_dtype = torch.uint8 if gf2 else X.dtype
    K = X.shape[0]
    out = torch.zeros((K, num_mutations if direction == UP else num_samples), dtype=acc_dtype, device=X.device)

    def run(i, cols):
        src = V[:, cols.start:cols.stop] if direction == DOWN else V
        if not is_tensor:
            src = np.ascontiguousarray(src)
        elif direction == DOWN:
            src = src.contiguous()
        res = matmul_fn(shards[i], src, direction)
        return torch.as_tensor(np.asarray(res) if not isinstance(res, torch.Tensor) else res,
                               device=X.device).to(acc_dtype)

    for i in owned:
        r = ranges[i]
        if direction == UP:
            out[:, r.start:r.stop] = run(i, r)
        else:
            out += run(i, r)
    dist.all_reduce(out, op=dist.ReduceOp.SUM)
    if gf2:
        out = (out & 1).to(torch.bool)
    return out if is_tensor else out.numpy()


def combine_rank_output(out, direction, ranges: Sequence[range]):
    """The whole product from this rank's product over its own range (rank r of the process group
    owns ranges[r]): DOWN partial sums are all-reduced in place; UP column blocks, which differ in
    width, are all-gathered padded to the widest and concatenated in range order.  `out` is a
    torch tensor (CUDA under nccl, host under gloo)."""
    import torch
    import torch.distributed as dist

    if int(direction) == int(DOWN):
        dist.all_reduce(out, op=dist.ReduceOp.SUM)
        return out
    widest = max(len(r) for r in ranges)
    block = torch.zeros((out.shape[0], widest), dtype=out.dtype, device=out.device)
    block[:, :out.shape[1]] = out
    parts = [torch.empty_like(block) for _ in range(len(ranges))]
    dist.all_gather(parts, block)
    return torch.cat([p[:, :len(r)] for p, r in zip(parts, ranges)], dim=1)
