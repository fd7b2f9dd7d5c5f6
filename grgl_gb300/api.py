"""Python mirror of pygrgl's matmul surface, running on the GB300 kernels of libgrgx.

Names, argument meanings, output dtypes and error messages follow the reference binding
(src/python/_grgl.cpp:80-241, :1141-1230): ``matmul(grg, input, direction, emit_all_nodes=False,
by_individual=False, init=None, miss=None)`` returns a new K x cols array of the input's dtype;
misuse raises ``RuntimeError`` with the reference's message text.

Inputs may be numpy arrays (host memory; copies to and from the GPU are part of the call) or
CUDA tensors (device memory; the call runs on the current torch stream and returns a CUDA
tensor without synchronising).
"""
from __future__ import annotations

import ctypes
import enum
import os
import tempfile
from typing import Optional

import numpy as np

from . import _lib

INVALID_NODE = 0x7FFFFFFF  # include/grgl/grgnode.h:58
COAL_COUNT_NOT_SET = 0xFFFFFFFF  # include/grgl/node_data.h:31


class TraversalDirection(enum.IntEnum):
    """include/grgl/visitor.h:26 (exported by _grgl.cpp:750-757)."""

    DOWN = 1
    UP = 2


DOWN = TraversalDirection.DOWN
UP = TraversalDirection.UP

# numpy dtype -> grgx_dtype (include/grgx.h), in the order _grgl.cpp:205-238 dispatches.
_DTYPE_CODES = {
    np.dtype(np.float64): 0, np.dtype(np.float32): 1, np.dtype(np.int64): 2, np.dtype(np.int32): 3,
    np.dtype(np.int16): 4, np.dtype(np.int8): 5, np.dtype(np.uint64): 6, np.dtype(np.uint32): 7,
    np.dtype(np.uint16): 8, np.dtype(np.uint8): 9, np.dtype(np.bool_): 10,
}
_DOT_DTYPES = (np.dtype(np.float64), np.dtype(np.float32), np.dtype(np.int64), np.dtype(np.int32))


def _check(cond: bool, msg: str):
    if not cond:
        raise RuntimeError(msg)


class GRG:
    """A GRG resident for matmul: host arrays plus, after first use, the device level plan.

    Wraps a ``grgx_graph`` handle.  Immutable; safe to share between threads.
    """

    def __init__(self, handle: int):
        self._h = ctypes.c_void_p(handle)
        info = _lib.GraphInfo()
        _lib.check(_lib.lib().grgx_graph_info_get(self._h, ctypes.byref(info)))
        self._info = info

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().grgx_graph_destroy(h)
            except Exception:
                pass
            self._h = None

    # -- properties named like pygrgl.GRG ----------------------------------------------------
    @property
    def num_nodes(self) -> int:
        return int(self._info.num_nodes)

    @property
    def num_edges(self) -> int:
        return int(self._info.num_edges)

    @property
    def num_samples(self) -> int:
        return int(self._info.num_samples)

    @property
    def num_mutations(self) -> int:
        return int(self._info.num_mutations)

    @property
    def ploidy(self) -> int:
        return int(self._info.ploidy)

    @property
    def num_individuals(self) -> int:
        return self.num_samples // self.ploidy

    @property
    def has_missing_data(self) -> bool:
        return bool(self._info.has_missing)

    @property
    def has_coal_counts(self) -> bool:
        return bool(self._info.has_coals)

    def info(self) -> dict:
        info = _lib.GraphInfo()
        _lib.check(_lib.lib().grgx_graph_info_get(self._h, ctypes.byref(info)))
        return {name: int(getattr(info, name)) for name, _ in info._fields_}

    def save(self, path: str) -> None:
        """Write the graph as a .grg file (pygrgl.save_grg without simplification)."""
        _lib.check(_lib.lib().grgx_graph_save(self._h, str(path).encode()))

    def upload(self) -> "GRG":
        """Build the level plan and make it resident on the current CUDA device."""
        _lib.check(_lib.lib().grgx_graph_upload(self._h))
        return self

    def export_arrays(self) -> dict:
        """Copies of the down-edge CSR, mutation/missingness nodes and coal counts."""
        n, e, m = self.num_nodes, self.num_edges, self.num_mutations
        out = {
            "down_off": np.zeros(n + 1, dtype=np.uint64),
            "down_adj": np.zeros(e, dtype=np.uint32),
            "mut_node": np.zeros(m, dtype=np.uint32),
            "miss_node": np.zeros(m, dtype=np.uint32),
            "coals": np.zeros(n - self.num_samples, dtype=np.uint32),
        }
        _lib.check(_lib.lib().grgx_graph_export(self._h, *(a.ctypes.data for a in out.values())))
        return out

    def subset_mutations(self, mutation_ids) -> "GRG":
        """The sub-GRG of the given mutations (saveGRGSubset by mutations, serialize.h:147-166)."""
        ids = np.ascontiguousarray(mutation_ids, dtype=np.uint32)
        return _new(_lib.lib().grgx_graph_subset, self._h, ids.ctypes.data if len(ids) else None, len(ids))

    def get_down_edges(self, node: int) -> list:
        a = self._cached_arrays()
        return a["down_adj"][a["down_off"][node]:a["down_off"][node + 1]].tolist()

    def get_sample_nodes(self) -> list:
        return list(range(self.num_samples))

    def _cached_arrays(self) -> dict:
        if not hasattr(self, "_arrays"):
            self._arrays = self.export_arrays()
        return self._arrays

    def __repr__(self) -> str:
        return (f"<[grgl_gb300.GRG] mutations={self.num_mutations}, individuals={self.num_individuals}, "
                f"ploidy={self.ploidy}, mutable=No>")


def _new(fn, *args) -> GRG:
    h = ctypes.c_void_p()
    _lib.check(fn(*args, ctypes.byref(h)))
    return GRG(h.value)


def load_immutable_grg(filename: str, load_up_edges: bool = True) -> Optional[GRG]:
    """pygrgl.load_immutable_grg (_grgl.cpp:937-953): None (and a message on stderr) on failure."""
    h = ctypes.c_void_p()
    status = _lib.lib().grgx_graph_load(os.fsencode(filename), ctypes.byref(h))
    if status != _lib.OK:
        import sys

        print(f"Failed to load GRG: {_lib.last_error()}", file=sys.stderr)
        return None
    return GRG(h.value)


def from_csr(num_samples: int, ploidy: int, down_off, down_adj, mut_node, miss_node=None, coals=None) -> GRG:
    """A GRG from CSR arrays (children of node v: down_adj[down_off[v]:down_off[v+1]])."""
    off = np.ascontiguousarray(down_off, dtype=np.uint64)
    adj = np.ascontiguousarray(down_adj, dtype=np.uint32)
    mut = np.ascontiguousarray(mut_node, dtype=np.uint32)
    miss = None if miss_node is None else np.ascontiguousarray(miss_node, dtype=np.uint32)
    co = None if coals is None else np.ascontiguousarray(coals, dtype=np.uint32)
    return _new(_lib.lib().grgx_graph_from_csr, len(off) - 1, num_samples, ploidy, off.ctypes.data,
                adj.ctypes.data if len(adj) else None, len(mut), mut.ctypes.data if len(mut) else None,
                miss.ctypes.data if miss is not None else None, co.ctypes.data if co is not None else None)


def from_pygrgl(grg) -> GRG:
    """Convert a reference ``pygrgl.GRG`` (saved unsimplified through pygrgl.save_grg, then loaded)."""
    import pygrgl  # the caller's reference installation

    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "g.grg")
        pygrgl.save_grg(grg, path, False)
        out = load_immutable_grg(path)
    _check(out is not None, "conversion from pygrgl failed")
    return out


def window_tree_grg(num_samples: int, num_mutations: int, seed: int = 42, window: int = 100,
                    threads: int = 0) -> GRG:
    """Seeded window-tree GRG (one Kingman tree per window, collapsed to mutation nodes)."""
    return _new(_lib.lib().grgx_graph_generate, num_samples, num_mutations, seed, window, threads)


def _is_torch_cuda(x) -> bool:
    mod = type(x).__module__
    return mod.startswith("torch") and getattr(x, "is_cuda", False)


def _torch_dtype_to_np(t):
    import torch

    return {torch.float64: np.float64, torch.float32: np.float32, torch.int64: np.int64, torch.int32: np.int32,
            torch.int16: np.int16, torch.int8: np.int8, torch.uint8: np.uint8, torch.bool: np.bool_}.get(t)


_GRAPHS_ENABLED = [True]


def set_graph_replay(enabled: bool):
    """Enable (default) or disable replaying captured CUDA graphs for small-graph calls."""
    _GRAPHS_ENABLED[0] = bool(enabled)


def _flags(f32_compensated: bool, f64_native: bool) -> int:
    return ((0 if f32_compensated else _lib.FLAG_F32_PLAIN) | (_lib.FLAG_F64_NATIVE if f64_native else 0)
            | (0 if _GRAPHS_ENABLED[0] else _lib.FLAG_NO_GRAPH))


_PINNED_MIN_BYTES = 4 << 20


class _PinnedBlock:
    """Owner of one pinned host block from libgrgx's pool; returns it when collected."""

    __slots__ = ("ptr",)

    def __init__(self, ptr):
        self.ptr = ptr

    def __del__(self):
        try:
            _lib.lib().grgx_host_free(self.ptr)
        except Exception:  # interpreter shutdown
            pass


def _host_empty(shape, dtype):
    """An uninitialised host array for a result: pinned (pooled) memory when it is large, so
    the device-to-host copy into it runs at full speed; plain numpy memory otherwise."""
    dtype = np.dtype(dtype)
    nbytes = int(np.prod(shape)) * dtype.itemsize
    if nbytes < _PINNED_MIN_BYTES:
        return np.empty(shape, dtype=dtype)
    ptr = ctypes.c_void_p()
    if _lib.lib().grgx_host_alloc(nbytes, ctypes.byref(ptr)) != _lib.OK:
        return np.empty(shape, dtype=dtype)
    buf = (ctypes.c_char * nbytes).from_address(ptr.value)
    buf.owner = _PinnedBlock(ptr.value)
    return np.frombuffer(buf, dtype=dtype).reshape(shape)


def matmul(grg: GRG, input, direction, emit_all_nodes: bool = False, by_individual: bool = False, init=None,
           miss=None, *, f32_compensated: bool = True, f64_native: bool = False):
    """pygrgl.matmul on the GPU (reference: _grgl.cpp:187-241, grg.h:1341-1517).

    ``f32_compensated`` (float32 only, default True) accumulates with TwoSum compensation; False
    gives plain float summation.  ``f64_native`` (float64 only, default False) accumulates on the
    FP64 pipe instead of as scaled float pairs with double folds (same tolerance, slower on GB300).
    """
    if _is_torch_cuda(input):
        return _matmul_device(grg, input, direction, emit_all_nodes, by_individual, init, miss,
                              _flags(f32_compensated, f64_native))
    out, keep = _matmul_host(grg, input, direction, emit_all_nodes, by_individual, init, miss,
                             _flags(f32_compensated, f64_native), None)
    _finish_miss(miss, keep[2])
    return out


def _matmul_host(grg, input, direction, emit_all, by_indiv, init, miss, extra_flags, stream):
    """The numpy form of matmul: validation as in dispatchMult (_grgl.cpp:108-183), then one
    grgx_matmul on host buffers.  Returns the output and the buffers the call reads or writes
    (input, init, miss as passed to the library), which an asynchronous call keeps alive."""
    direction = TraversalDirection(int(direction))
    if not isinstance(input, np.ndarray):
        raise RuntimeError(f"Unsupported numpy dtype: {np.asarray(input).dtype}")
    arr = np.ascontiguousarray(input)
    _check(arr.ndim == 2, "matmul() only support two dimensional numpy arrays as input.")
    rows, cols = arr.shape
    _check(rows != 0 and cols != 0, "matmul() requires non-zero dimensions.")
    _check(arr.dtype in _DTYPE_CODES, f"Unsupported numpy dtype: {arr.dtype}")
    code = _DTYPE_CODES[arr.dtype]
    nsamp = grg.num_individuals if by_indiv else grg.num_samples
    out_cols = grg.num_nodes if emit_all else (nsamp if direction == DOWN else grg.num_mutations)
    init_kind, init_arr = _parse_init(grg, init, arr.dtype, rows, code == 10)
    miss_arr = _parse_miss(miss, arr.dtype, rows, cols, out_cols, direction, emit_all)
    out = _host_empty((rows, out_cols), arr.dtype)
    flags = _lib.FLAG_OVERWRITE | extra_flags
    _lib.check(_lib.lib().grgx_matmul(grg._h, code, arr.ctypes.data, cols, rows, int(direction), out.ctypes.data,
                                      out.size, int(bool(emit_all)), int(bool(by_indiv)),
                                      init_arr.ctypes.data if init_arr is not None else None, init_kind,
                                      miss_arr.ctypes.data if miss_arr is not None else None, flags, stream))
    return out, (arr, init_arr, miss_arr)


def _finish_miss(miss, miss_arr):
    """UP writes `miss` in place: copy back when the library worked on a converted copy."""
    if miss_arr is not None and miss_arr is not miss:
        miss[...] = miss_arr


class PendingMatmul:
    """A matmul on host buffers queued on a CUDA stream by matmul_async.  result() waits for the
    stream to reach the end of the call and returns the output array; until then the output
    (and an UP `miss`) are being written and the buffers passed to the call stay referenced."""

    def __init__(self, out, miss, keep, event):
        self._out, self._miss, self._keep, self._event = out, miss, keep, event

    def done(self) -> bool:
        """True once the call has finished on the device (result() will not wait)."""
        return self._event.query()

    def result(self):
        if self._keep is not None:
            self._event.synchronize()
            _finish_miss(self._miss, self._keep[2])
            self._keep = None
        return self._out


def matmul_async(grg: GRG, input, direction, emit_all_nodes: bool = False, by_individual: bool = False,
                 init=None, miss=None, *, stream=None, f32_compensated: bool = True,
                 f64_native: bool = False) -> PendingMatmul:
    """matmul on numpy buffers without waiting for it (no counterpart in the reference).

    The copy of the input to the device, the product and the copy of the result back are
    queued on `stream` (a torch.cuda.Stream; default the current stream) and the call returns a
    PendingMatmul at once; its result() returns the same array matmul would.  With inputs in
    page-locked memory (host_empty), calls queued on two streams overlap one call's copies with
    the other's product.  The arguments, checks and messages are those of matmul.
    """
    import torch

    if _is_torch_cuda(input):
        raise RuntimeError("matmul_async takes numpy arrays; device tensors are asynchronous with matmul already")
    if stream is None:
        stream = torch.cuda.current_stream()
    out, keep = _matmul_host(grg, input, direction, emit_all_nodes, by_individual, init, miss,
                             _flags(f32_compensated, f64_native) | _lib.FLAG_ASYNC, stream.cuda_stream)
    event = torch.cuda.Event()
    event.record(stream)
    return PendingMatmul(out, miss, keep, event)


def host_empty(shape, dtype):
    """An uninitialised numpy array in page-locked (pinned, pooled) host memory when it is 4 MiB
    or larger, else in plain numpy memory: inputs in it reach the device at the link's full
    speed and let matmul_async overlap their copies with other work."""
    return _host_empty(shape, dtype)


def _parse_init(grg, init, dtype, rows, is_bool):
    """init handling of dispatchMult (_grgl.cpp:116-142)."""
    if init is None:
        return 0, None
    _check(not is_bool, "init=... is not supported with boolean dtype")
    if isinstance(init, str):
        _check(init == "xtx", f"Unexpected init value: {init}")
        return 3, None
    arr = init if _is_torch_cuda(init) else np.asarray(init)
    got = _torch_dtype_to_np(arr.dtype) if _is_torch_cuda(arr) else arr.dtype
    _check(isinstance(init, np.ndarray) or _is_torch_cuda(init), f"The init matrix must match the dtype of the "
           f"input matrix. Got: {np.asarray(init).dtype}")
    _check(np.dtype(got) == dtype, f"The init matrix must match the dtype of the input matrix. Got: {np.dtype(got)}")
    if arr.ndim == 1:
        _check(arr.shape[0] == rows,
               "If init has a single dimension, it must match the number of rows in the input matrix")
        return 1, (arr.contiguous() if _is_torch_cuda(arr) else np.ascontiguousarray(arr))
    if arr.ndim == 2:
        _check(tuple(arr.shape) == (rows, grg.num_nodes),
               "If init is a matrix, it must match the dimensions ROW x NODES")
        return 2, (arr.contiguous() if _is_torch_cuda(arr) else np.ascontiguousarray(arr))
    return 0, None


def _parse_miss(miss, dtype, rows, cols, out_cols, direction, emit_all):
    """miss handling of dispatchMult (_grgl.cpp:144-167)."""
    if miss is None:
        return None
    _check(not emit_all, 'The "miss" parameter cannot be mixed with the "emit_all_nodes" parameter')
    if _is_torch_cuda(miss):
        got = np.dtype(_torch_dtype_to_np(miss.dtype))
    else:
        _check(isinstance(miss, np.ndarray),
               f'The "miss" input must be a matrix with dtype matching the input matrix. Got: '
               f'{np.asarray(miss).dtype}')
        got = miss.dtype
    _check(got == dtype, f'The "miss" input must be a matrix with dtype matching the input matrix. Got: {got}')
    _check(miss.ndim == 2, f'"miss" must be a two-dimension numpy array (matrix). ndim={miss.ndim}')
    mrows, mcols = miss.shape
    _check(mrows == rows, f'"miss" has {mrows} rows, but must match the input and output matrices ({rows})')
    if direction == DOWN:
        _check(mcols == cols, f'The "miss" matrix must match the number of columns in the input matrix. Got: {mcols}')
    else:
        _check(mcols == out_cols,
               f'The "miss" matrix must match the number of columns in the output matrix. Got: {mcols}')
    if _is_torch_cuda(miss):
        _check(miss.is_contiguous(), '"miss" must be contiguous')
        return miss
    return miss if miss.flags.c_contiguous else np.ascontiguousarray(miss)


def _matmul_device(grg, x, direction, emit_all, by_indiv, init, miss, extra_flags):
    import torch

    direction = TraversalDirection(int(direction))
    _check(x.dim() == 2, "matmul() only support two dimensional numpy arrays as input.")
    x = x.contiguous()
    rows, cols = x.shape
    _check(rows != 0 and cols != 0, "matmul() requires non-zero dimensions.")
    npd = _torch_dtype_to_np(x.dtype)
    _check(npd is not None, f"Unsupported dtype: {x.dtype}")
    code = _DTYPE_CODES[np.dtype(npd)]
    nsamp = grg.num_individuals if by_indiv else grg.num_samples
    out_cols = grg.num_nodes if emit_all else (nsamp if direction == DOWN else grg.num_mutations)
    init_kind, init_t = _parse_init(grg, init, np.dtype(npd), rows, code == 10)
    if init_t is not None and not _is_torch_cuda(init_t):
        init_t = torch.from_numpy(np.ascontiguousarray(init_t)).to(x.device)
    miss_t = _parse_miss(miss, np.dtype(npd), rows, cols, out_cols, direction, emit_all)
    _check(miss_t is None or _is_torch_cuda(miss_t), '"miss" must be a CUDA tensor when the input is one')
    out = torch.empty((rows, out_cols), dtype=x.dtype, device=x.device)
    stream = torch.cuda.current_stream(x.device).cuda_stream
    flags = _lib.FLAG_OVERWRITE | _lib.FLAG_DEVICE_POINTERS | extra_flags
    with torch.cuda.device(x.device):
        _lib.check(_lib.lib().grgx_matmul(grg._h, code, x.data_ptr(), cols, rows, int(direction), out.data_ptr(),
                                          out.numel(), int(bool(emit_all)), int(bool(by_indiv)),
                                          init_t.data_ptr() if init_t is not None else None, init_kind,
                                          miss_t.data_ptr() if miss_t is not None else None, flags, stream))
    return out


def dot_product(grg: GRG, input, direction):
    """pygrgl.dot_product (_grgl.cpp:80-98): 1-D input, f64/f32/i64/i32 only."""
    if not isinstance(input, np.ndarray):
        raise RuntimeError(f"Unsupported numpy dtype: {np.asarray(input).dtype}")
    arr = np.ascontiguousarray(input)
    _check(arr.ndim == 1, "dot_product() only support one-dimensional numpy arrays as input.")
    _check(arr.shape[0] != 0, "dot_product() requires non-empty array input.")
    _check(arr.dtype in _DOT_DTYPES, f"Unsupported numpy dtype: {arr.dtype}")
    return matmul(grg, arr.reshape(1, -1), direction)[0]


def measure_l2_bandwidth(nbytes: int = 48 << 20, reps: int = 40) -> float:
    """Measured L2 -> SM read bandwidth of the current device, GB/s (diagnostic)."""
    v = ctypes.c_double()
    _lib.check(_lib.lib().grgx_measure_l2_bandwidth(nbytes, reps, ctypes.byref(v)))
    return v.value


def pool_usage(device: int = 0) -> dict:
    """Bytes of the library's own device memory pool on `device`: handed out to calls in flight
    (`used`) and held from the device (`reserved`, cached between calls)."""
    u, r = ctypes.c_uint64(), ctypes.c_uint64()
    _lib.check(_lib.lib().grgx_pool_usage(int(device), ctypes.byref(u), ctypes.byref(r)))
    return {"used": u.value, "reserved": r.value}


def set_timing(enabled):
    """Per-call CUDA-event timing on this thread: True (read back per call, see last_timing),
    "deferred" (no per-call sync, see collect_timings) or False."""
    _lib.lib().grgx_set_timing(2 if enabled == "deferred" else int(bool(enabled)))


def collect_timings() -> list:
    """The deferred timings of this thread's calls since the last collection, in call order."""
    cap = 65536
    buf = (_lib.Timing * cap)()
    n = ctypes.c_uint64()
    _lib.check(_lib.lib().grgx_collect_timings(buf, cap, ctypes.byref(n)))
    return [{"total_ms": t.total_ms, "sweep_ms": t.sweep_ms, "launches": int(t.launches), "alg_bytes": int(t.alg_bytes)}
            for t in buf[:n.value]]


def last_timing() -> dict:
    t = _lib.Timing()
    _lib.check(_lib.lib().grgx_last_timing(ctypes.byref(t)))
    return {"total_ms": t.total_ms, "sweep_ms": t.sweep_ms, "launches": int(t.launches),
            "alg_bytes": int(t.alg_bytes)}


def matmul_standardized(grg: GRG, input, direction, *, f32_compensated: bool = True, f64_native: bool = False):
    """Product with the standardized genotype matrix Z = (X - mu) / sigma (haploid p_j, sigma_j =
    sqrt(p_j(1-p_j)), zero-variance columns masked): ``V Z`` for UP (V: K x N), ``V Z^T`` for DOWN
    (V: K x M).  float32/float64; the reductions it divides by are float64 on the GPU."""
    direction = TraversalDirection(int(direction))
    flags = _flags(f32_compensated, f64_native)
    rows_out = grg.num_mutations if direction == UP else grg.num_samples
    if _is_torch_cuda(input):
        import torch

        x = input.contiguous()
        _check(x.dim() == 2 and x.dtype in (torch.float32, torch.float64),
               "standardized products take 2-D float32 or float64 input")
        out = torch.empty((x.shape[0], rows_out), dtype=x.dtype, device=x.device)
        code = 0 if x.dtype == torch.float64 else 1
        stream = torch.cuda.current_stream(x.device).cuda_stream
        _lib.check(_lib.lib().grgx_matmul_standardized(grg._h, code, x.data_ptr(), x.shape[1], x.shape[0],
                                                       int(direction), out.data_ptr(), out.numel(),
                                                       flags | _lib.FLAG_DEVICE_POINTERS, stream))
        return out
    _check(isinstance(input, np.ndarray), f"Unsupported numpy dtype: {np.asarray(input).dtype}")
    x = np.ascontiguousarray(input)
    _check(x.ndim == 2, "matmul() only support two dimensional numpy arrays as input.")
    _check(x.dtype in (np.float32, np.float64), "standardized products take float32 or float64 input")
    out = _host_empty((x.shape[0], rows_out), x.dtype)
    _lib.check(_lib.lib().grgx_matmul_standardized(grg._h, 0 if x.dtype == np.float64 else 1, x.ctypes.data,
                                                   x.shape[1], x.shape[0], int(direction), out.ctypes.data,
                                                   out.size, flags, None))
    return out


def matmul_gram(grg: GRG, input, first_direction, *, standardized: bool = False, f32_compensated: bool = True,
                f64_native: bool = False):
    """Two chained traversals with the intermediate kept on the GPU: ``V X X^T`` (first UP, V:
    K x N) or ``V X^T X`` (first DOWN, V: K x M); with ``standardized`` the standardized Z
    replaces X.  numpy in -> numpy out, CUDA tensor in -> CUDA tensor out."""
    first = TraversalDirection(int(first_direction))
    flags = _flags(f32_compensated, f64_native)
    if _is_torch_cuda(input):
        import torch

        x = input.contiguous()
        npd = _torch_dtype_to_np(x.dtype)
        _check(x.dim() == 2 and npd is not None, "matmul() only support two dimensional numpy arrays as input.")
        out = torch.empty_like(x)
        stream = torch.cuda.current_stream(x.device).cuda_stream
        _lib.check(_lib.lib().grgx_matmul_gram(grg._h, _DTYPE_CODES[np.dtype(npd)], x.data_ptr(), x.shape[1],
                                               x.shape[0], int(first), out.data_ptr(), out.numel(),
                                               int(bool(standardized)), flags | _lib.FLAG_DEVICE_POINTERS, stream))
        return out
    _check(isinstance(input, np.ndarray), f"Unsupported numpy dtype: {np.asarray(input).dtype}")
    x = np.ascontiguousarray(input)
    _check(x.ndim == 2, "matmul() only support two dimensional numpy arrays as input.")
    _check(x.dtype in _DTYPE_CODES, f"Unsupported numpy dtype: {x.dtype}")
    out = _host_empty(x.shape, x.dtype)
    _lib.check(_lib.lib().grgx_matmul_gram(grg._h, _DTYPE_CODES[x.dtype], x.ctypes.data, x.shape[1], x.shape[0],
                                           int(first), out.ctypes.data, out.size, int(bool(standardized)), flags,
                                           None))
    return out


# ---- batching and serving ----------------------------------------------------------------------


def _request_for(grg, x, direction, standardized=False, by_individual=False):
    """Validate one request and allocate its output (host or device like the input)."""
    direction = TraversalDirection(int(direction))
    opts = (_lib.REQUEST_STANDARDIZED if standardized else 0) | (_lib.REQUEST_BY_INDIVIDUAL if by_individual else 0)
    _check(not (standardized and by_individual), "standardized products are per haplotype (no by_individual)")
    nsamp = grg.num_individuals if by_individual else grg.num_samples
    cols = nsamp if direction == UP else grg.num_mutations
    out_cols = grg.num_mutations if direction == UP else nsamp
    if _is_torch_cuda(x):
        import torch

        x = x.contiguous()
        npd = _torch_dtype_to_np(x.dtype)
        _check(npd is not None, f"Unsupported dtype: {x.dtype}")
        _check(x.dim() == 2 and x.shape[0] > 0 and x.shape[1] == cols,
               "Input vector is not size N (numSamples, or numIndividuals depending on flags)" if direction == UP
               else "Input vector is not size M (numMutations)")
        out = torch.empty((x.shape[0], out_cols), dtype=x.dtype, device=x.device)
        code = _DTYPE_CODES[np.dtype(npd)]
        if standardized:
            _check(npd in (np.float32, np.float64), "standardized products take float32 or float64 input")
        return x, out, _lib.Request(code, int(direction), x.shape[0], x.data_ptr(), out.data_ptr(), opts)
    _check(isinstance(x, np.ndarray), f"Unsupported numpy dtype: {np.asarray(x).dtype}")
    x = np.ascontiguousarray(x)
    _check(x.ndim == 2, "matmul() only support two dimensional numpy arrays as input.")
    _check(x.dtype in _DTYPE_CODES, f"Unsupported numpy dtype: {x.dtype}")
    _check(x.shape[0] > 0 and x.shape[1] > 0, "matmul() requires non-zero dimensions.")
    _check(x.shape[1] == cols,
           "Input vector is not size N (numSamples, or numIndividuals depending on flags)" if direction == UP
           else "Input vector is not size M (numMutations)")
    if standardized:
        _check(x.dtype in (np.float32, np.float64), "standardized products take float32 or float64 input")
    out = _host_empty((x.shape[0], out_cols), x.dtype)
    return x, out, _lib.Request(_DTYPE_CODES[x.dtype], int(direction), x.shape[0], x.ctypes.data, out.ctypes.data,
                                opts)


def autotune(grg: GRG, dtype, rows: int, direction, *, f32_compensated: bool = True,
             f64_native: bool = False) -> str:
    """Measure every launch shape on each level of one traversal of ``grg`` for ``rows`` x cols
    inputs of ``dtype`` in ``direction`` and record the winners in the process-wide shape table
    (keyed on the level's width, mean degree, the storage kind and K).  Returns the per-level
    report.  Later calls on any graph whose levels match an entry run the tuned shape."""
    code = _DTYPE_CODES[np.dtype(dtype)]
    need = ctypes.c_uint64()
    buf = ctypes.create_string_buffer(1 << 16)
    _lib.check(_lib.lib().grgx_autotune(grg._h, code, int(rows), int(TraversalDirection(int(direction))),
                                        _flags(f32_compensated, f64_native), buf, len(buf), ctypes.byref(need)))
    return buf.value.decode()


def autotune_table() -> str:
    """The shape table as text (one ``kind stride rows_log2 degree_log2 g tiles variant`` per line)."""
    need = ctypes.c_uint64()
    _lib.check(_lib.lib().grgx_autotune_export(None, 0, ctypes.byref(need)))
    buf = ctypes.create_string_buffer(int(need.value) + 1)
    _lib.check(_lib.lib().grgx_autotune_export(buf, len(buf), ctypes.byref(need)))
    return buf.value.decode()


def autotune_load(text: str) -> None:
    """Merge a saved shape table (``autotune_table()`` output) into the process-wide table."""
    _lib.check(_lib.lib().grgx_autotune_import(text.encode()))


def autotune_clear() -> None:
    """Empty the shape table: every level runs its default shape."""
    _lib.lib().grgx_autotune_clear()


def matmul_batch(grg: GRG, requests, max_cols: int = 0, *, f32_compensated: bool = True, f64_native: bool = False):
    """Several products on one graph, coalesced into shared traversals.

    ``requests`` is a list of ``(input, direction)``, ``(input, direction, standardized)`` or
    ``(input, direction, standardized, by_individual)``; inputs are all numpy arrays or all CUDA
    tensors.  A standardized request computes what ``matmul_standardized`` does; by_individual
    has ``matmul``'s meaning.  Returns the outputs in order.  Requests of the same direction
    and dtype are stacked into traversals of at most ``max_cols`` rows (0 = 512 for 4-byte and
    smaller dtypes, 256 for 8-byte ones); a request's rows may be cut across two traversals.
    """
    prepared = [_request_for(grg, r[0], r[1], bool(r[2]) if len(r) > 2 else False,
                             bool(r[3]) if len(r) > 3 else False) for r in requests]
    if not prepared:
        return []
    dev = _is_torch_cuda(prepared[0][0])
    _check(all(_is_torch_cuda(p[0]) == dev for p in prepared), "inputs must be all host or all device arrays")
    arr = (_lib.Request * len(prepared))(*[p[2] for p in prepared])
    flags = _flags(f32_compensated, f64_native)
    stream = None
    if dev:
        import torch

        flags |= _lib.FLAG_DEVICE_POINTERS
        stream = torch.cuda.current_stream(prepared[0][0].device).cuda_stream
    _lib.check(_lib.lib().grgx_matmul_batch(grg._h, arr, len(prepared), max_cols, flags, stream))
    return [p[1] for p in prepared]


class Server:
    """Serving loop with continuous batching over resident graphs (native worker threads).

    ``submit`` queues a plain product and returns a ticket; ``result`` waits for it and returns
    ``(output, stats)`` where stats has the submit/start/done times (seconds since the server
    started) and the size of the batch the request ran in.
    """

    def __init__(self, workers: int = 2, memory_budget: int = 0, max_cols: int = 0):
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().grgx_server_create(workers, memory_budget, max_cols, ctypes.byref(h)))
        self._h = h
        self._graphs = []
        self._live = {}

    def add_graph(self, grg: GRG) -> int:
        gid = ctypes.c_uint32()
        _lib.check(_lib.lib().grgx_server_add_graph(self._h, grg._h, ctypes.byref(gid)))
        self._graphs.append(grg)
        return int(gid.value)

    def submit(self, graph_id: int, input, direction, standardized: bool = False, by_individual: bool = False) -> int:
        x, out, req = _request_for(self._graphs[graph_id], input, direction, standardized, by_individual)
        _check(not _is_torch_cuda(x), "the server takes host (numpy) arrays")
        t = ctypes.c_uint64()
        _lib.check(_lib.lib().grgx_server_submit(self._h, graph_id, ctypes.byref(req), ctypes.byref(t)))
        self._live[int(t.value)] = (x, out)
        return int(t.value)

    def result(self, ticket: int, timeout: float = 0.0):
        st = _lib.RequestStats()
        status = _lib.lib().grgx_server_wait(self._h, ticket, float(timeout), ctypes.byref(st))
        x, out = self._live.pop(ticket, (None, None))
        _lib.check(status)
        return out, {"submit_s": st.submit_s, "start_s": st.start_s, "done_s": st.done_s,
                     "latency_s": st.done_s - st.submit_s, "batch_requests": int(st.batch_requests),
                     "batch_rows": int(st.batch_rows)}

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.lib().grgx_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
