"""CPU oracle for GRG matrix multiplication -- TEST INFRASTRUCTURE ONLY.

This package is the checker.  Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline
legs of ``bench.py`` may import it; the product (``grgl_gb300``) never does.

* ``grg_oracle.c`` restates the reference CPU algorithm ``GRG::matrixMultiplication``
  (include/grgl/grg.h:1341-1517) in plain C; :func:`matmul` wraps it with the argument checks
  of the reference binding (src/python/_grgl.cpp:100-241).
* :func:`read_grg` is an independent numpy reader of the ``.grg`` format
  (src/serialize.cpp:697-890), used to cross-check the product's loader.
* ``build_ref.sh`` compiles the reference itself (where its sources exist) into ``oracle/_ref``
  so that golden fixtures can be produced by the reference and the restatement pinned to them.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading
import weakref
from dataclasses import dataclass
from pathlib import Path
from typing import Optional

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
INVALID_NODE = 0x7FFFFFFF
COAL_NOT_SET = 0xFFFFFFFF
DOWN, UP = 1, 2

_DTYPES = {
    np.dtype(np.float64): 0, np.dtype(np.float32): 1, np.dtype(np.int64): 2, np.dtype(np.int32): 3,
    np.dtype(np.int16): 4, np.dtype(np.int8): 5, np.dtype(np.uint64): 6, np.dtype(np.uint32): 7,
    np.dtype(np.uint16): 8, np.dtype(np.uint8): 9, np.dtype(np.bool_): 10,
}


SOURCES = ("grg_oracle.c", "window_tree.c")


def build(force: bool = False) -> Path:
    """Compile liboracle.so from grg_oracle.c and window_tree.c (gcc, no FMA contraction)."""
    srcs = [HERE / f for f in SOURCES]
    if not force and LIB_PATH.exists() and all(LIB_PATH.stat().st_mtime >= s.stat().st_mtime for s in srcs):
        return LIB_PATH
    tmp = LIB_PATH.with_suffix(f".so.tmp{os.getpid()}")
    subprocess.run(["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", *map(str, srcs), "-o",
                    str(tmp), "-lpthread"], check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def host_threads() -> int:
    """Host cores this process may run on."""
    try:
        return max(1, len(os.sched_getaffinity(0)))
    except AttributeError:
        return max(1, os.cpu_count() or 1)


class _Graph(ctypes.Structure):
    _fields_ = [("num_nodes", ctypes.c_uint64), ("num_samples", ctypes.c_uint64), ("ploidy", ctypes.c_uint64),
                ("num_mutations", ctypes.c_uint64), ("down_off", ctypes.c_void_p), ("down_adj", ctypes.c_void_p),
                ("mut_node", ctypes.c_void_p), ("miss_node", ctypes.c_void_p), ("coals", ctypes.c_void_p)]


class _WTGraph(ctypes.Structure):
    _fields_ = [("num_nodes", ctypes.c_uint64), ("num_edges", ctypes.c_uint64), ("num_mutations", ctypes.c_uint64),
                ("down_off", ctypes.c_void_p), ("down_adj", ctypes.c_void_p), ("mut_node", ctypes.c_void_p)]


_lib = None
_lib_lock = threading.Lock()


def _load():
    global _lib
    with _lib_lock:
        if _lib is None:
            if not LIB_PATH.exists():
                build()
            lib = ctypes.CDLL(str(LIB_PATH))
            lib.oracle_matmul.restype = ctypes.c_int
            lib.oracle_matmul.argtypes = [ctypes.POINTER(_Graph), ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64,
                                          ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64,
                                          ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
            lib.oracle_shards_create_mt.restype = ctypes.c_void_p
            lib.oracle_shards_create_mt.argtypes = [ctypes.POINTER(_Graph), ctypes.c_int, ctypes.c_int,
                                                    ctypes.c_uint64]
            lib.oracle_shards_destroy.argtypes = [ctypes.c_void_p]
            lib.oracle_shard_edges.restype = ctypes.c_uint64
            lib.oracle_shard_edges.argtypes = [ctypes.c_void_p, ctypes.c_int]
            lib.oracle_matmul_shard_range.restype = ctypes.c_int
            lib.oracle_matmul_shard_range.argtypes = [ctypes.POINTER(_Graph), ctypes.c_void_p, ctypes.c_int,
                                                      ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64,
                                                      ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p,
                                                      ctypes.c_uint64, ctypes.POINTER(ctypes.c_double)]
            lib.oracle_window_tree.restype = ctypes.c_int
            lib.oracle_window_tree.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                                               ctypes.c_int, ctypes.POINTER(_WTGraph)]
            lib.oracle_window_tree_free.argtypes = [ctypes.POINTER(_WTGraph)]
            _lib = lib
    return _lib


@dataclass
class OracleGraph:
    """The arrays of a CSRGRG that matmul reads (grg.h:1232-1303); samples are nodes 0..N-1."""

    num_samples: int
    ploidy: int
    down_off: np.ndarray  # uint64, nodes + 1
    down_adj: np.ndarray  # uint32
    mut_node: np.ndarray  # uint32 (INVALID_NODE = unmapped)
    miss_node: Optional[np.ndarray] = None
    coals: Optional[np.ndarray] = None

    def __post_init__(self):
        self.down_off = np.ascontiguousarray(self.down_off, dtype=np.uint64)
        self.down_adj = np.ascontiguousarray(self.down_adj, dtype=np.uint32)
        self.mut_node = np.ascontiguousarray(self.mut_node, dtype=np.uint32)
        if self.miss_node is not None:
            self.miss_node = np.ascontiguousarray(self.miss_node, dtype=np.uint32)
        if self.coals is not None:
            self.coals = np.ascontiguousarray(self.coals, dtype=np.uint32)

    @property
    def num_nodes(self) -> int:
        return len(self.down_off) - 1

    @property
    def num_mutations(self) -> int:
        return len(self.mut_node)

    @property
    def num_edges(self) -> int:
        return int(self.down_off[-1])

    @property
    def num_individuals(self) -> int:
        return self.num_samples // self.ploidy

    def _struct(self) -> _Graph:
        s = _Graph()
        s.num_nodes, s.num_samples, s.ploidy, s.num_mutations = (self.num_nodes, self.num_samples, self.ploidy,
                                                                  self.num_mutations)
        s.down_off = self.down_off.ctypes.data
        s.down_adj = self.down_adj.ctypes.data if len(self.down_adj) else None
        s.mut_node = self.mut_node.ctypes.data if len(self.mut_node) else None
        s.miss_node = self.miss_node.ctypes.data if self.miss_node is not None else None
        s.coals = self.coals.ctypes.data if self.coals is not None else None
        return s

    def dense_X(self) -> np.ndarray:
        """N x M genotype matrix with path multiplicities (test/endtoend/test_matmul.py:21-38)."""
        eye = np.eye(self.num_samples, dtype=np.int64)
        return matmul(self, eye, UP)


def _check(cond: bool, msg: str):
    if not cond:
        raise RuntimeError(msg)


def matmul(g: OracleGraph, input, direction: int, emit_all_nodes: bool = False, by_individual: bool = False,
           init=None, miss=None) -> np.ndarray:
    """Oracle ``pygrgl.matmul`` (src/python/_grgl.cpp:100-241 checks, grg.h:1341-1517 math)."""
    direction = int(direction)
    if not isinstance(input, np.ndarray):
        raise RuntimeError(f"Unsupported numpy dtype: {np.asarray(input).dtype}")
    arr = np.ascontiguousarray(input)
    _check(arr.ndim == 2, "matmul() only support two dimensional numpy arrays as input.")
    rows, cols = arr.shape
    _check(rows != 0 and cols != 0, "matmul() requires non-zero dimensions.")
    _check(arr.dtype in _DTYPES, f"Unsupported numpy dtype: {arr.dtype}")
    code = _DTYPES[arr.dtype]
    nsamp = g.num_individuals if by_individual else g.num_samples
    out_cols = g.num_nodes if emit_all_nodes else (nsamp if direction == DOWN else g.num_mutations)
    init_kind, init_arr = 0, None
    if init is not None:
        _check(code != 10, "init=... is not supported with boolean dtype")
        if isinstance(init, str):
            _check(init == "xtx", f"Unexpected init value: {init}")
            init_kind = 3
        else:
            _check(isinstance(init, np.ndarray) and init.dtype == arr.dtype,
                   f"The init matrix must match the dtype of the input matrix. Got: {np.asarray(init).dtype}")
            init_arr = np.ascontiguousarray(init)
            if init_arr.ndim == 1:
                _check(init_arr.shape[0] == rows,
                       "If init has a single dimension, it must match the number of rows in the input matrix")
                init_kind = 1
            if init_arr.ndim == 2:
                _check(init_arr.shape == (rows, g.num_nodes),
                       "If init is a matrix, it must match the dimensions ROW x NODES")
                init_kind = 2
    miss_arr = None
    if miss is not None:
        _check(not emit_all_nodes, 'The "miss" parameter cannot be mixed with the "emit_all_nodes" parameter')
        _check(isinstance(miss, np.ndarray) and miss.dtype == arr.dtype,
               f'The "miss" input must be a matrix with dtype matching the input matrix. Got: {np.asarray(miss).dtype}')
        _check(miss.ndim == 2, f'"miss" must be a two-dimension numpy array (matrix). ndim={miss.ndim}')
        _check(miss.shape[0] == rows,
               f'"miss" has {miss.shape[0]} rows, but must match the input and output matrices ({rows})')
        if direction == DOWN:
            _check(miss.shape[1] == cols,
                   f'The "miss" matrix must match the number of columns in the input matrix. Got: {miss.shape[1]}')
        else:
            _check(miss.shape[1] == out_cols,
                   f'The "miss" matrix must match the number of columns in the output matrix. Got: {miss.shape[1]}')
        miss_arr = miss if miss.flags.c_contiguous else np.ascontiguousarray(miss)
    # validateMatMulInputs (internal_mult.h:130-158)
    if direction == DOWN:
        _check(cols == g.num_mutations, "Input vector is not size M (numMutations)")
        _check(emit_all_nodes or out_cols == nsamp,
               "Output vector is not size N (numSamples, or numIndividuals depending on flags)")
    else:
        _check(cols == nsamp, "Input vector is not size N (numSamples, or numIndividuals depending on flags)")
        _check(emit_all_nodes or out_cols == g.num_mutations, "Output vector is not size M (numMutations)")
    out = np.zeros((rows, out_cols), dtype=arr.dtype)
    gs = g._struct()
    rc = _load().oracle_matmul(ctypes.byref(gs), code, arr.ctypes.data, cols, rows, direction, out.ctypes.data,
                               out_cols, int(bool(emit_all_nodes)), int(bool(by_individual)),
                               init_arr.ctypes.data if init_arr is not None else None, init_kind,
                               miss_arr.ctypes.data if miss_arr is not None else None)
    if rc == -2:
        raise RuntimeError("Coalescent counts not available for this GRG (init=XTX won't work)")
    _check(rc == 0, f"oracle failure {rc}")
    if miss_arr is not None and miss_arr is not miss:
        miss[...] = miss_arr
    return out


class Shards:
    """The reference's range-split multi-core pattern (test/endtoend/test_matmul.py:264-325): the
    mutations cut into `nshards` contiguous ranges, each range's sub-graph (the nodes below its
    mutations, what saveGRGSubset keeps) multiplied on its own thread, DOWN partial outputs
    summed in shard order, UP outputs disjoint.  Range starts are rounded to multiples of
    `align` mutations (the window of a window-tree graph: then no two shards share a node with
    children).  `build_threads` threads build the shards."""

    def __init__(self, g: OracleGraph, nshards: int, build_threads: int = 0, align: int = 1):
        self.g = g
        self._gs = g._struct()
        self.ptr = _load().oracle_shards_create_mt(ctypes.byref(self._gs), int(nshards),
                                                   int(build_threads or host_threads()), int(align))
        _check(bool(self.ptr), "sharding needs a topologically ordered graph")
        self.nshards = nshards
        self.last_reduce_s = 0.0

    def edges(self, first: int = 0, count: Optional[int] = None) -> int:
        """Edges the shards [first, first + count) traverse."""
        count = self.nshards - first if count is None else count
        lib = _load()
        return sum(int(lib.oracle_shard_edges(self.ptr, i)) for i in range(first, first + count))

    def matmul(self, input: np.ndarray, direction: int, first: int = 0, count: Optional[int] = None) -> np.ndarray:
        """The product over shards [first, first + count) (all by default), one thread per shard;
        the DOWN partial-sum time is left in `last_reduce_s`."""
        arr = np.ascontiguousarray(input)
        rows, cols = arr.shape
        count = self.nshards - first if count is None else count
        out_cols = self.g.num_samples if int(direction) == DOWN else self.g.num_mutations
        out = np.zeros((rows, out_cols), dtype=arr.dtype)
        red = ctypes.c_double(0.0)
        rc = _load().oracle_matmul_shard_range(ctypes.byref(self._gs), self.ptr, int(first), int(count),
                                               _DTYPES[arr.dtype], arr.ctypes.data, cols, rows, int(direction),
                                               out.ctypes.data, out_cols, ctypes.byref(red))
        _check(rc == 0, f"oracle failure {rc}")
        self.last_reduce_s = red.value
        return out

    def __del__(self):
        if getattr(self, "ptr", None):
            _load().oracle_shards_destroy(self.ptr)
            self.ptr = None


def _owned(ptr: int, count: int, ctype, free_fn) -> np.ndarray:
    """A numpy view of `count` elements at `ptr` that frees the block (free_fn) when the last
    view of it goes away."""
    if count == 0:
        free_fn(ptr)
        return np.zeros(0, dtype=ctype)
    buf = (np.ctypeslib.as_ctypes_type(ctype) * count).from_address(ptr)
    weakref.finalize(buf, free_fn, ptr)
    return np.frombuffer(buf, dtype=ctype)


def window_tree(num_samples: int, num_mutations: int, seed: int = 42, window: int = 100,
                threads: int = 0) -> OracleGraph:
    """The seeded window-tree graph (window_tree.c), generated on `threads` host threads (all by
    default) without the product library: the same graph the product's generator makes."""
    lib = _load()
    wt = _WTGraph()
    rc = lib.oracle_window_tree(int(num_samples), int(num_mutations), int(seed), int(window),
                                int(threads or host_threads()), ctypes.byref(wt))
    _check(rc == 0, f"window-tree generator failed ({rc})")
    libc_free = _libc_free()
    off = _owned(wt.down_off, int(wt.num_nodes) + 1, np.uint64, libc_free)
    adj = _owned(wt.down_adj, int(wt.num_edges), np.uint32, libc_free)
    mut = _owned(wt.mut_node, int(wt.num_mutations), np.uint32, libc_free)
    return OracleGraph(num_samples=int(num_samples), ploidy=2, down_off=off, down_adj=adj, mut_node=mut)


_free = None


def _libc_free():
    global _free
    if _free is None:
        f = ctypes.CDLL(None).free
        f.argtypes = [ctypes.c_void_p]
        f.restype = None
        _free = f
    return _free


# ---- independent .grg reader ------------------------------------------------------------------

_MAGIC = 0xE9366C64DDC8C5B0


def _varint(buf: bytes, pos: int):
    value, shift = 0, 0
    while True:
        b = buf[pos]
        pos += 1
        value |= (b & 0x7F) << shift
        if not b & 0x80:
            return value, pos
        shift += 7


def read_grg(path) -> OracleGraph:
    """Parse a .grg file (src/serialize.cpp:815-890 + :697-758) into an OracleGraph."""
    data = Path(path).read_bytes()
    hdr = np.frombuffer(data[:128], dtype=np.uint64)
    h16 = np.frombuffer(data[8:16], dtype=np.uint16)
    _check(int(hdr[0]) == _MAGIC, "Invalid file header")
    vmaj, vmin, ploidy, npops = (int(x) for x in h16)
    nsamp, nmut, nnodes, nedges = (int(x) for x in hdr[2:6])
    flags = int(hdr[8])
    small = vmaj < 5 or (vmaj == 5 and vmin <= 1)
    pos = 128
    edge_bytes = int(np.frombuffer(data[pos:pos + 8], dtype=np.uint64)[0])
    pos += 8
    buckets = data[pos:pos + edge_bytes]
    pos += edge_bytes
    idx_t = np.uint32 if small else np.uint64
    isz = 4 if small else 8
    node_idx = np.frombuffer(data[pos:pos + isz * (nnodes + 1)], dtype=idx_t).astype(np.int64)
    pos += isz * (nnodes + 1)
    off = np.zeros(nnodes + 1, dtype=np.uint64)
    adj = []
    for v in range(nnodes):
        b0, b1 = int(node_idx[v]), int(node_idx[v + 1])
        if b0 < b1:
            cnt, p = _varint(buckets, b0)
            prev = 0
            for _ in range(cnt):
                d, p = _varint(buckets, p)
                prev += d
                adj.append(prev)
        off[v + 1] = len(adj)
    _check(len(adj) == nedges, "Malformed GRG file")
    mut_node = np.frombuffer(data[pos:pos + 4 * nmut], dtype=np.uint32).copy()
    pos += 4 * nmut
    recs = np.frombuffer(data[pos:pos + 24 * nmut], dtype=np.uint8).reshape(-1, 24) if nmut else np.zeros((0, 24))
    pos += 24 * nmut
    for _ in range(int(np.count_nonzero(recs[:, 0] & 1)) if nmut else 0):
        ln, pos = _varint(data, pos)
        pos += ln
    if npops > 0:
        for _ in range(npops):
            ln, pos = _varint(data, pos)
            pos += ln
        pos += 2 * nsamp
    coals = np.frombuffer(data[pos:pos + 4 * (nnodes - nsamp)], dtype=np.uint32).copy()
    pos += 4 * (nnodes - nsamp)
    if flags & 0x1:
        nbytes = int(np.frombuffer(data[pos:pos + 8], dtype=np.uint64)[0])
        pos += 8 + nbytes + (nsamp // ploidy + 1) * isz
    miss = None
    if flags & 0x4:
        miss = np.frombuffer(data[pos:pos + 4 * nmut], dtype=np.uint32).copy()
        pos += 4 * nmut
    return OracleGraph(num_samples=nsamp, ploidy=ploidy, down_off=off, down_adj=np.array(adj, dtype=np.uint32),
                       mut_node=mut_node, miss_node=miss, coals=coals)


def standardized(g: OracleGraph, V: np.ndarray, direction: int, return_scale: bool = False):
    """Float64 products with Z = (X - mu) / sigma from the dense genotype matrix (small graphs only).

    mu_j = count_j / N (haploid), sigma_j = sqrt(mu_j (1 - mu_j)), zero-variance columns set to 0:
    UP -> V @ Z, DOWN -> V @ Z.T.  With return_scale, also the magnitude of the terms the
    algorithm combines (|V| X + |V 1| mu) / sigma for UP, |W| X^T + |W mu| for DOWN: the scale the
    tolerance is relative to."""
    X = g.dense_X().astype(np.float64)
    N = X.shape[0]
    mu = X.sum(axis=0) / N
    var = mu * (1.0 - mu)
    inv = np.where(var > 0, 1.0 / np.sqrt(np.where(var > 0, var, 1.0)), 0.0)
    Z = (X - mu[None, :]) * inv[None, :]
    V64 = V.astype(np.float64)
    out = V64 @ Z if int(direction) == UP else V64 @ Z.T
    if not return_scale:
        return out
    # The algorithm combines V X with the correction (V 1) mu^T (UP), or X W^T with 1 (mu^T W^T)
    # (DOWN, W = V / sigma); its rounding is relative to the magnitudes of those terms.
    aV = np.abs(V64)
    if int(direction) == UP:
        scale = ((aV @ X) + np.abs(V64.sum(axis=1))[:, None] * mu[None, :]) * inv[None, :]
    else:
        W = V64 * inv[None, :]
        scale = np.abs(W) @ X.T + np.abs(W @ mu)[:, None]
    return out, scale
