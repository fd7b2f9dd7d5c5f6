"""Seeded matmul cases shared by the golden-fixture generator and the tests.

Each case is (name, (V, direction, kwargs)); direction 1 = DOWN, 2 = UP (visitor.h:26).  Inputs
are regenerated from fixed seeds, so fixtures only store the reference outputs.
"""
from __future__ import annotations

import numpy as np

DOWN, UP = 1, 2


def _rng(name: str) -> np.random.Generator:
    return np.random.default_rng(abs(hash_name(name)) % (2 ** 32))


def hash_name(name: str) -> int:
    h = 1469598103934665603
    for ch in name.encode():
        h = ((h ^ ch) * 1099511628211) % (2 ** 64)
    return h


def _values(rng, dtype, shape):
    dt = np.dtype(dtype)
    if dt == np.bool_:
        return rng.random(shape) < 0.5
    if dt.kind == "f":
        return rng.standard_normal(shape).astype(dt)
    info = np.iinfo(dt)
    lo, hi = max(info.min, -100), min(info.max, 100)
    return rng.integers(lo, hi + 1, size=shape).astype(dt)


def cases_for(N: int, M: int, n: int, ploidy: int, has_miss: bool = False, profile: str = "full"):
    """Yield the cases for a graph with N samples, M mutations, n nodes."""
    indiv = N // ploidy
    out = []

    def add(name, dtype, K, direction, **kw):
        rng = _rng(name)
        cols = (indiv if kw.get("by_individual") else N) if direction == UP else M
        if kw.get("ones"):
            kw.pop("ones")
            V = np.ones((K, cols), dtype=dtype)
        else:
            V = _values(rng, dtype, (K, cols))
        if kw.get("init") == "vector":
            kw["init"] = _values(rng, dtype, (K,))
        elif kw.get("init") == "matrix":
            kw["init"] = _values(rng, dtype, (K, n))
        if kw.get("miss") == "input":
            kw["miss"] = _values(rng, dtype, (K, M))
        out.append((name, (V, direction, kw)))

    # allele counts and single float64 vectors: DOWN int32 ones, DOWN/UP float64 N(0,1), K=1
    add("down_i32_ones_k1", np.int32, 1, DOWN, ones=True)
    add("up_i32_ones_k1", np.int32, 1, UP, ones=True)
    add("down_f64_k1", np.float64, 1, DOWN)
    add("up_f64_k1", np.float64, 1, UP)
    if profile == "k1":
        return out
    if has_miss:
        add("down_f64_miss_k2", np.float64, 2, DOWN, miss="input")
        add("up_f64_miss_k2", np.float64, 2, UP, miss="input")
        add("down_i32_miss_k1", np.int32, 1, DOWN, miss="input")
        add("up_i32_miss_k1", np.int32, 1, UP, miss="input", ones=True)
        add("up_bool_miss_k3", np.bool_, 3, UP, miss="input")
        if profile == "miss":
            return out
    add("down_f64_k3", np.float64, 3, DOWN)
    add("up_f64_k3", np.float64, 3, UP)
    add("down_f32_k4", np.float32, 4, DOWN)
    add("up_f32_k2", np.float32, 2, UP)
    add("down_i32_k2", np.int32, 2, DOWN)
    add("up_i32_k3", np.int32, 3, UP)
    add("down_i64_k2", np.int64, 2, DOWN)
    add("up_i64_k1", np.int64, 1, UP)
    add("up_i8_k3", np.int8, 3, UP)
    add("down_i16_k2", np.int16, 2, DOWN)
    add("up_u8_k2", np.uint8, 2, UP)
    add("down_u16_k1", np.uint16, 1, DOWN)
    add("up_u32_k2", np.uint32, 2, UP)
    add("down_u64_k2", np.uint64, 2, DOWN)
    add("up_bool_k5", np.bool_, 5, UP)
    add("down_bool_k33", np.bool_, 33, DOWN)
    add("up_f64_byind_k2", np.float64, 2, UP, by_individual=True)
    add("down_f64_byind_k2", np.float64, 2, DOWN, by_individual=True)
    add("down_i32_byind_k1", np.int32, 1, DOWN, by_individual=True, ones=True)
    add("up_f64_emit_k1", np.float64, 1, UP, emit_all_nodes=True)
    add("down_i32_emit_k2", np.int32, 2, DOWN, emit_all_nodes=True)
    add("up_f64_xtx_k2", np.float64, 2, UP, init="xtx", ones=True)
    add("down_i32_xtx_k1", np.int32, 1, DOWN, init="xtx")
    add("up_f64_initvec_k2", np.float64, 2, UP, init="vector")
    add("down_i64_initvec_k2", np.int64, 2, DOWN, init="vector")
    add("up_i32_initmat_k2", np.int32, 2, UP, init="matrix")
    add("down_f64_initmat_k1", np.float64, 1, DOWN, init="matrix")
    return out
