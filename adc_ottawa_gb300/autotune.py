"""Project autotuner for the sigma kernels' launch shape, with a JSON cache.

The tuned quantities are the pass-1 work-item size (rows of one slab a warp
processes before flushing its register accumulators) and the number of
vector columns per pass (register tile width).  Timing runs in the library
(adcgpu_sigma_autotune, CUDA events on the context's stream); this module
only keys, stores and re-applies the winners.
"""
from __future__ import annotations

import ctypes as C
import json
import os

from ._native import lib

DEFAULT_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "autotune.json")


def _key(g, m: int, precision: int) -> str:
    return f"no{g.nocc}-nv{g.nvirt}-p{precision}-m{m}"


def _load(path: str) -> dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def tune(g, m: int, precision: int, cache: str | None = DEFAULT_CACHE, force: bool = False) -> dict:
    """Tune (or re-apply the cached) launch shape of g's sigma product for
    blocks of m columns.  Returns {"chunk", "mc", "ms", "cached"}."""
    path = cache or DEFAULT_CACHE
    db = _load(path)
    k = _key(g, m, precision)
    if not force and k in db:
        e = db[k]
        mc64 = e["mc"] if precision == 0 else 2
        mc32 = e["mc"] if precision != 0 else 4
        st = lib().adcgpu_sigma_set_shape(g._h, e["chunk"], mc64, mc32)
        g._check(st, "sigma_set_shape")
        return {**e, "cached": True}
    ch, mc, ms = C.c_int(0), C.c_int(0), C.c_double(0.0)
    st = lib().adcgpu_sigma_autotune(g._h, m, C.byref(ch), C.byref(mc), C.byref(ms))
    g._check(st, "sigma_autotune")
    e = {"chunk": ch.value, "mc": mc.value, "ms": ms.value}
    db[k] = e
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            json.dump(db, f, indent=1)
    except OSError:
        pass
    return {**e, "cached": False}
