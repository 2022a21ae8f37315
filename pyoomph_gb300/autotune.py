"""Launch-shape autotuner for the element kernels.

The generated kernels have one free launch parameter that decides their
occupancy: the number of elements a block evaluates (EPB; the block runs EPB
x knots threads in phase A and EPB x rows threads in phase B, and holds EPB
elements' data in shared memory).  ``codegen._launch_shape`` picks it by a
waste heuristic; this module measures instead: it builds the problem once
per candidate, times the full assembly with CUDA events on the launching
stream, and keeps the fastest.  Results are cached per kernel family in a
JSON file so that a later run reuses them without timing again.
"""
from __future__ import annotations

import json
import os
import threading
from typing import Callable, Dict, Iterable, List, Optional, Tuple

CACHE_PATH = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "_build", "autotune.json")
_lock = threading.Lock()


def _load(path: str) -> Dict[str, dict]:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def cached(key: str, path: str = CACHE_PATH) -> Optional[dict]:
    """The stored tuning result of a kernel family, or None."""
    with _lock:
        return _load(path).get(key)


def store(key: str, result: dict, path: str = CACHE_PATH) -> None:
    with _lock:
        d = _load(path)
        d[key] = result
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


def time_assembly(P, steps: int = 20, warmup: int = 3) -> float:
    """Mean milliseconds of one full R+J assembly of an initialised problem
    (CUDA events on the current stream, inputs resident)."""
    import torch
    for _ in range(warmup):
        P.assemble_device(with_jacobian=True)
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(steps):
        P.assemble_device(with_jacobian=True)
    e1.record(st)
    torch.cuda.synchronize()
    P.check()
    return e0.elapsed_time(e1) / steps


def tune(key: str, factory: Callable[[object], object], candidates: Iterable, steps: int = 20,
         warmup: int = 3, use_cache: bool = True, path: str = CACHE_PATH) -> Tuple[object, Dict[str, float]]:
    """Time ``factory(c)`` (an initialised problem) for every candidate c;
    return the fastest candidate and the table of ms per assembly.  A
    candidate whose kernel does not fit (launch shape, shared memory) is
    skipped."""
    if use_cache:
        hit = cached(key, path)
        if hit is not None:
            return hit["best"], hit["ms"]
    table: Dict[str, float] = {}
    best, best_ms = None, float("inf")
    for c in candidates:
        try:
            P = factory(c)
        except ValueError:
            continue
        ms = time_assembly(P, steps, warmup)
        table[str(c)] = ms
        if ms < best_ms:
            best, best_ms = c, ms
        del P
    if best is None:
        raise ValueError(f"no candidate launch shape fits for {key}")
    store(key, {"best": best, "ms": table}, path)
    return best, table


def epb_candidates(nq: int, nloc: int, max_threads: int = 1024) -> List[int]:
    """Elements-per-block values whose phase-B thread count fits a block."""
    out = []
    for e in (1, 2, 4, 6, 8, 12, 16, 20, 24, 32, 40, 48, 64):
        if max(e * nq, e * nloc) <= max_threads:
            out.append(e)
    return out
