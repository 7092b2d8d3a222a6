"""Autotuner for the packed layout of one workload.

The packer's knobs decide how a batch maps onto the GPU:

  target_ops  product + finalize operations per row a task aims for
              (families per task, hence CTAs per launch and row width)
  target_j    iterations per row a lane program aims for (lanes per task)
  root_group  root tasks take target_ops x root_group operations (all split
              levels together): how many families share a root task
  heavy_ops   operations per row above which a non-root task gets 256
              threads instead of 128
  heavy_c<i>  the same threshold for size class i alone (0 = heavy_ops):
              the CTA shape of each size bucket
  classes     which clade-count bounds split the families into size
              classes (an index into CLASS_BOUNDS; each class is packed and
              launched on its own, its launches sized for its tasks)
  persistent  1: one persistent launch per pass instead of the level
              launches (WG_BATCH_PERSISTENT), with persist_ctas CTAs per SM
  adj_overlap 2: each size class's adjoint follows its own forward at the
              class's stream priority; 1 (3): at the lowest (highest)
              priority; 0: after every class's forward (WG_ADJ_OVERLAP)
  level_j     iterations per same-row level a root task's level programs
              aim for (levels within one warp synchronize that warp only)
  comb_warp   forward split clades of at least this many partial sums are
              combined by a warp each (0: by one thread each)

``tune(wm, ccds)`` builds the batch under candidate settings, times a few
evaluations of each on the device (CUDA events around the launch sequence,
the same clock as ``bench.py``'s ``value``) and keeps the fastest, by
coordinate descent from the library's defaults: each knob in turn tries its
neighbours with the others fixed, and a move is kept only if it is faster by
more than ``min_gain``.  The result is the best setting and its batch, ready
for evaluations.  Every setting gives the same log-likelihood and gradient
to rounding; only the layout and the time change.

The knobs reach the packer through environment variables (WG_PACK_TARGET_OPS,
WG_PACK_TARGET_J, WG_PACK_ROOT_GROUP, WG_PACK_HEAVY_OPS, WG_PACK_LEVEL_J,
WG_PACK_COMB_WARP, ...), set only while a candidate batch is built.
"""
from __future__ import annotations

import contextlib
import os
import threading
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _native as N

# size-class bounds (clade counts) the ``classes`` knob chooses from; the
# first is the library's default
CLASS_BOUNDS: Tuple[Tuple[int, ...], ...] = (
    (192, 512, 1536),
    (128, 256, 512, 1024, 1536),
    (128, 512, 1536),
    (64, 128, 256, 512, 1024, 1536),
    (256, 1024),
    (),
)
N_CLASSES = max(len(b) for b in CLASS_BOUNDS) + 1

DEFAULTS: Dict[str, int] = {"target_ops": 480, "target_j": 3, "root_group": 16, "heavy_ops": 1024,
                            **{f"heavy_c{i}": 0 for i in range(N_CLASSES)},
                            "classes": 0, "persistent": 0, "persist_ctas": 3, "adj_overlap": 2, "level_j": 3,
                            "comb_warp": 24}
NEIGHBOURS: Dict[str, Tuple[int, ...]] = {
    "target_ops": (240, 320, 480, 720, 960),
    "target_j": (2, 3, 4, 5),
    "root_group": (4, 8, 16, 32),
    "heavy_ops": (512, 1024, 2048),
    **{f"heavy_c{i}": (0, 256, 512, 2048, 1 << 20) for i in range(N_CLASSES)},
    "classes": tuple(range(len(CLASS_BOUNDS))),
    "persistent": (0, 1),
    "adj_overlap": (0, 1, 2, 3),
    "level_j": (2, 3, 4),
    "comb_warp": (0, 16, 24, 48),
}
_ENV = {"target_ops": "WG_PACK_TARGET_OPS", "target_j": "WG_PACK_TARGET_J", "root_group": "WG_PACK_ROOT_GROUP",
        "heavy_ops": "WG_PACK_HEAVY_OPS", **{f"heavy_c{i}": f"WG_PACK_HEAVY_OPS_C{i}" for i in range(N_CLASSES)},
        "classes": "WG_CLASS_BOUNDS", "persistent": None, "persist_ctas": "WG_PERSIST_CTAS",
        "adj_overlap": "WG_ADJ_OVERLAP", "level_j": "WG_PACK_LEVEL_J", "comb_warp": "WG_PACK_COMB_WARP"}


def _env_value(knob: str, v: int):
    """The environment string of a knob's value (None: unset)."""
    if knob == "classes":
        b = CLASS_BOUNDS[int(v)]
        return ",".join(str(x) for x in b) if b else "1073741823"
    if knob.startswith("heavy_c") and int(v) == 0:
        return None  # the class follows heavy_ops
    return str(int(v))


def shapes(setting: Dict[str, int]) -> List[Dict[str, object]]:
    """Per size class of a setting: its clade-count range and the operations
    per row above which its non-root tasks take 256-thread CTAs (root tasks
    always take 128), or the persistent launch's single class."""
    if setting.get("persistent"):
        return [{"clades": (1, None), "threads": 128, "layout": "persistent",
                 "ctas_per_sm": setting.get("persist_ctas", 3)}]
    b = CLASS_BOUNDS[setting.get("classes", 0)]
    out, lo = [], 1
    for i, hi in enumerate(list(b) + [None]):
        h = setting.get(f"heavy_c{i}", 0) or setting.get("heavy_ops", 1024)
        out.append({"clades": (lo, hi), "threads": (128, 256), "heavy_ops": h, "layout": "levels"})
        lo = (hi or 0) + 1
    return out
_env_lock = threading.RLock()  # nested settings restore in order


@contextlib.contextmanager
def packing(setting: Dict[str, int]):
    """Batches created inside use the given packer knobs.  The knobs are
    process-wide environment variables: a batch another thread creates
    meanwhile packs with them too."""
    with _env_lock:
        old = {k: os.environ.get(v) for k, v in _ENV.items() if v is not None}
        old.update({k: None for k, v in _ENV.items() if v is None})
        try:
            for k, v in setting.items():
                if k not in _ENV:
                    raise KeyError(f"unknown packing knob {k!r}")
                if _ENV[k] is None:
                    continue  # a batch flag, not an environment knob
                e = _env_value(k, v)
                if e is None:
                    os.environ.pop(_ENV[k], None)
                else:
                    os.environ[_ENV[k]] = e
            yield
        finally:
            for k, v in old.items():
                if _ENV[k] is None:
                    continue
                if v is None:
                    os.environ.pop(_ENV[k], None)
                else:
                    os.environ[_ENV[k]] = v


def _descend(measure: Callable[[Dict[str, int]], float], start: Dict[str, int],
             neighbours: Dict[str, Sequence[int]], min_gain: float, rounds: int) -> Tuple[Dict[str, int], float, List]:
    best = dict(start)
    best_t = measure(best)
    log = [(dict(best), best_t)]
    seen = {tuple(sorted(best.items())): best_t}
    for _ in range(rounds):
        moved = False
        for knob, values in neighbours.items():
            for v in values:
                if v == best[knob]:
                    continue
                cand = dict(best)
                cand[knob] = v
                key = tuple(sorted(cand.items()))
                if key not in seen:
                    seen[key] = measure(cand)
                    log.append((dict(cand), seen[key]))
                if seen[key] < best_t * (1.0 - min_gain):
                    best, best_t, moved = cand, seen[key], True
        if not moved:
            break
    return best, best_t, log


def tune(wm, ccds: Sequence, grad: bool = True, steps: int = 5, warmup: int = 2, ctx=None,
         neighbours: Optional[Dict[str, Sequence[int]]] = None, min_gain: float = 0.01, rounds: int = 2,
         measure: Optional[Callable[[Dict[str, int]], float]] = None):
    """Fastest packing of ``ccds`` for ``wm`` (gradient evaluations when
    ``grad``).  Returns ``(setting, batch, log)``: the knob values, the batch
    built with them (None when ``measure`` is given), and every
    (setting, ms per evaluation) tried.  ``measure`` replaces the device
    timing (a function of the setting returning milliseconds).  Event timing
    stays enabled on the context afterwards (``wg_ctx_set_timing``)."""
    from .core import Batch, default_context

    neighbours = dict(NEIGHBOURS if neighbours is None else neighbours)
    start = {k: v for k, v in DEFAULTS.items() if k in neighbours or k in ("heavy_ops", "persist_ctas")}
    if measure is not None:
        best, _, log = _descend(measure, start, neighbours, min_gain, rounds)
        return best, None, log
    ctx = ctx or default_context()
    L = N.lib()
    N.check(L.wg_ctx_set_timing(ctx.h, 1))
    f, a, r = N.C.c_float(), N.C.c_float(), N.C.c_float()
    kept = {"key": None, "ms": float("inf"), "batch": None}  # the fastest batch so far only

    def device_ms(setting):
        with packing(setting):
            b = Batch(wm, ccds, grad=grad, ctx=ctx, persistent=bool(setting.get("persistent", 0)))
        times = []
        for i in range(warmup + steps):
            if grad:
                b.grad_nodes(wm)
                N.check(L.wg_ctx_timings(ctx.h, N.C.byref(f), N.C.byref(a), N.C.byref(r)))
                t = f.value + a.value + r.value
            else:
                b.logpdf(wm)
                N.check(L.wg_ctx_timings(ctx.h, N.C.byref(f), None, None))
                t = f.value
            if i >= warmup:
                times.append(t)
        ms = float(np.median(times))
        if ms < kept["ms"]:
            kept.update(key=tuple(sorted(setting.items())), ms=ms, batch=b)
        return ms

    best, _, log = _descend(device_ms, start, neighbours, min_gain, rounds)
    if kept["key"] != tuple(sorted(best.items())):
        kept["batch"] = None
        with packing(best):
            kept["batch"] = Batch(wm, ccds, grad=grad, ctx=ctx, persistent=bool(best.get("persistent", 0)))
    return best, kept["batch"], log


def report(best: Dict[str, int], log: List) -> Dict[str, object]:
    """The tuned setting against the library's defaults: per size class its
    clade range and CTA shape (``shapes``), the milliseconds per evaluation
    of the defaults (the first setting timed) and of the best setting."""
    default_ms = log[0][1]
    best_ms = min(ms for s, ms in log if all(s.get(k) == v for k, v in best.items()))
    return {"setting": dict(best), "shapes": shapes(best), "default_shapes": shapes(log[0][0]),
            "default_ms": default_ms, "best_ms": best_ms, "speedup": default_ms / best_ms,
            "candidates": len(log)}
