"""Autotuner for the FP32 tiled gridder/degridder.

The tunables are the grid tile edge T, threads per CTA, the footprint piece
cap (the largest period) and the work granularity (bundles per resident CTA,
i.e. how many visibilities one CTA takes at a time).  The best choice depends
on the support sizes and on how densely visibilities fall on the grid, so
results are keyed on both:

    key = (largest support, taps-weighted mean support bucket,
           visibilities per occupied 32x32 tile bucket, grid edge bucket)

tune() times grid + degrid (CUDA events, median of `reps`) for every
candidate on the caller's own data and remembers the winner in a JSON cache
(RC_GB300_TUNE_CACHE, default ~/.cache/rc_gb300/autotune.json).  best()
returns a cached choice or the defaults.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

DEFAULT = {"tile": 24, "threads": 256, "period_cap": 40, "bundles_per_cta": 4}

CANDIDATES = [
    {"tile": t, "threads": nt, "period_cap": cap, "bundles_per_cta": b}
    for t in (16, 24, 32)
    for nt in (256, 512)
    for cap in (24, 32, 40)
    for b in (2, 4, 8)
]


def cache_path():
    return os.environ.get("RC_GB300_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "rc_gb300",
                                       "autotune.json"))


def _bucket(x, base=2.0):
    return int(round(math.log(max(x, 1e-9), base)))


def signature(supports, plane_counts, kept, tiles_occupied, grid_edge):
    """Workload key from the per-plane supports and visibility counts."""
    s = np.asarray(supports, np.float64)
    c = np.asarray(plane_counts, np.float64)
    taps = float((c * s * s).sum())
    mean_s = math.sqrt(taps / max(c.sum(), 1.0))
    density = kept / max(tiles_occupied, 1)
    return (f"smax{int(s.max())}-s{_bucket(mean_s, 1.25)}-d{_bucket(density)}"
            f"-g{_bucket(grid_edge)}")


def _load():
    try:
        return json.load(open(cache_path()))
    except Exception:
        return {}


def _store(db):
    p = cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + ".tmp"
        json.dump(db, open(tmp, "w"), indent=1, sort_keys=True)
        os.replace(tmp, p)
    except OSError:
        pass


def best(key):
    return dict(_load().get(key, {}).get("params", DEFAULT))


def plan_signature(plan, plane_counts):
    st = plan.stats()
    # occupied tiles counted on the 32x32 tiling, whatever the plan's own tile
    occ = st["tiles"] * (st["tile"] / 32.0) ** 2
    return signature(plan.supports, plane_counts, st["kept"], occ, max(plan.grid_shape))


def tune(make_plan, vis, gcf, grid, candidates=None, reps=3, key=None, log=None):
    """Time every candidate: make_plan(**params) -> engine.Plan.  Returns
    (best params, best ms, table).  Stores the winner under `key` if given."""
    import torch

    cands = candidates or CANDIDATES
    s = torch.cuda.current_stream()
    table = []
    best_p, best_t = None, float("inf")
    pred = None
    for p in cands:
        try:
            plan = make_plan(**p)
        except Exception as e:  # e.g. a tile/period that does not fit shared memory
            table.append((p, None, str(e)[:80]))
            continue
        if pred is None or pred.numel() != plan.n:
            pred = torch.empty(plan.n, dtype=torch.complex64, device=grid.device)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ts = []
        for r in range(reps + 1):
            grid.zero_()
            ev[0].record(s)
            plan.grid(vis, gcf, grid)
            plan.degrid(gcf, grid, out=pred)
            ev[1].record(s)
            ev[1].synchronize()
            if r:
                ts.append(ev[0].elapsed_time(ev[1]))
        t = float(np.median(ts))
        table.append((p, t, ""))
        if log:
            log(f"{p} {t:.3f} ms")
        if t < best_t:
            best_p, best_t = p, t
        plan.close()
    if key is not None and best_p is not None:
        db = _load()
        db[key] = {"params": best_p, "ms": best_t}
        _store(db)
    return best_p, best_t, table
