"""Autotuner for session parameters (page size, host workers, ring depth,
staging depth, grid size): times short trial runs of the real workload on
each candidate and keeps the fastest.

A tuning result is cached per workload signature (a string the caller
builds from what determines performance: file count and size histogram,
operation mix, device) in an optional JSON file, so a later run of the same
workload skips the search.  The search itself is plain measurement: every
candidate runs the caller's trial, and a candidate that fails is skipped,
not chosen.
"""
import json
import os
import time


def signature(**parts):
    """Stable string key of a workload description."""
    return json.dumps(parts, sort_keys=True, separators=(",", ":"))


def _load(path):
    if not path or not os.path.exists(path):
        return {}
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path, table):
    if not path:
        return
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def tune(candidates, trial, key=None, cache_path=None, repeats=1):
    """Pick the candidate whose trial runs fastest.

    candidates: list of dicts (session/launch parameters).
    trial(cfg) -> seconds for one representative run (it may return its own
        device time; wall time is used when it returns None).
    Returns (best_cfg, results) where results lists (cfg, seconds or None).
    With key and cache_path, a cached choice for key is returned without
    running anything (results is then empty), and a new choice is stored.
    """
    if not candidates:
        raise ValueError("no candidates")
    table = _load(cache_path) if key is not None else {}
    if key is not None and key in table:
        cached = table[key]["best"]
        for c in candidates:
            if c == cached:
                return c, []
    results = []
    best, best_t = None, None
    for cfg in candidates:
        t = None
        try:
            ts = []
            for _ in range(max(1, repeats)):
                t0 = time.perf_counter()
                r = trial(cfg)
                ts.append(r if r is not None else time.perf_counter() - t0)
            t = min(ts)
        except Exception:  # noqa: BLE001 -- a failing candidate is skipped
            t = None
        results.append((cfg, t))
        if t is not None and (best_t is None or t < best_t):
            best, best_t = cfg, t
    if best is None:
        raise RuntimeError("every candidate failed")
    if key is not None and cache_path:
        table[key] = {"best": best, "seconds": best_t,
                      "tried": [{"cfg": c, "seconds": s} for c, s in results]}
        _store(cache_path, table)
    return best, results
