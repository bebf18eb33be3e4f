"""Autotuner for session parameters (page size, host workers, ring depth,
staging depth, grid size): times short trial runs of the real workload on
each candidate and keeps the fastest.

A tuning result is cached per workload signature (a string the caller
builds from what determines performance: file count and size histogram,
operation mix, device) in an optional JSON file, so a later run of the same
workload skips the search.  A candidate that fails is skipped, not chosen.

Three searches:
  tune         every candidate runs the caller's trial (exhaustive);
  tune_random  a fixed budget of trials on seeded random candidates;
  tune_guided  the same budget, chosen by the learned cost model
               (gpufs_gb300.costmodel): after a few random trials, the model
               is trained on the device on every measurement so far -- this
               workload's and those cached for other workloads -- and the
               candidate it predicts fastest runs next.
"""
import json
import math
import os
import time

import numpy as np


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


def _run_trial(trial, cfg, repeats):
    try:
        ts = []
        for _ in range(max(1, repeats)):
            t0 = time.perf_counter()
            r = trial(cfg)
            ts.append(r if r is not None else time.perf_counter() - t0)
        return min(ts)
    except Exception:  # noqa: BLE001 -- a failing candidate is skipped
        return None


def history_from_cache(cache_path, exclude_key=None):
    """(features, seconds) of every trial cached with features, except those
    of exclude_key."""
    out = []
    for k, rec in _load(cache_path).items():
        if k == exclude_key:
            continue
        for tr in rec.get("tried", []):
            if tr.get("features") is not None and tr.get("seconds") is not None:
                out.append((tr["features"], tr["seconds"]))
    return out


def _finish(results, key, cache_path, feats=None):
    ok = [(c, t) for c, t in results if t is not None]
    if not ok:
        raise RuntimeError("every candidate failed")
    best, best_t = min(ok, key=lambda x: x[1])
    if key is not None and cache_path:
        table = _load(cache_path)
        tried = []
        for i, (c, t) in enumerate(results):
            e = {"cfg": c, "seconds": t}
            if feats is not None:
                e["features"] = [float(v) for v in feats[i]]
            tried.append(e)
        table[key] = {"best": best, "seconds": best_t, "tried": tried}
        _store(cache_path, table)
    return best, results


def tune_random(candidates, trial, budget, seed=0, repeats=1):
    """Seeded random search: `budget` distinct candidates, fastest kept."""
    import random
    if not candidates:
        raise ValueError("no candidates")
    order = list(range(len(candidates)))
    random.Random(seed).shuffle(order)
    results = [(candidates[i], _run_trial(trial, candidates[i], repeats)) for i in order[:budget]]
    return _finish(results, None, None)


def tune_guided(candidates, trial, featurize, budget, history=(), n_init=2, seed=0, model=None, fit_steps=400,
                lr=3e-3, key=None, cache_path=None, repeats=1, device=0):
    """Model-guided search under a trial budget.

    featurize(cfg) -> 1-D feature vector of this workload joined with cfg.
    history: (features, seconds) measured on other workloads; with
        cache_path, every cached trial of another key is added.
    The first n_init trials are seeded random picks; each later trial runs
    the untried candidate with the lowest predicted log time.
    Returns (best_cfg, results) like tune; trials are cached with their
    features under key.
    """
    import random
    if not candidates:
        raise ValueError("no candidates")
    feats = np.asarray([featurize(c) for c in candidates], dtype=np.float64)
    hist = list(history)
    if cache_path:
        hist += history_from_cache(cache_path, exclude_key=key)
    hx = [np.asarray(f, dtype=np.float64) for f, _ in hist]
    hy = [math.log(max(t, 1e-12)) for _, t in hist]
    own = None
    if model is None:
        from .costmodel import CostModel
        model = own = CostModel(feats.shape[1], device=device, seed=seed)
    order = list(range(len(candidates)))
    random.Random(seed).shuffle(order)
    runs = []  # (candidate index, seconds or None)
    try:
        while len(runs) < min(budget, len(candidates)):
            done = {i for i, _ in runs}
            left = [i for i in order if i not in done]
            good = [(i, t) for i, t in runs if t is not None and t > 0]
            idx = left[0]
            if len(runs) >= n_init and len(hy) + len(good) >= 2:
                X = np.asarray(hx + [feats[i] for i, _ in good], dtype=np.float64)
                y = np.asarray(hy + [math.log(t) for _, t in good], dtype=np.float64)
                model.fit(X, y, steps=fit_steps, lr=lr)
                idx = left[int(np.argmin(model.predict(feats[left])))]
            runs.append((idx, _run_trial(trial, candidates[idx], repeats)))
    finally:
        if own is not None:
            own.close()
    return _finish([(candidates[i], t) for i, t in runs], key, cache_path, [feats[i] for i, _ in runs])
