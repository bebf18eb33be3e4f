"""CPU checks of the cost model's oracle and of the tuner's host logic: the
oracle's FP64 backpropagation equals central finite differences of its
loss (the definition of the gradient the device kernels are checked
against), its Adam loop lowers the loss, and tune_guided / tune_random keep
their budget, never repeat a candidate, skip failing ones and cache
features for later workloads (with a stand-in model, no GPU)."""
import math
import os

import numpy as np
import pytest

from gpufs_gb300 import autotune
from gpufs_gb300 import costmodel as gcm
from oracle import costmodel as cm


def _params(d, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(0, 0.3, cm.n_params(d))


@pytest.mark.parametrize("d,n", [(1, 1), (7, 33), (19, 70)])
def test_oracle_gradient_matches_finite_differences(d, n):
    rng = np.random.default_rng(d * 100 + n)
    X = rng.normal(0, 1, (n, d))
    t = rng.normal(0, 1, n)
    p = _params(d, d + n)
    _, g = cm.loss_grad(p, X, t)
    idx = sorted(set(rng.choice(p.size, min(p.size, 120), replace=False).tolist()) | {0, p.size - 1})
    fd = cm.fd_grad(p, X, t, eps=1e-6, idx=idx)
    for i in idx:
        assert abs(g[i] - fd[i]) <= 1e-6 + 1e-5 * abs(fd[i]), (i, g[i], fd[i])


def test_oracle_adam_lowers_loss():
    rng = np.random.default_rng(5)
    X = rng.uniform(-1, 1, (200, 3))
    t = np.sin(2 * X[:, 0]) + X[:, 1] * X[:, 2]
    p = _params(3, 1) * 0.5
    _, losses = cm.adam_train(p, X, t, 300, 3e-3)
    assert losses[-1] < 0.1 * losses[0]


def test_layout_matches_header_constants():
    assert cm.H == gcm.HIDDEN
    hdr = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                            "gpufs_gb300.h")).read()
    assert "#define GFS_CM_HIDDEN %d" % gcm.HIDDEN in hdr
    assert "#define GFS_CM_MAX_INPUTS %d" % gcm.MAX_INPUTS in hdr


def test_workload_features():
    f = gcm.workload_features([100, 5000, 1 << 20, 1 << 23], op_mix=(0.8, 0.15, 0.05))
    assert f.shape == (4 + 7 + 3,)
    assert f[0] == 2.0  # log2 of 4 files
    assert abs(f[4:11].sum() - 1.0) < 1e-12
    assert list(f[-3:]) == [0.8, 0.15, 0.05]
    p = gcm.param_features({"log_page": 1 << 16, "workers": 8}, ["log_page", "workers"])
    assert list(p) == [16.0, 3.0]


class _LinearModel:
    """Least-squares stand-in with the CostModel fit/predict interface."""

    def __init__(self):
        self.fits = 0

    def fit(self, X, y, steps=0, lr=0.0):
        self.fits += 1
        A = np.c_[X, np.ones(len(X))]
        self.w = np.linalg.lstsq(A, y, rcond=None)[0]

    def predict(self, X):
        return np.c_[X, np.ones(len(X))] @ self.w


def test_guided_and_random_keep_budget_and_skip_failures(tmp_path):
    cands = [{"a": a, "b": b} for a in range(1, 9) for b in range(1, 5)]

    def trial(c):
        if c["a"] == 3:
            raise RuntimeError("candidate fails")
        return math.exp(0.2 * (c["a"] - 6) ** 2 + 0.1 * c["b"])

    feat = lambda c: [c["a"], c["a"] ** 2, c["b"]]  # noqa: E731
    seen = []

    def counted(c):
        seen.append((c["a"], c["b"]))
        return trial(c)

    cache = str(tmp_path / "tune.json")
    m = _LinearModel()
    best, res = autotune.tune_guided(cands, counted, feat, budget=7, n_init=2, seed=3, model=m, key="w1",
                                     cache_path=cache)
    assert len(res) == 7 and len(set(seen)) == 7  # budget kept, no repeats
    assert 4 <= m.fits <= 5  # one fit per trial after the random ones, once two succeeded
    assert best == {"a": 6, "b": 1}  # the quadratic in a is learnable from a, a^2
    assert all(t is None for c, t in res if c["a"] == 3)
    hist = autotune.history_from_cache(cache)
    assert len(hist) == sum(1 for _, t in res if t is not None) and len(hist[0][0]) == 3
    assert autotune.history_from_cache(cache, exclude_key="w1") == []
    rb, rres = autotune.tune_random(cands, trial, budget=5, seed=3)
    assert len(rres) == 5 and len({(c["a"], c["b"]) for c, _ in rres}) == 5
    with pytest.raises(RuntimeError):
        autotune.tune_random([{"a": 3, "b": 1}], trial, budget=1)
