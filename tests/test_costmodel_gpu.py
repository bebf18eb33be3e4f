"""The autotuner's cost model on the GPU: the device forward/backward
kernels give the FP64 oracle's loss, gradient and predictions (FP32
tolerances below), Adam training on the device follows the oracle's
trajectory and is bit-reproducible, and the trained network earns its
place: on a cost surface with a known optimum, the model-guided search
finds far better configurations than seeded random search under the same
trial budget."""
import itertools
import math

import numpy as np
import pytest

from gpufs_gb300 import autotune
from gpufs_gb300.costmodel import CostModel
from oracle import costmodel as cm

pytestmark = pytest.mark.gpu

# FP32 kernels against FP64: relative loss error, and gradient error
# relative to the largest gradient component.
LOSS_RTOL = 2e-5
GRAD_TOL = 2e-4
PRED_TOL = 2e-5


@pytest.mark.parametrize("d,n", [(1, 1), (7, 31), (7, 33), (19, 500), (64, 5000), (13, 9731)])
def test_gradient_and_prediction_match_oracle(built, d, n):
    rng = np.random.default_rng(d * 7 + n)
    X = rng.normal(0, 1, (n, d)).astype(np.float32)
    t = rng.normal(0, 1, n).astype(np.float32)
    with CostModel(d, seed=d + n) as m:
        p = (rng.normal(0, 0.3, m.n_params)).astype(np.float32)
        m.set_params(p)
        assert np.array_equal(m.params(), p)
        loss, g = m.grad(X, t)
        rl, rg = cm.loss_grad(p.astype(np.float64), X.astype(np.float64), t.astype(np.float64))
        assert abs(loss - rl) <= LOSS_RTOL * rl, (loss, rl)
        err = np.abs(g.astype(np.float64) - rg).max() / np.abs(rg).max()
        assert err <= GRAD_TOL, err
        y = m.predict_raw(X)
        ry = cm.forward(p.astype(np.float64), X.astype(np.float64))
        assert np.abs(y - ry).max() <= PRED_TOL * max(1.0, np.abs(ry).max())


def test_training_follows_oracle_and_is_deterministic(built):
    rng = np.random.default_rng(4)
    X = rng.uniform(-1, 1, (700, 5)).astype(np.float32)
    t = (np.sin(2 * X[:, 0]) + X[:, 1] * X[:, 2] - 0.5 * X[:, 3] ** 2).astype(np.float32)
    with CostModel(5, seed=11) as m:
        p0 = m.params()
        losses = m.train(X, t, steps=100, lr=3e-3)
        p1 = m.params()
        _, ref = cm.adam_train(p0.astype(np.float64), X.astype(np.float64), t.astype(np.float64), 100, 3e-3)
        ref = np.asarray(ref)
        assert np.abs(losses - ref).max() <= 2e-3 * ref[0], np.abs(losses - ref).max()
        m.set_params(p0)
        again = m.train(X, t, steps=100, lr=3e-3)
        assert np.array_equal(again, losses) and np.array_equal(m.params(), p1)  # reproducible
        more = m.train(X, t, steps=1500, lr=3e-3)
        assert more[-1] < 0.05 * losses[0]


def test_invalid_arguments(built):
    from gpufs_gb300 import GfsError
    with pytest.raises(ValueError):
        CostModel(0)
    with pytest.raises(ValueError):
        CostModel(65)
    with CostModel(3) as m:
        with pytest.raises(ValueError):
            m.train(np.zeros((4, 2), np.float32), np.zeros(4, np.float32))
        with pytest.raises(GfsError):
            m.train(np.zeros((4, 3), np.float32), np.zeros(4, np.float32), lr=0.0)


# A cost surface with the structure tuning meets: the best page size follows
# the file size, small-file workloads want more host workers, the grid size
# follows the file count, staging depth trades against workers, and writes
# prefer small pages.  Workload: (mean log2 file size, read share, log2 file
# count); candidate: (log2 page, host workers, CTAs per SM, staging depth).
PAGES = list(range(12, 22))
WORKERS = [2, 4, 8, 16, 32]
CTAS = [1, 2, 4, 8]
STAGING = [2, 4, 8, 16]
CANDS = [dict(log_page=p, workers=w, ctas=c, staging=s) for p, w, c, s in itertools.product(PAGES, WORKERS, CTAS,
                                                                                            STAGING)]


def _log_time(wl, c):
    mlog, rf, nf = wl
    best_page = min(21, max(12, mlog - 2))
    best_workers = 1 + 4 * (1 - (mlog - 13) / 11)
    best_ctas = min(3, max(0, (nf - 8) / 3))
    lw = math.log2(c["workers"])
    best_staging = min(4, max(1, 5 - lw))
    return (0.08 * (c["log_page"] - best_page) ** 2 + 0.25 * (lw - best_workers) ** 2
            + 0.15 * (math.log2(c["ctas"]) - best_ctas) ** 2 + 0.1 * (math.log2(c["staging"]) - best_staging) ** 2
            + 0.3 * (1 - rf) * (c["log_page"] - 12) / 9)


def _features(wl, c):
    return np.array([wl[0], wl[1], wl[2], c["log_page"], math.log2(c["workers"]), math.log2(c["ctas"]),
                     math.log2(c["staging"])])


def test_guided_search_beats_random_search(built):
    rng = np.random.default_rng(1)

    def workload():
        return (rng.uniform(13, 24), rng.uniform(0.5, 1), rng.uniform(8, 17))

    history = []  # 40 measured trials on each of 8 earlier workloads
    for _ in range(8):
        wl = workload()
        for i in rng.choice(len(CANDS), 40, replace=False):
            history.append((_features(wl, CANDS[i]), math.exp(_log_time(wl, CANDS[i]) + rng.normal(0, 0.02))))
    budget = 8
    regret_guided, regret_random = [], []
    with CostModel(7, seed=5) as model:
        for k in range(12):
            wl = workload()
            best = min(_log_time(wl, c) for c in CANDS)
            noise = np.random.default_rng(100 + k)

            def trial(c):
                return math.exp(_log_time(wl, c) + noise.normal(0, 0.02))

            g, res = autotune.tune_guided(CANDS, trial, lambda c: _features(wl, c), budget, history=history, seed=k,
                                          model=model, fit_steps=300)
            assert len(res) == budget
            r, _ = autotune.tune_random(CANDS, trial, budget, seed=k)
            regret_guided.append(math.exp(_log_time(wl, g) - best) - 1)
            regret_random.append(math.exp(_log_time(wl, r) - best) - 1)
    mg, mr = float(np.mean(regret_guided)), float(np.mean(regret_random))
    print("mean regret over 12 workloads, %d trials of %d candidates: guided %.3f, random %.3f"
          % (budget, len(CANDS), mg, mr))
    assert mg < 0.1 and mg < 0.25 * mr, (regret_guided, regret_random)
