"""The autotuner's learned cost model: a small network trained on the GPU by
the library's own kernels (C ABI gfs_cm_*, csrc/gfs_costmodel.cu) that
predicts a run's log time from a feature vector -- workload features
(file-size histogram, op mix, file count, bytes) joined with session
parameters (page size, host workers, grid, staging depth).

It never touches file bytes: the tuner only uses it to choose which
candidate configuration to try next, so results stay exact whatever it
predicts.
"""
import ctypes
import math

import numpy as np

from . import _check, lib

HIDDEN = 64      # GFS_CM_HIDDEN
MAX_INPUTS = 64  # GFS_CM_MAX_INPUTS


def _fp(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class CostModel:
    """n_in -> 64 -> 64 -> 1 tanh network on `device`, seeded weights.

    grad/train/predict_raw work on the values given; fit/predict
    standardise features and targets with the statistics of the fitted
    set (what the tuner uses)."""

    def __init__(self, n_in, device=0, seed=0):
        if not 1 <= n_in <= MAX_INPUTS:
            raise ValueError("n_in must be 1..%d" % MAX_INPUTS)
        self.n_in = n_in
        h = ctypes.c_void_p()
        _check(lib().gfs_cm_create(n_in, device, seed, ctypes.byref(h)), "gfs_cm_create")
        self._h = h
        self._init = self.params()
        self._mx = self._sx = None
        self._my, self._sy = 0.0, 1.0

    @property
    def n_params(self):
        return int(lib().gfs_cm_n_params(self._h))

    def params(self):
        p = np.empty(self.n_params, dtype=np.float32)
        _check(lib().gfs_cm_get_params(self._h, _fp(p)), "gfs_cm_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.n_params:
            raise ValueError("expected %d parameters" % self.n_params)
        _check(lib().gfs_cm_set_params(self._h, _fp(p)), "gfs_cm_set_params")

    def _data(self, X, y):
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        if X.ndim != 2 or X.shape[1] != self.n_in or y.shape != (X.shape[0],) or X.shape[0] < 1:
            raise ValueError("X must be [n, %d] and y [n]" % self.n_in)
        _check(lib().gfs_cm_set_data(self._h, _fp(X), _fp(y), X.shape[0]), "gfs_cm_set_data")

    def grad(self, X, y):
        """(loss, gradient) of the mean squared error at the current parameters."""
        self._data(X, y)
        g = np.empty(self.n_params, dtype=np.float32)
        loss = ctypes.c_float()
        _check(lib().gfs_cm_grad(self._h, _fp(g), ctypes.byref(loss)), "gfs_cm_grad")
        return float(loss.value), g

    def train(self, X, y, steps=300, lr=3e-3):
        """Full-batch Adam on the device; returns the loss before each step."""
        self._data(X, y)
        losses = np.empty(max(1, steps), dtype=np.float32)
        _check(lib().gfs_cm_train(self._h, steps, ctypes.c_float(lr), _fp(losses)), "gfs_cm_train")
        return losses[:steps]

    def predict_raw(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        if X.ndim != 2 or X.shape[1] != self.n_in:
            raise ValueError("X must be [n, %d]" % self.n_in)
        y = np.empty(X.shape[0], dtype=np.float32)
        if X.shape[0]:
            _check(lib().gfs_cm_predict(self._h, _fp(X), X.shape[0], _fp(y)), "gfs_cm_predict")
        return y

    def fit(self, X, y, steps=400, lr=3e-3):
        """Train from the seeded initial weights on standardised data."""
        X = np.asarray(X, dtype=np.float64)
        y = np.asarray(y, dtype=np.float64)
        self._mx = X.mean(0)
        self._sx = np.maximum(X.std(0), 1e-6)
        self._my = float(y.mean())
        self._sy = float(max(y.std(), 1e-6))
        self.set_params(self._init)
        return self.train((X - self._mx) / self._sx, (y - self._my) / self._sy, steps, lr)

    def predict(self, X):
        X = np.asarray(X, dtype=np.float64)
        if self._mx is None:
            raise RuntimeError("fit() first")
        return self.predict_raw((X - self._mx) / self._sx) * self._sy + self._my

    def close(self):
        if self._h:
            lib().gfs_cm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 -- interpreter shutdown
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


SIZE_BUCKETS = (12, 14, 16, 18, 20, 22)  # log2 size edges of the histogram


def workload_features(sizes, op_mix=(1.0, 0.0, 0.0)):
    """Workload part of a feature vector: log2 file count, log2 total bytes,
    mean and spread of log2 size, the share of files in each log2-size
    bucket (below 4 KiB, 4-16 KiB, ..., 1-4 MiB, above), and the op mix
    (read, grep, write shares)."""
    s = np.maximum(np.asarray(sizes, dtype=np.float64), 1.0)
    ls = np.log2(s)
    hist = np.histogram(ls, bins=(-1.0,) + SIZE_BUCKETS + (64.0,))[0] / max(1, s.size)
    return np.concatenate([[math.log2(max(1, s.size)), math.log2(max(1.0, s.sum())), ls.mean(), ls.std()], hist,
                           np.asarray(op_mix, dtype=np.float64)])


def param_features(cfg, keys):
    """Session-parameter part: log2 of each named parameter."""
    return np.asarray([math.log2(max(1e-9, float(cfg[k]))) for k in keys], dtype=np.float64)
