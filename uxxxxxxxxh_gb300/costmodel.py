"""Learned cost model: predicts a launch's time per point from the program's
and the launch's features, so the tuner can rank candidates of a program it
has never timed.

The network is the library's MLP (include/uhs.h, uhs_mlp_*): 25 features
(tuner.features) -> 3 x 64 (ReLU) -> 1, trained on the GPU by the library's own forward, backward
and Adam kernels on the tuner's timing records (tuner.Tuner.records).  Target:
log(ns per point), standardised.  pick() runs the network over every
candidate of a program and returns the one it predicts fastest; exhaustive
tuning (tuner.Tuner.tune) stays the fallback and the yardstick of the model's
regret.
"""
from __future__ import annotations

import ctypes
import json
import math
import os

import numpy as np

from . import _lib
from .runtime import RunParams
from .stencil import Stencil
from .tuner import N_FEATURES, candidates, class_features, features, measure

# The model trained on GB300 timings by tuner_study (shipped with the package).
DEFAULT_MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "costmodel.json")


def _fptr(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class MLP:
    """Handle on a uhs_mlp."""

    def __init__(self, in_dim: int, hidden: int = 64, layers: int = 3, seed: int = 0):
        self.in_dim, self.hidden, self.layers = in_dim, hidden, layers
        self._h = ctypes.c_void_p()
        _lib.check(_lib.lib().uhs_mlp_create(in_dim, hidden, layers, seed, ctypes.byref(self._h)))

    def __del__(self):
        try:
            if self._h:
                _lib.lib().uhs_mlp_destroy(self._h)
        except Exception:
            pass

    @property
    def num_params(self) -> int:
        return int(_lib.lib().uhs_mlp_num_params(self._h))

    def get_params(self) -> np.ndarray:
        out = np.empty(self.num_params, np.float32)
        _lib.check(_lib.lib().uhs_mlp_get_params(self._h, _fptr(out)))
        return out

    def set_params(self, w: np.ndarray) -> None:
        w = np.ascontiguousarray(w, np.float32)
        assert w.size == self.num_params
        _lib.check(_lib.lib().uhs_mlp_set_params(self._h, _fptr(w)))

    def forward(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32)
        y = np.empty(x.shape[0], np.float32)
        _lib.check(_lib.lib().uhs_mlp_forward(self._h, _fptr(x), x.shape[0], _fptr(y)))
        return y

    def loss_grad(self, x: np.ndarray, y: np.ndarray):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        loss = np.zeros(1, np.float32)
        g = np.empty(self.num_params, np.float32)
        _lib.check(_lib.lib().uhs_mlp_loss_grad(self._h, _fptr(x), _fptr(y), x.shape[0], _fptr(loss), _fptr(g)))
        return float(loss[0]), g

    def train(self, x: np.ndarray, y: np.ndarray, epochs: int, batch: int, lr: float, seed: int = 0) -> float:
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        loss = np.zeros(1, np.float32)
        _lib.check(_lib.lib().uhs_mlp_train(self._h, _fptr(x), _fptr(y), x.shape[0], epochs, batch, lr, seed,
                                            _fptr(loss)))
        return float(loss[0])


class CostModel:
    def __init__(self, hidden: int = 64, layers: int = 3, seed: int = 0):
        self.net = MLP(N_FEATURES, hidden, layers, seed)
        self.mu = 0.0
        self.sigma = 1.0
        self.trained_on = 0

    def fit(self, records: list, epochs: int = 300, batch: int = 256, lr: float = 2e-3, seed: int = 0) -> float:
        x = np.array([r["features"] for r in records], np.float32)
        t = np.log(np.array([r["ns_per_point"] for r in records], np.float64))
        self.mu, self.sigma = float(t.mean()), float(t.std() or 1.0)
        y = ((t - self.mu) / self.sigma).astype(np.float32)
        self.trained_on = len(records)
        return self.net.train(x, y, epochs, min(batch, len(records)), lr, seed)

    def predict_ns(self, feats) -> np.ndarray:
        y = self.net.forward(np.asarray(feats, np.float32))
        return np.exp(y.astype(np.float64) * self.sigma + self.mu)

    def rank(self, st: Stencil) -> list:
        """Candidates of st ordered by predicted time, fastest first."""
        cands = candidates(st)
        cls = class_features(st)
        ns = self.predict_ns([features(st, p, cls) for p in cands])
        return [cands[i] for i in np.argsort(ns)]

    def pick(self, st: Stencil) -> RunParams:
        """The candidate the network predicts fastest (no timing)."""
        return self.rank(st)[0]

    def pick_verified(self, st: Stencil, a, b, k: int = 3, reps: int = 3) -> RunParams:
        """Time only the network's k best candidates and keep the fastest:
        k timings instead of the exhaustive search's dozens."""
        top = self.rank(st)[:k]
        return min(top, key=lambda p: measure(st, a, b, p, reps))

    def save(self, path: str) -> None:
        with open(path, "w") as f:
            json.dump({"features": N_FEATURES, "hidden": self.net.hidden, "layers": self.net.layers,
                       "mu": self.mu, "sigma": self.sigma,
                       "trained_on": self.trained_on, "params": self.net.get_params().tolist()}, f)

    @staticmethod
    def default() -> "CostModel":
        """The shipped model (data/costmodel.json)."""
        return CostModel.load(DEFAULT_MODEL)

    @staticmethod
    def load(path: str) -> "CostModel":
        with open(path) as f:
            d = json.load(f)
        if d.get("features", N_FEATURES) != N_FEATURES:
            raise ValueError(f"{path}: model of {d.get('features')} features, this library has {N_FEATURES}")
        m = CostModel(d["hidden"], d["layers"])
        m.mu, m.sigma, m.trained_on = d["mu"], d["sigma"], d.get("trained_on", 0)
        m.net.set_params(np.array(d["params"], np.float32))
        return m
