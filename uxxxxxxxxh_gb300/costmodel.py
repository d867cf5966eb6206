"""Learned cost model: predicts a launch's time per point from the program's
and the launch's features, so the tuner can rank candidates of a program it
has never timed.

The network is the library's MLP (include/uhs.h, uhs_mlp_*): 30 features
(tuner.features) -> 3 x 64 (ReLU) -> 1, trained on the GPU by the library's own forward, backward
and Adam kernels on the tuner's timing records (tuner.Tuner.records), five
of them from different seeds averaged as an ensemble.  Target: log(ns per
point), standardised.  pick() runs the network over every
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
    """An ensemble of `members` networks of the same shape, each trained from
    its own seed (initial weights and minibatch order) on the same records;
    the prediction is the mean of their standardised outputs, which lowers
    the variance that decides between candidates a few per cent apart."""

    def __init__(self, hidden: int = 64, layers: int = 3, seed: int = 0, members: int = 5):
        self.nets = [MLP(N_FEATURES, hidden, layers, seed + 7919 * i) for i in range(members)]
        self.seed = seed
        self.mu = 0.0
        self.sigma = 1.0
        self.trained_on = 0

    @property
    def net(self) -> MLP:
        return self.nets[0]

    def fit(self, records: list, epochs: int = 300, batch: int = 256, lr: float = 2e-3, seed: int = 0) -> float:
        """Train every member; returns the members' mean final loss.  The
        target is log(ns per point).  (Targets relative to each program's
        fastest launch were tried and ranked worse on held-out programs:
        mean pick 0.961 of the exhaustive best against 0.974.)"""
        x = np.array([r["features"] for r in records], np.float32)
        t = np.log(np.array([r["ns_per_point"] for r in records], np.float64))
        self.mu, self.sigma = float(t.mean()), float(t.std() or 1.0)
        y = ((t - self.mu) / self.sigma).astype(np.float32)
        self.trained_on = len(records)
        losses = [n.train(x, y, epochs, min(batch, len(records)), lr, seed + 104729 * i)
                  for i, n in enumerate(self.nets)]
        return float(np.mean(losses))

    def predict_ns(self, feats) -> np.ndarray:
        """Predicted nanoseconds per point of each launch."""
        x = np.asarray(feats, np.float32)
        y = np.mean([n.forward(x).astype(np.float64) for n in self.nets], axis=0)
        return np.exp(y * self.sigma + self.mu)

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
                       "mu": self.mu, "sigma": self.sigma, "trained_on": self.trained_on,
                       "members": [n.get_params().tolist() for n in self.nets]}, f)

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
        members = d["members"] if "members" in d else [d["params"]]
        m = CostModel(d["hidden"], d["layers"], members=len(members))
        m.mu, m.sigma, m.trained_on = d["mu"], d["sigma"], d.get("trained_on", 0)
        for n, w in zip(m.nets, members):
            n.set_params(np.array(w, np.float32))
        return m
