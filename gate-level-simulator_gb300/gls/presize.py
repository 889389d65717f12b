"""Learned presize of gate-output lists: training data from simulator runs,
GPU training of the MLP, and its evaluation.

The library computes every gate output's 32 features (feature order in
include/gls.h) on the GPU, the same way for training rows
(`Simulator.presize_samples`) and for the per-level predictions of
ALLOC_LEARNED.  The target is log(1 + length of the output list); the
reserve a prediction y buys is min(fan-in events + 1,
ceil((exp(y) - 1) * (1 + margin)) + slack), and a gate whose list is longer
is placed exactly (the fallback the overflow count reports).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from .capi import ALLOC_BOUND, MLP_PARAMS, Simulator, Trainer

DEFAULT_MARGIN = 0.25
DEFAULT_SLACK = 8
# the model trained on the medium and large synthetic configurations
DEFAULT_MODEL = Path(__file__).resolve().parent / "presize_model.npz"


def collect(nl, stimuli, t_end, device: int = 0):
    """(features, target) rows from plain runs of `nl` on each stimulus."""
    feats, targets = [], []
    with Simulator(device=device, alloc_mode=ALLOC_BOUND) as s:
        s.load(nl)
        for st in stimuli:
            s.clear_windows()
            w = s.add_window(st, 0, t_end)
            s.run()
            f, c = s.presize_samples(w)
            feats.append(f)
            targets.append(np.log1p(c.astype(np.float64)).astype(np.float32))
    return np.concatenate(feats), np.concatenate(targets)


def train(feat, target, epochs: int = 8, batch: int = 8192, lr: float = 2e-3, seed: int = 0, device: int = 0):
    """Train on the GPU; returns (flat FP32 parameters, per-epoch mean loss)."""
    with Trainer(device=device, seed=seed) as tr:
        tr.set_data(feat, target)
        loss = tr.fit(epochs, batch=batch, lr=lr, huber=1.0, seed=seed)
        return tr.params(), loss


def reserve(y: np.ndarray, bound: np.ndarray, margin: float = DEFAULT_MARGIN, slack: int = DEFAULT_SLACK):
    """Events the learned mode reserves for predictions y (before 4-event rounding)."""
    length = np.expm1(np.clip(y, 0.0, 30.0)) * (1.0 + margin)
    return np.minimum(bound, np.ceil(length) + slack)


def evaluate(y: np.ndarray, count: np.ndarray, margin: float = DEFAULT_MARGIN, slack: int = DEFAULT_SLACK) -> dict:
    """Predictor quality on (y, true lengths): MAE in events and in log
    space, and the share of gate outputs whose reserve is too short."""
    c = count.astype(np.float64)
    pred = np.expm1(np.clip(y.astype(np.float64), 0.0, 30.0))
    res = np.ceil(pred * (1.0 + margin)) + slack
    return {
        "mae_events": float(np.abs(pred - c).mean()),
        "mae_log": float(np.abs(y - np.log1p(c)).mean()),
        "overflow_rate": float((c > res).mean()),
        "reserve_over_exact": float(res.sum() / max(1.0, c.sum())),
    }


def save(path, params: np.ndarray, **meta):
    np.savez(Path(path), params=np.asarray(params, np.float32), **meta)


def load(path) -> np.ndarray:
    p = np.load(Path(path))["params"]
    if p.shape != (MLP_PARAMS,):
        raise ValueError(f"{path}: not a presize model")
    return p
