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

from .capi import ALLOC_EXACT, MLP_PARAMS, Simulator, Trainer

DEFAULT_MARGIN = 0.25
DEFAULT_SLACK = 8
# the model trained on the medium and large synthetic configurations
DEFAULT_MODEL = Path(__file__).resolve().parent / "presize_model.npz"


def collect(nl, stimuli, t_end, device: int = 0):
    """(features, target) rows from plain runs of `nl` on each stimulus."""
    feats, targets = [], []
    with Simulator(device=device, alloc_mode=ALLOC_EXACT) as s:
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


def save(path, params: np.ndarray, margin: float = DEFAULT_MARGIN, slack: int = DEFAULT_SLACK, **meta):
    np.savez(Path(path), params=np.asarray(params, np.float32), margin=np.float32(margin),
             slack=np.uint32(slack), **meta)


def load(path):
    """(parameters, margin, slack) of a saved model."""
    z = np.load(Path(path))
    p = z["params"]
    if p.shape != (MLP_PARAMS,):
        raise ValueError(f"{path}: not a presize model")
    margin = float(z["margin"]) if "margin" in z else DEFAULT_MARGIN
    slack = int(z["slack"]) if "slack" in z else DEFAULT_SLACK
    return p, margin, slack


def train_default(out=DEFAULT_MODEL, device: int = 0, epochs: int = 4, log=print):
    """The shipped model: rows from runs of a medium (c2-shaped) and a large
    (c3-shaped) netlist at their own netlist and stimulus seeds, none of them
    the benchmark's; the margin is the smallest that keeps the overflow rate of
    a held-out stimulus of the large netlist at or below 1 %."""
    import time
    from . import synth
    feats, targets = [], []
    plan = [("c2", 7, list(range(11, 21))), ("c3", 8, [21, 22, 23, 24])]
    for name, nseed, sseeds in plan:
        cfg = synth.CONFIGS[name]
        nl = synth.make_netlist(cfg, seed=nseed)
        for s in sseeds:
            t0 = time.time()
            st = synth.make_stimulus(cfg, nl.ppi_nets, seed=s)
            f, t = collect(nl, [st], cfg.t_end, device)
            feats.append(f)
            targets.append(t)
            log(f"{name} netlist {nseed} stimulus {s}: {len(t)} rows ({time.time() - t0:.1f}s)")
    feat, target = np.concatenate(feats), np.concatenate(targets)
    del feats, targets
    t0 = time.time()
    params, loss = train(feat, target, epochs=epochs, batch=8192, lr=2e-3, seed=1, device=device)
    log(f"trained on {len(target)} rows in {time.time() - t0:.1f}s; loss per epoch {np.round(loss, 4).tolist()}")
    # margin on a held-out stimulus of the large netlist
    cfg = synth.CONFIGS["c3"]
    nl = synth.make_netlist(cfg, seed=8)
    f, t = collect(nl, [synth.make_stimulus(cfg, nl.ppi_nets, seed=99)], cfg.t_end, device)
    with Simulator(device=device) as s:
        y = s.presize_predict(params, f)
    count = np.round(np.expm1(t.astype(np.float64))).astype(np.uint32)
    margin = 1.0
    for m in (0.05, 0.1, 0.15, 0.2, 0.3, 0.5, 0.75, 1.0):
        q = evaluate(y, count, m, DEFAULT_SLACK)
        log(f"held out, margin {m}: {q}")
        if q["overflow_rate"] <= 0.01:
            margin = m
            break
    save(out, params, margin, DEFAULT_SLACK, rows=np.uint64(len(target)), loss=np.asarray(loss, np.float32))
    return params, margin


if __name__ == "__main__":
    import sys
    train_default(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_MODEL)
