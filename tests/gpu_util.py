"""Helpers for the GPU tests: run libgls through its C ABI and compare with
the oracle."""
from __future__ import annotations

import os

import numpy as np

from gls.capi import Simulator

U64 = 2**64 - 1
U32 = 2**32 - 1


def simulator(warp_mask=None, env=None, **kw):
    """A Simulator; warp_mask picks which fan-in classes (bit 0: one input
    net, 1: two, 2: three) run the warp-per-segment kernel instead of the
    thread-per-segment one, env sets other library knobs (both are read when
    a context is made)."""
    env = dict(env or {})
    if warp_mask is not None:
        env["GLS_SIM_WARP_MASK"] = str(warp_mask)
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        return Simulator(**kw)
    finally:
        for k, v in old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v


def gpu_run(nl, st, t_begin, t_end, calc=0, seg=0, nets=None, pool_events=0, warp_mask=None, env=None):
    """-> (waves: dict net -> (times, values), saif (n,3) uint64, lengths, stats)."""
    with simulator(warp_mask, env, calc_mode=calc, seg_events=seg, pool_events=pool_events) as s:
        s.load(nl)
        w = s.add_window(st, t_begin, t_end)
        s.run()
        lens = s.lengths(w)
        saif = s.saif(w)
        waves = {}
        todo = range(nl.n_nets) if nets is None else nets
        for n in todo:
            if lens[n] != U32:
                waves[int(n)] = s.waveform(int(n), w)
        return waves, saif, lens, s.stats()


def assert_same(gw, gsaif, ow, osaif, what=""):
    """GPU result == oracle result on every net the oracle produced."""
    for n, (t, v) in ow.items():
        assert n in gw, f"{what}: GPU did not produce net {n}"
        gt, gv = gw[n]
        if not (np.array_equal(np.asarray(gt, np.int64), np.asarray(t, np.int64))
                and np.array_equal(np.asarray(gv, np.int64), np.asarray(v, np.int64))):
            k = 0
            m = min(len(gt), len(t))
            while k < m and gt[k] == t[k] and gv[k] == v[k]:
                k += 1
            raise AssertionError(f"{what}: net {n} differs at event {k}: gpu {list(zip(gt[k:k+4], gv[k:k+4]))} "
                                 f"oracle {list(zip(t[k:k+4], v[k:k+4]))} (len {len(gt)} vs {len(t)})")
    rows = [n for n in range(len(osaif)) if osaif[n][0] != U64]
    assert np.array_equal(gsaif[rows], osaif[rows]), f"{what}: SAIF differs"


def waveform_properties(waves, saif, t_begin, t_end, driven):
    """Checks that hold for any correct run, whatever the size."""
    dur = t_end - t_begin
    for n, (t, v) in waves.items():
        t = np.asarray(t, np.int64)
        v = np.asarray(v, np.int64)
        assert len(t) >= 1
        assert (np.diff(t) > 0).all(), f"net {n}: times not strictly increasing"
        if n in driven:
            assert t[0] == 0, f"net {n}: gate output must start at time 0"
            assert (v[1:] != v[:-1]).all(), f"net {n}: repeated value in a gate output"
        assert int(saif[n].sum()) == dur, f"net {n}: T0+T1+TX != duration"
