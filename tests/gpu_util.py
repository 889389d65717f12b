"""Helpers for the GPU tests: run libgls through its C ABI and compare with
the oracle."""
from __future__ import annotations

import numpy as np

from gls.capi import Simulator

U64 = 2**64 - 1
U32 = 2**32 - 1


def gpu_run(nl, st, t_begin, t_end, calc=0, seg=0, nets=None, pool_events=0):
    """-> (waves: dict net -> (times, values), saif (n,3) uint64, lengths, stats)."""
    with Simulator(calc_mode=calc, seg_events=seg, pool_events=pool_events) as s:
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
