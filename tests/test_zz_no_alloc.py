"""GPU test of gls_run_level_static, the entry point for callers that cannot
allocate device memory while they simulate (they own every device buffer,
e.g. through their own arena).  It must give exactly the waveforms and SAIF
counts of the normal gls_run path, on two runs in a row over the same
static scratch."""
import numpy as np
import pytest

from gls import synth
from gls.capi import Simulator

pytestmark = pytest.mark.gpu
U32 = 2**32 - 1


def pack_stimulus(st):
    """Stimulus as event words (time << 2 | value), every net 4-word aligned."""
    lens = np.diff(st.ev_start.astype(np.int64))
    alen = (lens + 3) & ~3
    off = np.zeros(len(lens) + 1, np.int64)
    np.cumsum(alen, out=off[1:])
    words = np.full(int(off[-1]), 0xFFFFFFFF, np.uint32)
    for k in range(len(lens)):
        t, v = st.events_of(k)
        words[off[k]: off[k] + len(t)] = (t.astype(np.uint32) << 2) | v.astype(np.uint32)
    return words, off[:-1], lens


def outputs_per_level(nl):
    n_out = np.array([c.n_out for c in nl.cells], np.int64)[nl.inst_cell]
    return [int(n_out[nl.level_start[L]: nl.level_start[L + 1]].sum()) for L in range(nl.n_levels)]


class CallerBuffers:
    """The device buffers a caller of gls_run_level_static owns: event pool
    (stimulus packed at its start), pool pointer, net table and SAIF counters."""

    def __init__(self, nl, st, cap):
        import torch
        dev = torch.device("cuda", 0)
        words, off, lens = pack_stimulus(st)
        self.cap = cap
        self.base = len(words)
        self.pool = torch.zeros(cap, dtype=torch.int32, device=dev)
        self.pool[: len(words)] = torch.from_numpy(words.view(np.int32)).to(dev)
        self.net_off = torch.zeros(nl.n_nets, dtype=torch.int64, device=dev)
        self.net_len = torch.full((nl.n_nets,), -1, dtype=torch.int32, device=dev)
        self.net_off[torch.from_numpy(st.nets.astype(np.int64))] = torch.from_numpy(off).to(dev)
        self.net_len[torch.from_numpy(st.nets.astype(np.int64))] = torch.from_numpy(lens.astype(np.int32)).to(dev)
        self.saif = torch.zeros(3 * nl.n_nets, dtype=torch.int64, device=dev)
        self.top = torch.tensor([len(words)], dtype=torch.int64, device=dev)
        torch.cuda.synchronize()

    def run(self, sim, level, first, count, t_end):
        sim.run_level_static(level, first, count, self.pool.data_ptr(), self.cap, self.top.data_ptr(),
                             self.net_off.data_ptr(), self.net_len.data_ptr(), self.saif.data_ptr(), 0, t_end)

    def check(self, outs, ref, ref_len, ref_saif, what):
        h_pool = self.pool.cpu().numpy().view(np.uint32)
        h_off = self.net_off.cpu().numpy()
        h_len = self.net_len.cpu().numpy().view(np.uint32)
        h_saif = self.saif.cpu().numpy().view(np.uint64).reshape(-1, 3)
        for n in outs:
            n = int(n)
            assert h_len[n] == ref_len[n], f"{what}: net {n} length"
            wd = h_pool[h_off[n]: h_off[n] + h_len[n]]
            t, v = ref[n]
            assert np.array_equal(wd >> 2, t) and np.array_equal(wd & 3, v), f"{what}: net {n} waveform"
        assert np.array_equal(h_saif[outs], ref_saif[outs]), f"{what}: SAIF"


def reference_run(sim, nl, st, t_end):
    """gls_run's waveforms, lengths and SAIF counts of every gate output."""
    outs = nl.gate_output_nets()
    w = sim.add_window(st, 0, t_end)
    sim.run()
    ref_len = sim.lengths(w)
    return outs, {int(n): sim.waveform(int(n), w) for n in outs}, ref_len, sim.saif(w)


def test_run_level_static_matches_gls_run(gpu):
    cfg = synth.scaled(synth.CONFIGS["c1"], cells=900, cycles=400, depth=12)
    nl = synth.make_netlist(cfg, seed=21)
    st = synth.make_stimulus(cfg, nl.ppi_nets, seed=22)
    with Simulator() as sim:
        sim.load(nl)
        outs, ref, ref_len, ref_saif = reference_run(sim, nl, st, cfg.t_end)
        cap = len(pack_stimulus(st)[0]) + 8 * int(ref_len[outs].astype(np.int64).sum()) + (1 << 16)
        for run in range(2):    # two calls in a row share the static scratch
            buf = CallerBuffers(nl, st, cap)
            for L, cnt in enumerate(outputs_per_level(nl)):
                buf.run(sim, L, 0, cnt, cfg.t_end)
            buf.check(outs, ref, ref_len, ref_saif, f"run {run}")


def test_run_level_static_split_levels(gpu):
    """Every level in several calls of 7 gate outputs (first > 0, fan-in
    class ranges clipped to each call's share), twice in a row."""
    cfg = synth.scaled(synth.CONFIGS["c1"], cells=900, cycles=400, depth=12)
    nl = synth.make_netlist(cfg, seed=23)
    st = synth.make_stimulus(cfg, nl.ppi_nets, seed=24)
    with Simulator() as sim:
        sim.load(nl)
        outs, ref, ref_len, ref_saif = reference_run(sim, nl, st, cfg.t_end)
        cap = len(pack_stimulus(st)[0]) + 8 * int(ref_len[outs].astype(np.int64).sum()) + (1 << 16)
        for run in range(2):
            buf = CallerBuffers(nl, st, cap)
            for L, cnt in enumerate(outputs_per_level(nl)):
                for first in range(0, cnt, 7):
                    buf.run(sim, L, first, min(7, cnt - first), cfg.t_end)
            buf.check(outs, ref, ref_len, ref_saif, f"split run {run}")


def test_run_level_static_retry_after_scratch_limit(gpu):
    """A level whose fan-in needs more than the static segment scratch fails
    with GLS_ERANGE and leaves the caller's pool pointer and tables as they
    were; the same level in smaller calls then gives gls_run's results."""
    from gls.capi import GlsError

    # one level of 3,000 gates over ~1,200-event stimulus nets: ~8 M
    # segment-stack words, about twice the static scratch
    cfg = synth.scaled(synth.CONFIGS["c2"], cells=3_000, cycles=6_000, depth=1, ppi=512)
    nl = synth.make_netlist(cfg, seed=25)
    st = synth.make_stimulus(cfg, nl.ppi_nets, seed=26)
    (cnt,) = outputs_per_level(nl)
    with Simulator() as sim:
        sim.load(nl)
        outs, ref, ref_len, ref_saif = reference_run(sim, nl, st, cfg.t_end)
        cap = len(pack_stimulus(st)[0]) + 8 * int(ref_len[outs].astype(np.int64).sum()) + (1 << 16)
        buf = CallerBuffers(nl, st, cap)
        with pytest.raises(GlsError) as e:
            buf.run(sim, 0, 0, cnt, cfg.t_end)
        assert e.value.code == 5, e.value   # GLS_ERANGE
        assert int(buf.top.item()) == buf.base, "a failed call must not move the pool pointer"
        assert (buf.net_len[torch_index(outs)] == -1).all().item(), "a failed call must not write net lengths"
        step = 500
        for first in range(0, cnt, step):
            buf.run(sim, 0, first, min(step, cnt - first), cfg.t_end)
        buf.check(outs, ref, ref_len, ref_saif, "after retry")


def torch_index(a):
    import torch
    return torch.from_numpy(np.asarray(a, np.int64)).to("cuda")


def test_run_level_static_rejects_oversized_request(gpu):
    import torch
    from gls.capi import GlsError

    # one level of 20,000 gate outputs: more than one call may take
    cfg = synth.scaled(synth.CONFIGS["c1"], cells=20_000, cycles=10, depth=1)
    nl = synth.make_netlist(cfg, seed=3)
    with Simulator() as sim:
        sim.load(nl)
        buf = torch.zeros(64, dtype=torch.int64, device="cuda")
        p = buf.data_ptr()
        with pytest.raises(GlsError) as e:
            sim.run_level_static(0, 0, 20_000, p, 16, p, p, p, p, 0, 10)
        assert e.value.code == 5     # GLS_ERANGE, before any device work
        with pytest.raises(GlsError):   # more outputs than the level has
            sim.run_level_static(0, 10, 20_000, p, 16, p, p, p, p, 0, 10)
