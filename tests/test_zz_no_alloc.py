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


def test_run_level_static_matches_gls_run(gpu):
    import torch

    cfg = synth.scaled(synth.CONFIGS["c1"], cells=900, cycles=400, depth=12)
    nl = synth.make_netlist(cfg, seed=21)
    st = synth.make_stimulus(cfg, nl.ppi_nets, seed=22)
    outs = nl.gate_output_nets()
    with Simulator() as sim:
        sim.load(nl)
        w = sim.add_window(st, 0, cfg.t_end)
        sim.run()
        ref_len = sim.lengths(w)
        ref_saif = sim.saif(w)
        ref = {int(n): sim.waveform(int(n), w) for n in outs}
        words, off, lens = pack_stimulus(st)
        cap = len(words) + 8 * int(ref_len[outs].astype(np.int64).sum()) + (1 << 16)
        dev = torch.device("cuda", 0)
        for run in range(2):    # two calls in a row share the static scratch
            pool = torch.zeros(cap, dtype=torch.int32, device=dev)
            pool[: len(words)] = torch.from_numpy(words.view(np.int32)).to(dev)
            net_off = torch.zeros(nl.n_nets, dtype=torch.int64, device=dev)
            net_len = torch.full((nl.n_nets,), -1, dtype=torch.int32, device=dev)
            net_off[torch.from_numpy(st.nets.astype(np.int64))] = torch.from_numpy(off).to(dev)
            net_len[torch.from_numpy(st.nets.astype(np.int64))] = torch.from_numpy(lens.astype(np.int32)).to(dev)
            saif = torch.zeros(3 * nl.n_nets, dtype=torch.int64, device=dev)
            top = torch.tensor([len(words)], dtype=torch.int64, device=dev)
            torch.cuda.synchronize()
            for L, cnt in enumerate(outputs_per_level(nl)):
                sim.run_level_static(L, 0, cnt, pool.data_ptr(), cap, top.data_ptr(), net_off.data_ptr(),
                                     net_len.data_ptr(), saif.data_ptr(), 0, cfg.t_end)
            h_pool = pool.cpu().numpy().view(np.uint32)
            h_off = net_off.cpu().numpy()
            h_len = net_len.cpu().numpy().view(np.uint32)
            h_saif = saif.cpu().numpy().view(np.uint64).reshape(-1, 3)
            for n in outs:
                n = int(n)
                assert h_len[n] == ref_len[n], f"run {run}: net {n} length"
                wd = h_pool[h_off[n]: h_off[n] + h_len[n]]
                t, v = ref[n]
                assert np.array_equal(wd >> 2, t) and np.array_equal(wd & 3, v), f"run {run}: net {n} waveform"
            assert np.array_equal(h_saif[outs], ref_saif[outs]), f"run {run}: SAIF"


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
