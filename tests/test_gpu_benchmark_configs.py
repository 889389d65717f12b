"""GPU parity on the benchmark configurations themselves, with the
benchmark's seeds (netlist 2024, stimulus 2025).

* c2 in full (200,000 cells, depth 60, 10,000 cycles): every net's waveform
  and SAIF row against the C oracle, in the learned and exact allocation
  modes.
* c3 (2,000,000 cells, depth 120, 20,000 cycles): too large for the oracle
  to keep every list, so an inductive check: a fixed-seed sample of 2,000
  gates from every level, each fed its input waveforms as the GPU produced
  them, run through the reference's own serial core; every sampled gate's
  output waveform and SAIF counts must equal the GPU's bit for bit.  With
  each gate exact given its inputs, and the stimulus exact, the whole run is
  exact on the sampled gates' cones.
"""
import os

import numpy as np
import pytest

from gls import presize, synth
from gls.capi import ALLOC_EXACT, ALLOC_LEARNED, Simulator
from gls.replicas import rank_seed
from oracle.runner import run_oracle
from oracle.sample import compare_outputs, run_sample, sample_order

pytestmark = pytest.mark.gpu
SEED = 2024
U32 = 2**32 - 1
U64 = 2**64 - 1


def bench_workload(name):
    cfg = synth.CONFIGS[name]
    nl = synth.make_netlist(cfg, seed=SEED)
    st = synth.make_stimulus(cfg, nl.ppi_nets, seed=rank_seed(SEED, 0))
    return cfg, nl, st


def learned_sim(alloc):
    s = Simulator(alloc_mode=alloc)
    if alloc == ALLOC_LEARNED:
        s.set_presize_model(*presize.load(presize.DEFAULT_MODEL))
    return s


@pytest.fixture(scope="module")
def c2_oracle(oracle_bin):
    cfg, nl, st = bench_workload("c2")
    ow, osaif, _ = run_oracle(nl, st, 0, cfg.t_end, threads=os.cpu_count() or 1)
    return cfg, nl, st, ow, osaif


@pytest.mark.parametrize("alloc", [ALLOC_LEARNED, ALLOC_EXACT])
def test_gpu_c2_full_config_vs_oracle(alloc, gpu, c2_oracle):
    cfg, nl, st, ow, osaif = c2_oracle
    with learned_sim(alloc) as s:
        s.load(nl)
        w = s.add_window(st, 0, cfg.t_end)
        s.run()
        lens = s.lengths(w)
        saif = s.saif(w)
        done = osaif[:, 0] != U64
        assert np.array_equal(saif[done], osaif[done]), "c2: SAIF rows differ"
        assert (lens[done] != U32).all()
        for n, (t, v) in ow.items():
            assert lens[n] == len(t), f"c2: net {n} length {lens[n]} vs {len(t)}"
            gt, gv = s.waveform(n, w)
            assert np.array_equal(gt.astype(np.int64), t.astype(np.int64)) and np.array_equal(gv, v), \
                f"c2: net {n} waveform differs"
        stats = s.stats()
    assert stats["gate_events"] > 1_000_000_000


def test_gpu_c3_sampled_gates_vs_reference(gpu, ref_bin):
    cfg, nl, st = bench_workload("c3")
    with learned_sim(ALLOC_LEARNED) as s:
        s.load(nl)
        w = s.add_window(st, 0, cfg.t_end)
        s.run()
        order = sample_order(nl)[:2000]
        levels = np.searchsorted(nl.level_start, order, side="right") - 1
        assert len(np.unique(levels)) == nl.n_levels, "the sample must reach every level"
        cache = {}

        def gpu_wave(n):
            if n not in cache:
                cache[n] = s.waveform(int(n), w)
            return cache[n]

        r = run_sample(nl, gpu_wave, order, 0, cfg.t_end, os.cpu_count() or 1)
        res = compare_outputs(lambda n: s.waveform(int(n), w), s.saif(w), r)
    assert res["gates_checked"] == 2000 and res["checker"] == "reference"
    assert res["mismatches"] == 0, res
