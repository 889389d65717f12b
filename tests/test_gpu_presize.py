"""GPU tests of the learned presize: the training kernels' gradients and the
two inference kernels against the CPU reference of the MLP, bit-exact
simulation in the exact and learned allocation modes (including gates that
outgrow their predicted slot), and what a trained network gains over the
plain upper-bound allocation."""
import numpy as np
import pytest

from cases import random_case
from gls import presize, synth
from gls.capi import ALLOC_BOUND, ALLOC_EXACT, ALLOC_LEARNED, MLP_PARAMS, Simulator, Trainer
from gpu_util import assert_same
from oracle import mlp_ref
from oracle.runner import run_oracle

pytestmark = pytest.mark.gpu


def constant_model(y: float) -> np.ndarray:
    """Parameters whose network outputs y for every row."""
    p = np.zeros(MLP_PARAMS, np.float32)
    p[-1] = y
    return p


def random_rows(rng, n):
    X = rng.uniform(0, 1.2, (n, 32)).astype(np.float32)
    X[:, :13] = 0
    X[np.arange(n), rng.integers(0, 13, n)] = 1
    X[:, 31] = 1
    return X


def test_trainer_gradient_matches_cpu_reference(gpu):
    rng = np.random.default_rng(1)
    X = random_rows(rng, 3000)
    t = rng.uniform(0, 8, 3000).astype(np.float32)
    with Trainer(seed=3) as tr:
        tr.set_data(X, t)
        p = tr.params()
        for first, n, huber in ((0, 3000, 1.0), (100, 700, 0.3)):
            g, loss = tr.grad(first, n, huber)
            lref, gref = mlp_ref.loss_grad(p, X[first:first + n], t[first:first + n], huber)
            assert abs(loss - lref) <= 1e-4 * max(1.0, abs(lref))
            # FP32 sums over the batch against float64: relative to the gradient's scale
            err = np.abs(g - gref)
            assert err.max() <= 2e-4 * np.abs(gref).max() + 1e-7, (err.max(), np.abs(gref).max())
            for name_lo, name_hi in ((0, 4096), (4096, 4224), (4224, 20608), (20608, 20736), (20736, 20864)):
                a, b = g[name_lo:name_hi], gref[name_lo:name_hi]
                cos = float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-30))
                assert cos > 0.9999 or np.linalg.norm(b) < 1e-9, (name_lo, cos)


def test_trainer_adam_steps_match_cpu_reference(gpu):
    """Full-batch epochs are plain Adam steps: three of them against float64."""
    rng = np.random.default_rng(4)
    X = random_rows(rng, 512)
    t = rng.uniform(0, 8, 512).astype(np.float32)
    with Trainer(seed=5) as tr:
        tr.set_data(X, t)
        p = tr.params().astype(np.float64)
        tr.fit(3, batch=512, lr=1e-3, huber=1.0, seed=0)
        got = tr.params()
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    for step in range(1, 4):
        _, g = mlp_ref.loss_grad(p, X, t, 1.0)
        m = 0.9 * m + 0.1 * g
        v = 0.999 * v + 0.001 * g * g
        p = p - 1e-3 * (m / (1 - 0.9 ** step)) / (np.sqrt(v / (1 - 0.999 ** step)) + 1e-8)
    # Adam moves every weight by about lr per step whatever its gradient, so
    # compare the displacement; weights with near-zero gradients may differ in sign
    assert np.median(np.abs(got - p)) < 1e-5, np.median(np.abs(got - p))
    assert np.mean(np.abs(got - p) < 3e-4) > 0.99


def test_inference_kernels_match_cpu_reference(gpu):
    rng = np.random.default_rng(2)
    X = random_rows(rng, 1000)
    p = rng.normal(0, 0.15, MLP_PARAMS).astype(np.float32)
    with Simulator() as s:
        y32 = s.presize_predict(p, X, tensor_cores=False)
        ytc = s.presize_predict(p, X, tensor_cores=True)
    yref, _ = mlp_ref.forward(p, X)
    assert np.abs(y32 - yref).max() <= 1e-4 * (1 + np.abs(yref).max())
    # tensor cores: BF16 operands, FP32 accumulation (tolerance for the
    # accumulation order and the rounding of hidden layer 1 at ties)
    ybf = mlp_ref.forward_bf16(p, X)
    assert np.abs(ytc - ybf).max() <= 2e-3 * (1 + np.abs(ybf).max()), np.abs(ytc - ybf).max()
    assert np.abs(ytc - yref).max() <= 0.05 * (1 + np.abs(yref).max())
    # rows past a multiple of 128 and a single row
    y1 = Simulator().presize_predict(p, X[:1], tensor_cores=True)
    assert abs(y1[0] - ytc[0]) <= 1e-6 * (1 + abs(ytc[0]))


@pytest.mark.parametrize("seed", range(6))
def test_exact_and_learned_allocation_bit_exact(seed, gpu, oracle_bin):
    nl, st = random_case(500 + seed, max_gates=60, max_in=6, horizon=5000, max_events=400)
    ow, osaif, _ = run_oracle(nl, st, 0, 6000)
    runs = [(ALLOC_EXACT, None), (ALLOC_LEARNED, constant_model(0.0)),   # every slot too short: all fall back
            (ALLOC_LEARNED, constant_model(25.0)),                      # every slot the upper bound
            (ALLOC_LEARNED, constant_model(2.5))]                       # some too short
    for mode, params in runs:
        with Simulator(alloc_mode=mode, seg_events=16 if seed % 2 else 0) as s:
            if params is not None:
                s.set_presize_model(params, margin=0.0, slack=1)
            s.load(nl)
            w = s.add_window(st, 0, 6000)
            s.run()
            gw = {n: s.waveform(n, w) for n in ow}
            assert_same(gw, s.saif(w), ow, osaif, f"seed {seed} mode {mode}")
            stats = s.stats()
            if params is not None and params[-1] == 0.0:
                assert stats["presize_overflows"] > 0
            if params is not None and params[-1] == 25.0:
                assert stats["presize_overflows"] == 0


def test_learned_mode_needs_a_model(gpu):
    nl, st = random_case(7)
    with Simulator(alloc_mode=ALLOC_LEARNED) as s:
        s.load(nl)
        s.add_window(st, 0, 500)
        with pytest.raises(Exception, match="presize_model"):
            s.run()


def test_trained_presize_gains_over_bound_allocation(gpu):
    """Train on two seeds of a scaled medium design, then run an unseen seed:
    the learned reserves take far less pool than the upper bound, few gate
    outputs fall back, and every result is identical to the plain run."""
    cfg = synth.scaled(synth.CONFIGS["c2"], cells=20_000, cycles=1_000, depth=30)
    nl = synth.make_netlist(cfg, seed=11)
    train_st = [synth.make_stimulus(cfg, nl.ppi_nets, seed=s) for s in (12, 13)]
    feat, target = presize.collect(nl, train_st, cfg.t_end)
    params, loss = presize.train(feat, target, epochs=10, batch=1024, lr=2e-3, seed=1)
    assert loss[-1] < 0.1 * loss[0]
    st = synth.make_stimulus(cfg, nl.ppi_nets, seed=99)
    res = {}
    for mode in (ALLOC_BOUND, ALLOC_EXACT, ALLOC_LEARNED):
        with Simulator(alloc_mode=mode) as s:
            if mode == ALLOC_LEARNED:
                s.set_presize_model(params)
            s.load(nl)
            w = s.add_window(st, 0, cfg.t_end)
            s.run()
            res[mode] = (s.lengths(w), s.saif(w), s.stats())
            if mode == ALLOC_BOUND:
                f, c = s.presize_samples(w)
                q = presize.evaluate(s.presize_predict(params, f), c)
    for mode in (ALLOC_EXACT, ALLOC_LEARNED):
        assert np.array_equal(res[mode][0], res[ALLOC_BOUND][0]) and np.array_equal(res[mode][1], res[ALLOC_BOUND][1])
    bound, exact, learned = (res[m][2] for m in (ALLOC_BOUND, ALLOC_EXACT, ALLOC_LEARNED))
    # gate-output slots: exact mode holds every list in 4-event-rounded slots
    lens = res[ALLOC_EXACT][0][nl.gate_output_nets()].astype(np.int64)
    stim = exact["pool_used"] - int(((lens + 3) // 4 * 4).sum())
    out_bound, out_learned = bound["pool_used"] - stim, learned["pool_used"] - stim
    assert out_learned < 0.75 * out_bound, (out_learned, out_bound)
    n_drv = len(c)
    assert learned["presize_overflows"] <= 0.02 * n_drv
    assert q["overflow_rate"] <= 0.02 and q["mae_log"] < 0.2, q


@pytest.mark.parametrize("knobs", [{}, {"GLS_PLAN_OVERLAP": "0"}, {"GLS_SIM_CONCURRENT": "0"},
                                   {"GLS_BALANCE_WEIGHT": "1"}, {"GLS_SIM_PIPELINE": "0"}])
def test_learned_mode_stream_orders_agree(knobs, gpu, oracle_bin):
    """Learned allocation in every stream order: the split plan (segments
    beside the previous level's copies, then the presize and the slots; the
    default), the whole plan after the copies (no plan overlap, no
    concurrent classes, no per-class pipeline) and the learned balance,
    which keeps the plan whole.  Some slots too short, some not."""
    from gpu_util import simulator
    nl, st = random_case(960, max_gates=120, max_in=8, horizon=20000, max_events=2000)
    ow, osaif, _ = run_oracle(nl, st, 100, 15000, threads=4)
    with simulator(None, knobs, alloc_mode=ALLOC_LEARNED) as s:
        s.set_presize_model(constant_model(3.0), margin=0.0, slack=1)
        s.load(nl)
        w = s.add_window(st, 100, 15000)
        s.run()
        gw = {n: s.waveform(n, w) for n in ow}
        assert_same(gw, s.saif(w), ow, osaif, str(knobs))
        assert s.stats()["presize_overflows"] > 0
