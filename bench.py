#!/usr/bin/env python
"""Benchmark of the simulate stage on one GB300 (or N replicas).

Workload (default `c3`, the large configuration): a synthetic levelized
netlist of 2,000,000 GEN_*_D1 cells, depth 120, 65,536 pseudo-primary
inputs, a 20,000-cycle clocked stimulus (1,000 ps period, toggle rates
log-uniform in [0.01, 0.5]), window 0..20,000,000 ps, simulated with the
learned presize (`--alloc learned`).  One step = one pass of the hot path
over one stimulus window: every level simulated on the GPU plus the fused
SAIF counts.

  value        gate-events/s with the stimulus resident in HBM (device time
               from CUDA events on the launch stream)
  e2e          the same metric through the C ABI with host buffers: stimulus
               upload from pinned memory, run, SAIF counts back to the host
  plain_exact  the same workload with the plain exact count-then-fill
               allocation, device-timed the same way, and value / plain
  parity       a fixed-seed sample of gates from every level, each fed its
               input waveforms as the GPU produced them, run through the
               reference's own serial core (oracle/_ref, built from the
               reference sources); its output waveforms and SAIF counts are
               compared with the GPU's bit for bit
  cpu_baseline the same reference run, timed on this host's cores
  --impl reference   the reference's own serial simulator core on this
               host's cores, on a fixed-seed sample of gates fed their exact
               input waveforms (computed beforehand by the CPU oracle, which
               keeps only the lists still to be read)
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
sys.path[:0] = [str(REPO), str(REPO / "gate-level-simulator_gb300")]

import numpy as np  # noqa: E402

C4_WINDOWS, C4_MIN_CYCLES, C4_MAX_CYCLES = 256, 1_000, 50_000

WORKLOADS = {
    "c1": "c1: 2,000 cells, depth 20, 192 pseudo-primary inputs, 1,000 cycles of 1,000 ps, p=0.2",
    "c2": "c2: 200,000 cells, depth 60, 4,096 pseudo-primary inputs, 10,000 cycles of 1,000 ps, p~Beta(2,8)",
    "c3": "c3: 2,000,000 cells, depth 120, 65,536 pseudo-primary inputs, 20,000 cycles of 1,000 ps, p log-uniform [0.01,0.5]",
    "c4": "c4: the c2 netlist with 256 windows of U[1,000, 50,000] cycles, each with its own seed and Beta(2,8) rates",
}


def workload_desc(args) -> str:
    base = WORKLOADS[args.config]
    if args.cells or args.depth or args.cycles:
        return (f"{args.config} generator scaled: cells={args.cells or 'default'}, depth={args.depth or 'default'}, "
                f"cycles={args.cycles or 'default'} (profiling case, not the benchmark workload)")
    return base


def bench_config(args) -> dict:
    """The `config` object; both arms print the same one."""
    cfg = {"workload": workload_desc(args), "seed": args.seed, "alloc": args.alloc,
           "parallelism": f"replicas x{args.gpus}"}
    if args.config == "c4":
        cfg["windows"] = args.windows or C4_WINDOWS
        cfg["l2"] = "every step streams GBs of event pool per window (> L2)"
    else:
        cfg["l2"] = "256 MiB buffer written between timed steps; per-step pool is GBs (> L2)"
    return cfg


def log(*a):
    print(*a, file=sys.stderr, flush=True)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in self.rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def peak_hbm():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def make_workload(name: str, seed: int, cells=None, depth=None, cycles=None):
    from gls import synth
    cfg = synth.CONFIGS["c2" if name == "c4" else name]
    if cells or depth or cycles:
        cfg = synth.scaled(cfg, cells=cells, depth=depth, cycles=cycles)
    t0 = time.time()
    nl = synth.make_netlist(cfg, seed=seed)
    log(f"netlist {name}: {nl.n_inst} cells, {nl.n_levels} levels ({time.time() - t0:.1f}s)")
    return cfg, nl


def stimulus_for(cfg, nl, seed):
    from gls import synth
    t0 = time.time()
    st = synth.make_stimulus(cfg, nl.ppi_nets, seed=seed)
    log(f"stimulus: {st.n_events} events on {len(st.nets)} nets ({time.time() - t0:.1f}s)")
    return st


def sample_desc(r, what):
    from oracle.sample import SAMPLE_SEED
    return (f"{r['gates']} gates sampled (seed {SAMPLE_SEED}) from all levels, each fed {what}; "
            f"{r['gev']} gate-events in {r['sec']:.2f}s")


# ------------------------------------------------------------- reference arm
def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from gls.replicas import rank_seed
    from oracle.runner import run_oracle
    from oracle.sample import sample_input_nets, sample_order, sized_sample
    cfg, nl = make_workload(args.config, args.seed, args.cells, args.depth, args.cycles)
    st = stimulus_for(cfg, nl, rank_seed(args.seed, 0))
    threads = os.cpu_count() or 1
    order = sample_order(nl)
    keep = sample_input_nets(nl, order)
    t0 = time.time()
    # exact input waveforms of the sample: the C oracle over the whole
    # design, keeping only the sampled gates' input lists (every other list
    # is dropped after the last level that reads it)
    ow, _, _ = run_oracle(nl, st, 0, cfg.t_end, threads=threads, keep=keep)
    log(f"oracle port produced the sample's exact input waveforms in {time.time() - t0:.1f}s")
    r = sized_sample(nl, lambda n: ow[n], cfg.t_end, threads, order, args.ref_budget)
    snl, sst, run = r["snl"], r["sst"], r["run"]
    for _ in range(args.warmup):
        run(snl, sst, 0, cfg.t_end, threads=threads)
    times = []
    for _ in range(args.steps):
        _, _, s = run(snl, sst, 0, cfg.t_end, threads=threads)
        times.append(s)
    v = r["gev"] / float(np.mean(times))
    one = single_core(nl, lambda n: ow[n], cfg.t_end, order, r)
    line = {
        "impl": "reference", "metric": "gate-events/s", "value": v, "unit": "gate-events/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * float(np.mean(times)), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": bench_config(args),
        "cpu_baseline": {"value": v, "unit": "gate-events/s", "cores": threads, "kind": r["kind"],
                         "sample": sample_desc(r, "its exact input waveforms (C oracle over the whole design)"),
                         "single_core": one},
        "e2e": {"value": v, "unit": "gate-events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def single_core(nl, waves_of, t_end, order, r, budget_s=4.0):
    """The reference core on one thread (the reference's own loop is
    serial), on a prefix of the sample sized to about budget_s."""
    from oracle.sample import run_sample
    threads = os.cpu_count() or 1
    k = max(1, min(r["gates"], int(r["gates"] * budget_s / max(r["sec"] * threads, 1e-3))))
    one = run_sample(nl, waves_of, order[:k], 0, t_end, 1)
    return {"value": one["rate"], "unit": "gate-events/s", "cores": 1,
            "sample": f"the first {k} gates of the sample; {one['gev']} gate-events in {one['sec']:.2f}s"}


# ------------------------------------------------------------------ GPU arm
def device_timed_runs(sim, stream, flush, steps):
    """Mean device ms of `steps` runs (CUDA events on the launch stream, L2
    flushed before every run)."""
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    for k in range(steps):
        flush.zero_()
        ev[k][0].record(stream)
        sim.run()
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    return float(np.mean([a.elapsed_time(b) for a, b in ev]))


def make_sim(args, alloc, local, stream, **kw):
    from gls.capi import Simulator
    sim = Simulator(device=local, stream=stream.cuda_stream, seg_events=args.seg, alloc_mode=alloc, **kw)
    if args.alloc == "learned":
        from gls import presize
        sim.set_presize_model(*presize.load(args.model or presize.DEFAULT_MODEL))
    return sim


def parity_check(sim, r, w=0):
    """The sampled gates' outputs as the GPU made them against the reference
    core's, bit for bit (waveforms and SAIF counts)."""
    from oracle.sample import compare_outputs
    out = compare_outputs(lambda n: sim.waveform(int(n), w), sim.saif(w), r)
    out["how"] = ("each sampled gate fed its input waveforms as the GPU produced them, run through "
                  + ("the reference's own serial core (oracle/_ref)" if r["kind"] == "reference"
                     else "the C oracle") + "; output waveform and T0/T1/TX compared bit for bit")
    return out


def gls_arm(args):
    import torch
    from gls.capi import ALLOC_BOUND, ALLOC_EXACT, ALLOC_LEARNED
    from gls.replicas import max_over_ranks, rank_seed, whole_job_rate, world_rank

    world, rank, local = world_rank()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    stream = torch.cuda.current_stream()
    cfg, nl = make_workload(args.config, args.seed, args.cells, args.depth, args.cycles)
    # replicas: every rank simulates its own independent window (weak scaling)
    st = stimulus_for(cfg, nl, rank_seed(args.seed, rank))
    modes = {"bound": ALLOC_BOUND, "exact": ALLOC_EXACT, "learned": ALLOC_LEARNED}
    alloc = modes[args.alloc]
    sim = make_sim(args, alloc, local, stream)
    sim.load(nl)
    w = sim.add_window(st, 0, cfg.t_end)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")   # > 129 MB L2

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    if args.schedule:   # a fixed schedule (profiling cases): no autotuning launches
        seg_sm, mask, flags = (int(x) for x in args.schedule.split(","))
        sim.set_schedule(seg_sm, mask, flags)
        tune = {"best": {"seg_per_sm": seg_sm, "warp_mask": mask, "flags": flags}, "candidates": []}
    else:
        tune = sim.autotune()   # untimed: the schedule for this workload (results never depend on it)
    sched = {k: tune["best"][k] for k in ("seg_per_sm", "warp_mask", "flags")}
    log(f"autotune: {tune['best']}; candidates (segments/SM, warp mask, flags: ms): " +
        ", ".join(f"{c['seg_per_sm']}/{c['warp_mask']}/{c['flags']}: {c['ms']:.2f}" for c in tune["candidates"]))
    for _ in range(args.warmup):
        sim.run()
    stats = sim.stats()
    # device-timed region: stimulus resident in HBM
    barrier()
    with ClockSampler(local) as clk:
        step_ms = device_timed_runs(sim, stream, flush, args.steps)
    barrier()

    presize_q = None
    if args.alloc == "learned":
        # the predictor against the lengths this run produced (unseen stimulus seed)
        from gls import presize
        params, margin, slack = presize.load(args.model or presize.DEFAULT_MODEL)
        f, c = sim.presize_samples(w)
        q = presize.evaluate(sim.presize_predict(params, f), c, margin, slack)
        presize_q = {"gate_outputs": int(len(c)), "overflows": int(stats["presize_overflows"]),
                     "overflow_rate": stats["presize_overflows"] / max(1, len(c)), "margin": margin,
                     "mae_events": q["mae_events"], "mae_log": q["mae_log"],
                     "reserve_over_exact": q["reserve_over_exact"]}
    step_ms = max_over_ranks(step_ms, "cuda")
    gate_ev = stats["gate_events"]
    value = whole_job_rate(gate_ev, world, step_ms / 1000.0)
    sim_cycles = whole_job_rate(cfg.cycles, world, step_ms / 1000.0)
    # end to end through the C ABI with host buffers
    pinned = {k: torch.from_numpy(np.ascontiguousarray(getattr(st, k))).pin_memory().numpy()
              for k in ("nets", "ev_start", "time", "value")}
    from gls.netlist import Stimulus
    pst = Stimulus(pinned["nets"], pinned["ev_start"], pinned["time"], pinned["value"])
    h2d = pst.time.nbytes + pst.value.nbytes + 12 * nl.n_nets
    d2h = 24 * nl.n_nets
    sim.clear_windows()
    for _ in range(max(1, args.warmup // 2)):
        sim.add_window(pst, 0, cfg.t_end)
        sim.run()
        sim.saif(0)
        sim.clear_windows()
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        wid = sim.add_window(pst, 0, cfg.t_end)
        sim.run()
        sim.saif(wid)
        sim.clear_windows()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_s = max_over_ranks(e2e_s, "cuda")
    e2e = whole_job_rate(gate_ev, world, e2e_s)
    cpu = parity = None
    if rank == 0 and not args.no_cpu_baseline:
        # the reference core on a sample of gates fed the GPU's own input
        # waveforms: a bit-exact check of those gates, and the CPU timing
        sim.add_window(st, 0, cfg.t_end)
        sim.run()
        cache = {}

        def waves_of(n):
            if n not in cache:
                cache[n] = sim.waveform(int(n), 0)
            return cache[n]

        from oracle.sample import run_sample, sample_order
        t0 = time.time()
        cpu = run_sample(nl, waves_of, sample_order(nl)[: args.parity_gates], 0, cfg.t_end, os.cpu_count() or 1)
        parity = parity_check(sim, cpu)
        log(f"parity sample: {parity['gates_checked']} gates, {parity['mismatches']} mismatches "
            f"({time.time() - t0:.1f}s)")
    sim.close()
    # the plain exact count-then-fill form on the same workload and schedule
    plain = None
    if args.alloc != "exact" and not args.no_plain:
        psim = make_sim(args, ALLOC_EXACT, local, stream)
        psim.load(nl)
        psim.set_schedule(sched["seg_per_sm"], sched["warp_mask"], sched["flags"])
        psim.add_window(st, 0, cfg.t_end)
        for _ in range(max(2, args.warmup // 2)):
            psim.run()
        barrier()
        plain_ms = max_over_ranks(device_timed_runs(psim, stream, flush, args.steps), "cuda")
        pstats = psim.stats()
        psim.close()
        plain = {"value": whole_job_rate(pstats["gate_events"], world, plain_ms / 1000.0), "unit": "gate-events/s",
                 "ms_per_step": plain_ms, "pool_used_bytes": 4 * pstats["pool_used"],
                 "what": "the same window with exact count-then-fill allocation, same schedule, device-timed",
                 "value_over_plain": plain_ms / step_ms}
    # kernel-class times (for the roofline) from a profiled twin, made after
    # the timed context is gone: it brackets the classes with events, so they
    # run one after another there
    prof_steps = min(args.steps, 5)
    tsim = make_sim(args, alloc, local, stream, profile=True)
    tsim.load(nl)
    tsim.set_schedule(sched["seg_per_sm"], sched["warp_mask"], sched["flags"])
    tsim.add_window(st, 0, cfg.t_end)
    tsim.run()
    sim_ms = comb_ms = plan_ms = 0.0
    for _ in range(prof_steps):
        flush.zero_()
        tsim.run()
        s = tsim.stats()
        sim_ms += s["sim_ms"]
        comb_ms += s["combine_ms"]
        plan_ms += s["plan_ms"]
    tsim.close()
    n_drv = int(nl.n_inst)
    # algorithmic bytes of the gate kernels per step: fan-in events read
    # (5 B each per distinct input net), output events written (5 B), gate
    # metadata (48 B) and arcs (16 B)
    sim_bytes = stats["fanin_bytes"] + 5 * stats["output_events"] + 48 * n_drv + 16 * int(len(nl.arcs))
    sim_ms_step = sim_ms / prof_steps
    achieved = sim_bytes / (sim_ms_step / 1000.0) / 1e9
    peak, src = peak_hbm()
    traffic, traffic_basis = scaled_traffic(args, stats)
    # whole-step algorithmic bytes (fan-in read + outputs written + SAIF)
    step_bytes = sim_bytes + 5 * stats["output_events"] * 2 + 24 * nl.n_nets
    line = {
        "metric": "gate-events/s", "value": value, "unit": "gate-events/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": bench_config(args),
        "schedule": dict(sched, seg_events=args.seg or "auto"),
        "sim_cycles_per_s": sim_cycles,
        "gate_events_per_step": gate_ev, "output_events_per_step": stats["output_events"],
        "fanin_events_per_step": stats["fanin_bytes"] // 5,
        "roofline": {"bound": "hbm", "kernel": "k_sim", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "traffic_basis": traffic_basis,
                     "peak_source": src,
                     "algorithmic_bytes_per_step": sim_bytes,
                     "kernel_ms_per_step": {"k_sim": sim_ms_step, "k_combine": comb_ms / prof_steps,
                                            "k_plan": plan_ms / prof_steps,
                                            "timed": f"profiled run with the fan-in classes in turn, "
                                                     f"mean of {prof_steps}"},
                     "step_achieved_gbs": step_bytes / (step_ms / 1000.0) / 1e9},
        "e2e": {"value": e2e, "unit": "gate-events/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": 1000.0 * e2e_s},
        "gpu_launches": int(stats["launches"]) * args.steps,
        "clocks": clk.summary(),
        "pool_bytes": stats["pool_bytes"],
        "pool_used_bytes": 4 * stats["pool_used"],
    }
    if plain is not None:
        line["plain_exact"] = plain
    if presize_q is not None:
        line["presize"] = presize_q
    if parity is not None:
        line["parity"] = parity
    if cpu is not None:
        line["cpu_baseline"] = {"value": cpu["rate"], "unit": "gate-events/s", "cores": os.cpu_count() or 1,
                                "kind": cpu["kind"],
                                "sample": sample_desc(cpu, "its input waveforms as the GPU produced them")}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def scaled_traffic(args, stats):
    """DRAM bytes of the gate kernels per step, scaled from an ncu capture
    of a smaller case of the same generator by the fan-in events processed
    (the kernels' traffic grows with the events they read and write)."""
    tp = REPO / "profiles" / "k_sim_traffic_c3-100k-depth6-profiling-case.json"
    if not tp.exists() or args.cells or args.depth or args.cycles:
        return None, None
    tr = json.loads(tp.read_text())
    per_ev = tr.get("dram_bytes_per_fanin_event")
    if not per_ev:
        return None, None
    fanin_events = stats["fanin_bytes"] / 5
    return per_ev * fanin_events, (f"{per_ev:.3f} DRAM bytes per fan-in event over the k_sim launches of "
                                   f"{tr.get('case', 'a smaller case')} (ncu), times this step's fan-in events")


def batched_arm(args):
    """c4: many windows of uneven length on one netlist.  One step simulates
    all windows with gls_run_batched (waves of windows, one launch per kernel
    and level over a wave, graph replay, pools freed after each wave); the
    same windows as sequential plain runs (one gls_run each, exact
    allocation) are timed beside it.  With N ranks every rank takes its
    share of the windows, split by predicted work (the window's length in
    cycles: every window draws its toggle rates from the same distribution)
    with no exchange; times are the maximum over ranks, gate-events the sum."""
    import torch
    from gls import synth
    from gls.capi import ALLOC_BOUND, ALLOC_EXACT, ALLOC_LEARNED, Simulator
    from gls.netlist import Stimulus
    from gls.replicas import max_over_ranks, partition_windows, world_rank

    world, rank, local = world_rank()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    cfg, nl = make_workload("c2", args.seed, args.cells, args.depth, None)
    rng = np.random.default_rng(args.seed + 4)
    n_win = args.windows or C4_WINDOWS
    lengths = rng.integers(C4_MIN_CYCLES, C4_MAX_CYCLES + 1, size=n_win)
    mine = partition_windows(lengths, world)[rank]
    t0 = time.time()
    wins = []
    for k in mine:
        c = synth.scaled(cfg, cycles=int(lengths[k]))
        st = synth.make_stimulus(c, nl.ppi_nets, seed=args.seed + 100 + k)
        # pinned host copies: the end-to-end leg uploads from them
        p = {f: torch.from_numpy(np.ascontiguousarray(getattr(st, f))).pin_memory().numpy()
             for f in ("nets", "ev_start", "time", "value")}
        wins.append((Stimulus(p["nets"], p["ev_start"], p["time"], p["value"]), c.t_end))
    my_cycles = int(lengths[mine].sum()) if mine else 0
    log(f"c4 rank {rank}/{world}: {len(mine)} of {n_win} windows, {my_cycles} cycles, "
        f"{sum(len(w[0].time) for w in wins)} stimulus events ({time.time() - t0:.1f}s)")
    alloc = {"bound": ALLOC_BOUND, "exact": ALLOC_EXACT, "learned": ALLOC_LEARNED}[args.alloc]

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def total(x):   # summed over ranks
        if world == 1:
            return float(x)
        t = torch.tensor([float(x)], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t)
        return float(t.item())

    def batched_pass(sim):
        sim.clear_windows()
        for st, t_end in wins:
            sim.add_window(st, 0, t_end)
        sim.run_batched(saif_only=True)
        return [sim.saif(k) for k in range(len(wins))]

    sim = Simulator(device=local, alloc_mode=alloc)
    if args.alloc == "learned":
        from gls import presize
        sim.set_presize_model(*presize.load(args.model or presize.DEFAULT_MODEL))
    sim.load(nl)
    for st, t_end in wins:
        sim.add_window(st, 0, t_end)
    tune = sim.autotune(saif_only=True)   # untimed: picks the schedule on the first wave
    log(f"autotune: {tune['best']} over {tune['windows']} windows")
    for _ in range(args.warmup):
        batched_pass(sim)
    stats = sim.stats()
    gate_ev = total(stats["gate_events"])
    barrier()
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dev_ms = 0.0
        for _ in range(args.steps):
            batched_pass(sim)
            dev_ms += sim.stats()["kernel_ms"]
        torch.cuda.synchronize()
        step_s = (time.perf_counter() - t0) / args.steps
    barrier()
    dev_s = max_over_ranks(dev_ms / 1000.0 / args.steps, "cuda")
    step_s = max_over_ranks(step_s, "cuda")
    launches = sim.stats()["launches"]
    pool_b = sim.stats()["pool_bytes"]
    sim.close()
    # What a persistent kernel could at most remove: the launches themselves.
    # One window of one cycle on the same netlist runs every kernel of every
    # level with next to no work (the plan still reads one window's gates):
    # its device time per launch bounds the cost of a launch from above;
    # times this step's launches, against this step's device time.
    fixed = Simulator(device=local, alloc_mode=alloc)
    if args.alloc == "learned":
        fixed.set_presize_model(*presize.load(args.model or presize.DEFAULT_MODEL))
    fixed.load(nl)
    fixed.set_schedule(tune["best"]["seg_per_sm"], tune["best"]["warp_mask"], tune["best"]["flags"])
    one = synth.scaled(cfg, cycles=1)
    tiny = [(synth.make_stimulus(one, nl.ppi_nets, seed=args.seed + 100), one.t_end)]
    fixed_ms = fixed_launches = 0
    for rep in range(3):   # the first pass warms up
        fixed.clear_windows()
        for st, t_end in tiny:
            fixed.add_window(st, 0, t_end)
        fixed.run_batched(saif_only=True)
        fixed_ms, fixed_launches = fixed.stats()["kernel_ms"], fixed.stats()["launches"]
    fixed.close()
    per_launch_us = 1000.0 * fixed_ms / max(1, fixed_launches)
    launch_cost = {"per_launch_us": per_launch_us, "launches_per_step": int(launches),
                   "est_ms_per_step": per_launch_us * launches / 1000.0,
                   "share_of_device_time": per_launch_us * launches / 1000.0 / (dev_ms / args.steps),
                   "what": "device time per launch of one window of one cycle on the same netlist (every kernel "
                           "of every level launched, next to no work): an upper bound of a launch's cost, times "
                           "this step's launches"}
    # sequential plain runs of the same windows (exact allocation, one gls_run each)
    plain = Simulator(device=local, alloc_mode=ALLOC_EXACT)
    plain.load(nl)
    plain_s = 0.0
    for rep in range(2):   # the first pass warms up
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for st, t_end in wins:
            plain.clear_windows()
            w = plain.add_window(st, 0, t_end)
            plain.run()
            plain.saif(w)
        torch.cuda.synchronize()
        plain_s = time.perf_counter() - t0
    plain_s = max_over_ranks(plain_s, "cuda")
    plain.close()
    cycles = total(my_cycles)
    h2d = total(sum(st.time.nbytes + st.value.nbytes for st, _ in wins))
    line = {
        "metric": "gate-events/s", "value": gate_ev / dev_s, "unit": "gate-events/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * dev_s, "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": bench_config(args),
        "schedule": tune["best"],
        "cycles": int(cycles),
        "windows_per_rank": len(mine), "split": "windows over ranks by predicted work (cycles), no exchange",
        "value_timing": "device time of the waves (stimulus uploads between waves excluded); e2e: wall clock "
                        "of add_window + run_batched + SAIF reads; both the maximum over ranks",
        "sim_cycles_per_s": cycles / dev_s,
        "gate_events_per_step": gate_ev,
        "e2e": {"value": gate_ev / step_s, "unit": "gate-events/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(24 * nl.n_nets * n_win), "ms_per_step": 1000.0 * step_s},
        "plain_sequential": {"value": gate_ev / plain_s, "unit": "gate-events/s", "ms": 1000.0 * plain_s,
                             "what": "the same windows as sequential gls_run calls, exact allocation, wall clock"},
        "batched_over_plain": plain_s / step_s,
        "launch_cost": launch_cost,
        "gpu_launches": int(launches),
        "pool_bytes": pool_b,
        "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gls", choices=["gls", "reference"])
    ap.add_argument("--config", default="c3", choices=sorted(WORKLOADS))
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--seg", type=int, default=0, help="fan-in events per time segment (0 = library default)")
    ap.add_argument("--no-cpu-baseline", action="store_true",
                    help="skip the reference sample (parity check and CPU timing)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain exact-allocation comparison")
    ap.add_argument("--alloc", default="learned", choices=["bound", "exact", "learned"],
                    help="gate-output slot allocation: upper bound, exact, or learned presize")
    ap.add_argument("--model", default=None, help="presize model (.npz) for --alloc learned")
    ap.add_argument("--cells", type=int, default=None, help="override the cell count (profiling cases)")
    ap.add_argument("--depth", type=int, default=None, help="override the logic depth (profiling cases)")
    ap.add_argument("--cycles", type=int, default=None, help="override the cycle count (profiling cases)")
    ap.add_argument("--windows", type=int, default=None, help="c4: number of windows (default 256)")
    ap.add_argument("--schedule", default=None,
                    help="c1-c3: fixed schedule 'segments_per_sm,warp_mask,flags' instead of autotuning")
    ap.add_argument("--parity-gates", type=int, default=2000,
                    help="gates of the sample checked against the reference core (and timed as the CPU baseline)")
    ap.add_argument("--ref-budget", type=float, default=6.0,
                    help="reference arm: seconds of CPU work per step (the sample is sized to it)")
    args = ap.parse_args()
    if args.warmup < 3:
        log("warmup raised to 3")
        args.warmup = 3
    if args.impl == "reference":
        reference_arm(args)
    elif args.config == "c4":
        batched_arm(args)
    else:
        gls_arm(args)


if __name__ == "__main__":
    main()
