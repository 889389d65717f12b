#!/usr/bin/env python
"""Benchmark of the simulate stage on one GB300 (or N replicas).

Workload (default `c2`, the medium configuration): a synthetic levelized
netlist of 200,000 GEN_*_D1 cells, depth 60, 4,096 pseudo-primary inputs, a
10,000-cycle clocked stimulus (1,000 ps period, Beta(2,8) toggle rates),
window 0..10,000,000 ps.  One step = one pass of the hot path over one
stimulus window: every level simulated on the GPU plus the fused SAIF counts.

  value   gate-events/s with the stimulus resident in HBM (device time from
          CUDA events on the launch stream)
  e2e     the same metric through the C ABI with host buffers: stimulus
          upload from pinned memory, run, SAIF counts back to the host
  --impl reference   the reference's own serial simulator core
          (oracle/_ref, built from the reference sources) on this host's
          cores, on a fixed-seed sample of gates fed their exact input
          waveforms (computed beforehand by the CPU oracle).
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


# ------------------------------------------------------------- reference leg
def sample_case(nl, waves_of, k, seed):
    """k gates drawn with a fixed seed from all levels, rewired as independent
    single gates whose inputs are stimulus nets carrying their exact input
    waveforms.  Returns (netlist, stimulus, gate_events)."""
    from gls.levelize import assemble
    from gls.netlist import Stimulus
    rng = np.random.default_rng(seed)
    pick = np.sort(rng.choice(nl.n_inst, size=min(k, nl.n_inst), replace=False))
    insts, stim, nxt, gev = [], {}, 0, 0
    for i in pick:
        c = nl.cells[int(nl.inst_cell[i])]
        src = nl.inputs_of(int(i))
        local = {}
        ins = []
        for n in src.tolist():
            if n not in local:
                local[n] = nxt
                stim[nxt] = waves_of(n)
                nxt += 1
            ins.append(local[n])
            gev += len(stim[local[n]][0])
        arcs = [(int(a["edge"]), int(a["in_pin"]), int(a["out_pin"]), float(a["rise"]), float(a["fall"]))
                for a in nl.arcs[int(nl.arc_start[i]): int(nl.arc_start[i + 1])]]
        insts.append((c.name, ins, [-1] * c.n_out, arcs))
    for inst in insts:
        inst[2][:] = list(range(nxt, nxt + len(inst[2])))
        nxt += len(inst[2])
    sn = sorted(stim)
    ev = np.zeros(len(sn) + 1, np.uint64)
    ev[1:] = np.cumsum([len(stim[n][0]) for n in sn])
    T = np.concatenate([np.asarray(stim[n][0], np.uint32) for n in sn]) if sn else np.zeros(0, np.uint32)
    V = np.concatenate([np.asarray(stim[n][1], np.uint8) for n in sn]) if sn else np.zeros(0, np.uint8)
    return assemble(insts, n_nets=nxt), Stimulus(np.array(sn, np.uint32), ev, T, V), gev


def time_reference_sample(nl, waves_of, t_end, threads, budget_s=8.0, seed=7, max_k=4000):
    """Time the reference core on a sample sized to ~budget_s of wall time.
    -> (gate-events/s, description, kind, threads)."""
    from oracle import build as obuild
    from oracle.runner import run_oracle, run_reference
    have_ref = obuild.build_reference() is not None
    k = 24
    while True:
        snl, sst, gev = sample_case(nl, waves_of, k, seed)
        if have_ref:
            _, _, sec = run_reference(snl, sst, 0, t_end, threads=threads)
        else:
            _, _, sec = run_oracle(snl, sst, 0, t_end, threads=threads)
        if sec >= budget_s / 3 or k >= max_k or k >= nl.n_inst:
            break
        k = min(max_k, nl.n_inst, int(k * max(2.0, budget_s / max(sec, 1e-3) * 0.8)))
    kind = "reference" if have_ref else "port"
    desc = (f"{len(snl.inst_cell)} gates sampled (seed {seed}) from all levels, each fed its exact "
            f"input waveforms; {gev} gate-events in {sec:.2f}s")
    return gev / sec, desc, kind, sec, snl, sst, gev


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle.runner import run_oracle
    cfg, nl = make_workload(args.config, args.seed, args.cells, args.depth, args.cycles)
    st = stimulus_for(cfg, nl, args.seed + 1)
    threads = os.cpu_count() or 1
    t0 = time.time()
    ow, _, _ = run_oracle(nl, st, 0, cfg.t_end, threads=threads)
    log(f"oracle port produced the exact waveforms in {time.time() - t0:.1f}s")
    rate, desc, kind, sec, snl, sst, gev = time_reference_sample(nl, lambda n: ow[n], cfg.t_end, threads)
    from oracle.runner import run_oracle as ro, run_reference as rr
    for _ in range(args.warmup):
        (rr if kind == "reference" else ro)(snl, sst, 0, cfg.t_end, threads=threads)
    times = []
    for _ in range(args.steps):
        _, _, s = (rr if kind == "reference" else ro)(snl, sst, 0, cfg.t_end, threads=threads)
        times.append(s)
    v = gev / float(np.mean(times))
    line = {
        "impl": "reference", "metric": "gate-events/s", "value": v, "unit": "gate-events/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * float(np.mean(times)), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": workload_desc(args), "seed": args.seed},
        "cpu_baseline": {"value": v, "unit": "gate-events/s", "cores": threads, "kind": kind, "sample": desc},
        "e2e": {"value": v, "unit": "gate-events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU arm
def gls_arm(args):
    import torch
    from gls.capi import Simulator
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
    from gls.capi import ALLOC_BOUND, ALLOC_EXACT, ALLOC_LEARNED
    alloc = {"bound": ALLOC_BOUND, "exact": ALLOC_EXACT, "learned": ALLOC_LEARNED}[args.alloc]
    sim = Simulator(device=local, stream=stream.cuda_stream, seg_events=args.seg, alloc_mode=alloc)
    if args.alloc == "learned":
        from gls import presize
        sim.set_presize_model(*presize.load(args.model or presize.DEFAULT_MODEL))
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
    log(f"autotune: {tune['best']}; candidates (segments/SM, warp mask, flags: ms): " +
        ", ".join(f"{c['seg_per_sm']}/{c['warp_mask']}/{c['flags']}: {c['ms']:.2f}" for c in tune["candidates"]))
    for _ in range(args.warmup):
        sim.run()
    stats = sim.stats()
    # device-timed region: stimulus resident in HBM
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    sim_ms = comb_ms = plan_ms = 0.0
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            sim.run()
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    barrier()
    step_ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))

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
        counts = sim.saif(wid)
        sim.clear_windows()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_s = max_over_ranks(e2e_s, "cuda")
    e2e = whole_job_rate(gate_ev, world, e2e_s)
    # roofline of the dominant kernel (k_sim): algorithmic bytes per step =
    # fan-in events read (5 B each per distinct net) + output events written
    # (5 B) + gate metadata (48 B) and arcs (16 B); divided by its event time.
    if rank == 0 and not args.no_cpu_baseline:
        # the reference core on a sample, fed exact waveforms from this run
        sim.clear_windows()
        sim.add_window(st, 0, cfg.t_end)
        sim.run()
        threads = os.cpu_count() or 1
        cache = {}

        def waves_of(n):
            if n not in cache:
                cache[n] = sim.waveform(int(n), 0)
            return cache[n]

        cpu = time_reference_sample(nl, waves_of, cfg.t_end, threads)
    sim.close()
    # kernel-class times (for the roofline) from a profiled twin, made after
    # the timed context is gone: it brackets the classes with events, so they
    # run one after another there
    psim = Simulator(device=local, stream=stream.cuda_stream, profile=True, seg_events=args.seg, alloc_mode=alloc)
    if args.alloc == "learned":
        from gls import presize
        psim.set_presize_model(*presize.load(args.model or presize.DEFAULT_MODEL))
    psim.load(nl)
    psim.set_schedule(tune["best"]["seg_per_sm"], tune["best"]["warp_mask"], tune["best"]["flags"])
    psim.add_window(st, 0, cfg.t_end)
    psim.run()
    for _ in range(args.steps):
        flush.zero_()
        psim.run()
        s = psim.stats()
        sim_ms += s["sim_ms"]
        comb_ms += s["combine_ms"]
        plan_ms += s["plan_ms"]
    psim.close()
    n_drv = int(nl.n_inst)
    sim_bytes = stats["fanin_bytes"] + 5 * stats["output_events"] + 48 * n_drv + 16 * int(len(nl.arcs))
    sim_ms_step = sim_ms / args.steps
    achieved = sim_bytes / (sim_ms_step / 1000.0) / 1e9
    peak, src = peak_hbm()
    # DRAM bytes of the k_sim launches of one step, from an ncu capture of
    # this workload (one-pass metrics; profiles/k_sim_c2-depth6-profiling-case.md)
    traffic = None
    tp = REPO / "profiles" / "k_sim_traffic.json"
    if tp.exists() and not (args.cells or args.depth or args.cycles):
        tr = json.loads(tp.read_text())
        if tr.get("workload") == args.config:
            traffic = tr.get("bytes_per_step")
    # whole-step algorithmic bytes (fan-in read + outputs written + SAIF)
    step_bytes = sim_bytes + 5 * stats["output_events"] * 2 + 24 * nl.n_nets
    line = {
        "metric": "gate-events/s", "value": value, "unit": "gate-events/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": workload_desc(args), "seed": args.seed, "parallelism": f"replicas x{world}",
                   "l2": "256 MiB buffer written between timed steps; per-step pool is GBs (> L2)",
                   "seg_events": args.seg or "auto", "alloc": args.alloc,
                   "schedule": {k: tune["best"][k] for k in ("seg_per_sm", "warp_mask", "flags")}},
        "sim_cycles_per_s": sim_cycles,
        "gate_events_per_step": gate_ev, "output_events_per_step": stats["output_events"],
        "roofline": {"bound": "hbm", "kernel": "k_sim", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "traffic_basis": "DRAM bytes per step over the k_sim launches, ncu capture of this workload"
                                      if traffic else None,
                     "peak_source": src,
                     "algorithmic_bytes_per_step": sim_bytes,
                     "kernel_ms_per_step": {"k_sim": sim_ms_step, "k_combine": comb_ms / args.steps,
                                            "k_plan": plan_ms / args.steps,
                                            "timed": "profiled run with the fan-in classes in turn"},
                     "step_achieved_gbs": step_bytes / (step_ms / 1000.0) / 1e9},
        "e2e": {"value": e2e, "unit": "gate-events/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": 1000.0 * e2e_s},
        "gpu_launches": int(stats["launches"]) * args.steps,
        "clocks": clk.summary(),
        "pool_bytes": stats["pool_bytes"],
        "pool_used_bytes": 4 * stats["pool_used"],
    }
    if presize_q is not None:
        line["presize"] = presize_q
    if rank == 0 and not args.no_cpu_baseline:
        rate, desc, kind, sec, *_ = cpu
        line["cpu_baseline"] = {"value": rate, "unit": "gate-events/s", "cores": os.cpu_count() or 1,
                                "kind": kind, "sample": desc}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def batched_arm(args):
    """c4: many windows of uneven length on one netlist.  One step simulates
    all windows with gls_run_batched (waves of windows, one launch per kernel
    and level over a wave, graph replay, pools freed after each wave); the
    same windows as sequential plain runs (one gls_run each, exact
    allocation) are timed beside it."""
    import torch
    from gls import synth
    from gls.capi import ALLOC_BOUND, ALLOC_EXACT, ALLOC_LEARNED, Simulator
    from gls.netlist import Stimulus
    torch.cuda.set_device(0)
    cfg, nl = make_workload("c2", args.seed, args.cells, args.depth, None)
    rng = np.random.default_rng(args.seed + 4)
    n_win = args.windows or C4_WINDOWS
    lengths = rng.integers(C4_MIN_CYCLES, C4_MAX_CYCLES + 1, size=n_win)
    t0 = time.time()
    wins = []
    for k, cyc in enumerate(lengths.tolist()):
        c = synth.scaled(cfg, cycles=int(cyc))
        st = synth.make_stimulus(c, nl.ppi_nets, seed=args.seed + 100 + k)
        # pinned host copies: the end-to-end leg uploads from them
        p = {f: torch.from_numpy(np.ascontiguousarray(getattr(st, f))).pin_memory().numpy()
             for f in ("nets", "ev_start", "time", "value")}
        wins.append((Stimulus(p["nets"], p["ev_start"], p["time"], p["value"]), c.t_end))
    log(f"c4: {n_win} windows, {int(lengths.sum())} cycles, "
        f"{sum(len(w[0].time) for w in wins)} stimulus events ({time.time() - t0:.1f}s)")
    alloc = {"bound": ALLOC_BOUND, "exact": ALLOC_EXACT, "learned": ALLOC_LEARNED}[args.alloc]

    def batched_pass(sim):
        sim.clear_windows()
        for st, t_end in wins:
            sim.add_window(st, 0, t_end)
        sim.run_batched(saif_only=True)
        return [sim.saif(k) for k in range(len(wins))]

    sim = Simulator(alloc_mode=alloc)
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
    gate_ev = stats["gate_events"]
    with ClockSampler(0) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dev_ms = 0.0
        for _ in range(args.steps):
            batched_pass(sim)
            dev_ms += sim.stats()["kernel_ms"]
        torch.cuda.synchronize()
        step_s = (time.perf_counter() - t0) / args.steps
    dev_s = dev_ms / 1000.0 / args.steps
    launches = sim.stats()["launches"]
    pool_b = sim.stats()["pool_bytes"]
    sim.close()
    # sequential plain runs of the same windows (exact allocation, one gls_run each)
    plain = Simulator(alloc_mode=ALLOC_EXACT)
    plain.load(nl)
    plain_s = 0.0
    for rep in range(2):   # the first pass warms up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for st, t_end in wins:
            plain.clear_windows()
            w = plain.add_window(st, 0, t_end)
            plain.run()
            plain.saif(w)
        torch.cuda.synchronize()
        plain_s = time.perf_counter() - t0
    plain.close()
    line = {
        "metric": "gate-events/s", "value": gate_ev / dev_s, "unit": "gate-events/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * dev_s, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": workload_desc(args), "seed": args.seed, "windows": n_win,
                   "cycles": int(lengths.sum()), "alloc": args.alloc, "parallelism": "replicas x1",
                   "l2": "every step streams GBs of event pool per window (> L2)",
                   "schedule": tune["best"], "value_timing": "device time of the waves (stimulus uploads "
                   "between waves excluded); e2e: wall clock of add_window + run_batched + SAIF reads"},
        "sim_cycles_per_s": float(lengths.sum()) / dev_s,
        "gate_events_per_step": gate_ev,
        "e2e": {"value": gate_ev / step_s, "unit": "gate-events/s",
                "h2d_bytes_per_step": int(sum(st.time.nbytes + st.value.nbytes for st, _ in wins)),
                "d2h_bytes_per_step": int(24 * nl.n_nets * n_win), "ms_per_step": 1000.0 * step_s},
        "plain_sequential": {"value": gate_ev / plain_s, "unit": "gate-events/s", "ms": 1000.0 * plain_s,
                             "what": f"{n_win} sequential gls_run calls, exact allocation, wall clock"},
        "batched_over_plain": plain_s / step_s,
        "gpu_launches": int(launches),
        "pool_bytes": pool_b,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gls", choices=["gls", "reference"])
    ap.add_argument("--config", default="c2", choices=sorted(WORKLOADS))
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--seg", type=int, default=0, help="fan-in events per time segment (0 = library default)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--alloc", default="bound", choices=["bound", "exact", "learned"],
                    help="gate-output slot allocation: upper bound, exact, or learned presize")
    ap.add_argument("--model", default=None, help="presize model (.npz) for --alloc learned")
    ap.add_argument("--cells", type=int, default=None, help="override the cell count (profiling cases)")
    ap.add_argument("--depth", type=int, default=None, help="override the logic depth (profiling cases)")
    ap.add_argument("--cycles", type=int, default=None, help="override the cycle count (profiling cases)")
    ap.add_argument("--windows", type=int, default=None, help="c4: number of windows (default 256)")
    ap.add_argument("--schedule", default=None,
                    help="c1-c3: fixed schedule 'segments_per_sm,warp_mask,flags' instead of autotuning")
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
