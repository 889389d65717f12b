"""GPU levelization (gls_levelize) against the Kahn levelization of the
reference (restated in gls/levelize.py, src/process.cpp:90-176), and the
gls_process tool with --gpu-levelize against its host path."""
import subprocess

import numpy as np
import pytest

from gls import files, synth
from gls.capi import GlsError, levelize_gpu, netlist_preds
from gls.levelize import levelize

pytestmark = pytest.mark.gpu


def random_instances(seed, n, max_in=4, loop=False):
    """Random instance list: instance i reads nets driven by earlier
    instances or primary inputs (a DAG), in shuffled instance order."""
    rng = np.random.default_rng(seed)
    n_pi = 16
    perm = rng.permutation(n)               # instance order differs from topological order
    out_of = {int(perm[k]): [n_pi + k] for k in range(n)}
    in_nets = [None] * n
    for k in range(n):
        avail = n_pi + k
        m = int(rng.integers(1, max_in + 1))
        in_nets[int(perm[k])] = [int(x) for x in rng.integers(0, avail, m)]   # repeats allowed
    out_nets = [out_of[i] for i in range(n)]
    if loop:   # the last two instances in topological order read each other's output
        in_nets[int(perm[n - 2])].append(n_pi + n - 1)
        in_nets[int(perm[n - 1])].append(n_pi + n - 2)
    return in_nets, out_nets


@pytest.mark.parametrize("seed", range(6))
def test_gpu_levels_match_kahn(seed, gpu):
    in_nets, out_nets = random_instances(seed, 300 + 200 * seed)
    ref = levelize(in_nets, out_nets)
    order, level_start = levelize_gpu(*netlist_preds(in_nets, out_nets))
    assert len(level_start) == len(ref) + 1
    for k, lv in enumerate(ref):
        assert order[level_start[k]:level_start[k + 1]].tolist() == lv, f"level {k}"


def test_gpu_levels_of_a_generated_netlist(gpu):
    """The generator's netlists are in level order already: the levels come
    back as they are, with every level in instance order."""
    cfg = synth.scaled(synth.CONFIGS["c2"], cells=60000, depth=30)
    nl = synth.make_netlist(cfg, 5)
    ins = [nl.inputs_of(i).tolist() for i in range(nl.n_inst)]
    outs = [nl.outputs_of(i).tolist() for i in range(nl.n_inst)]
    order, level_start = levelize_gpu(*netlist_preds(ins, outs))
    assert np.array_equal(level_start, nl.level_start)
    assert np.array_equal(order, np.arange(nl.n_inst))


def test_gpu_levelize_rejects_loops_and_bad_tables(gpu):
    in_nets, out_nets = random_instances(11, 200, loop=True)
    with pytest.raises(GlsError):
        levelize_gpu(*netlist_preds(in_nets, out_nets))
    with pytest.raises(GlsError):                     # an instance reading its own output
        levelize_gpu(np.array([0, 1], np.uint64), np.array([0], np.uint32))
    with pytest.raises(GlsError):                     # a predecessor out of range
        levelize_gpu(np.array([0, 1, 1], np.uint64), np.array([7], np.uint32))
    with pytest.raises(GlsError):                     # a start table that decreases
        levelize_gpu(np.array([0, 2, 1], np.uint64), np.array([1, 1], np.uint32))
    order, level_start = levelize_gpu(np.array([0], np.uint64), np.array([], np.uint32))
    assert len(order) == 0 and level_start.tolist() == [0]


def test_gls_process_gpu_levelize_writes_the_same_file(libgls, tmp_path):
    from gls import hostbuild
    tools = hostbuild.build()
    cfg = synth.scaled(synth.CONFIGS["c1"], cells=1500, cycles=50, depth=16)
    nl = synth.make_netlist(cfg, 21)
    files.write_vlib(tmp_path / "lib.vlib")
    files.write_gv(tmp_path / "d.gv", nl)
    files.write_sdf(tmp_path / "d.sdf", nl)
    outs = {}
    for flag in ([], ["--gpu-levelize"]):
        dst = tmp_path / f"inter{len(flag)}.dat"
        r = subprocess.run([str(tools["gls_process"]), *flag, str(tmp_path / "lib.vlib"), str(tmp_path / "d.gv"),
                            str(tmp_path / "d.sdf"), str(dst)], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout
        outs[len(flag)] = dst.read_bytes()
    assert outs[0] == outs[1]


@pytest.mark.parametrize("seed", range(4))
def test_gpu_levels_match_reference_code(seed, gpu, tmp_path):
    """gls_levelize against the reference's own TopologyOrder
    (src/process.cpp:90-176, compiled from the reference sources)."""
    from oracle import build
    from test_levelize_reference import random_instances, reference_levels
    if build.build_reference() is None or not build.REF_LEVELS_BIN.exists():
        pytest.skip("reference sources not available on this machine")
    ins, outs = random_instances(100 + seed, 500 + 500 * seed)
    ref = reference_levels(build.REF_LEVELS_BIN, ins, outs, tmp_path)
    order, level_start = levelize_gpu(*netlist_preds(ins, outs))
    assert [order[level_start[k]:level_start[k + 1]].tolist() for k in range(len(level_start) - 1)] == ref
