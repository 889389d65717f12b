"""The levelization against the reference's own code: GenerateAdjacencyList,
SetInDegrees and TopologyOrder of src/process.cpp:90-176, compiled from the
reference sources (oracle/_ref/ref_levels), on random instance graphs and a
generated netlist.  Checked here: the Python restatement (gls/levelize.py)
and the command-line tool's host path (gls_process); tests/test_gpu_levelize
checks gls_levelize on the GPU the same way."""
import subprocess

import numpy as np
import pytest

from gls import files, synth
from gls.levelize import levelize


def random_instances(seed, n, max_in=4):
    """Random acyclic instance list: instance i reads nets driven by other
    instances placed before it topologically, or primary inputs; the
    instance order is shuffled, inputs may repeat, some instances drive two
    outputs."""
    rng = np.random.default_rng(seed)
    n_pi = 16
    perm = rng.permutation(n)
    outs = [None] * n
    net = n_pi
    avail = list(range(n_pi))
    ins = [None] * n
    for k in range(n):
        i = int(perm[k])
        m = int(rng.integers(1, max_in + 1))
        ins[i] = [int(avail[int(x)]) for x in rng.integers(0, len(avail), m)]
        no = 2 if rng.random() < 0.1 else 1
        outs[i] = list(range(net, net + no))
        avail += outs[i]
        net += no
    return ins, outs


@pytest.fixture(scope="module")
def ref_levels():
    from oracle import build
    if build.build_reference() is None or not build.REF_LEVELS_BIN.exists():
        pytest.skip("reference sources not available on this machine")
    return build.REF_LEVELS_BIN


def reference_levels(exe, ins, outs, tmp_path):
    lines = [str(len(ins))]
    for i, (a, b) in enumerate(zip(ins, outs)):
        lines.append(" ".join([f"U{i}", str(len(b)), *(f"n{x}" for x in b), str(len(a)), *(f"n{x}" for x in a)]))
    p = tmp_path / "inst.txt"
    p.write_text("\n".join(lines) + "\n")
    r = subprocess.run([str(exe), str(p)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return [[int(x) for x in line.split()] for line in r.stdout.splitlines()]


@pytest.mark.parametrize("seed", range(6))
def test_kahn_restatement_matches_reference(seed, ref_levels, tmp_path):
    ins, outs = random_instances(seed, 200 + 300 * seed)
    assert levelize(ins, outs) == reference_levels(ref_levels, ins, outs, tmp_path)


def test_process_tool_levels_match_reference(ref_levels, tmp_path):
    """gls_process's host levelization on a generated netlist written as
    files (instances shuffled in the file, so that the file order is not a
    topological order)."""
    from gls import hostbuild
    cfg = synth.scaled(synth.CONFIGS["c1"], cells=1500, cycles=10, depth=25)
    nl = synth.make_netlist(cfg, 41)
    order = np.random.default_rng(3).permutation(nl.n_inst)
    files.write_vlib(tmp_path / "lib.vlib")
    files.write_gv(tmp_path / "d.gv", nl, order=order)
    files.write_sdf(tmp_path / "d.sdf", nl)
    exe = hostbuild.build()["gls_process"]
    r = subprocess.run([str(exe), "--native", str(tmp_path / "lib.vlib"), str(tmp_path / "d.gv"),
                        str(tmp_path / "d.sdf"), str(tmp_path / "i.dat")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    it = files.read_inter(tmp_path / "i.dat")
    # the file's instance ids are positions in the written order
    ins = [nl.inputs_of(int(i)).tolist() for i in order]
    outs = [nl.outputs_of(int(i)).tolist() for i in order]
    ref = reference_levels(ref_levels, ins, outs, tmp_path)
    pos = {nl.inst_name(int(i)): k for k, i in enumerate(order)}
    got = []
    for L in range(len(it["level_start"]) - 1):
        got.append([pos[it["insts"][k][0]] for k in range(it["level_start"][L], it["level_start"][L + 1])])
    assert got == ref
