"""gls_pack_levels: the packed per-level arrays that the reference's
`process` archives for its GPU simulator (src/process.cpp:423-566), on the
GPU, against a line-by-line restatement of that loop (`pack_ref` below),
and `gls_process --gpu-pack` against its host packing: the same archive,
byte for byte."""
import subprocess

import numpy as np
import pytest

from gls import files, synth
from gls.capi import PACK_ARC_DTYPE, pack_levels_gpu

pytestmark = pytest.mark.gpu


def pack_ref(level_start, n_in, n_out, arcs, rows):
    """src/process.cpp:423-566 for instances in level order: arcs[i] is a
    list of (edge, in_pos, out_pos, rise, fall), rows[i] a list of rows."""
    nl = len(level_start) - 1
    n = len(n_in)
    r = {k: [0] * nl for k in ("data_in_num_start", "data_out_num_start", "delay_start", "delay_width",
                               "functions_start", "functions_width")}
    r.update({k: [0] * n for k in ("data_in_num", "data_out_num", "val_num_start", "delay_val_num",
                                   "functions_func_num", "functions_val_num")})
    s = ds = fs = 0
    for L in range(nl):
        lv = range(level_start[L], level_start[L + 1])
        vw = dw = fw = 0
        r["data_in_num_start"][L] = r["data_out_num_start"][L] = s
        r["functions_start"][L], r["delay_start"][L] = fs, ds
        for j, i in enumerate(lv):
            r["data_in_num"][j + s], r["data_out_num"][j + s] = n_in[i], n_out[i]
            r["val_num_start"][j + s] = vw
            vw += n_in[i]
            r["delay_val_num"][j + s] = len(arcs[i])
            dw = max(dw, len(arcs[i]))
            w = max([len(x) for x in rows[i]], default=0)
            fw = max(fw, w * len(rows[i]))
            r["functions_func_num"][j + s], r["functions_val_num"][j + s] = len(rows[i]), w
        s += len(lv)
        ds += len(lv) * dw
        fs += len(lv) * fw
        r["delay_width"][L], r["functions_width"][L] = dw, fw
    d = {k: [0] * ds for k in ("host_delay_edges", "host_in_bit", "host_out_bit", "host_rise_val", "host_fall_val")}
    f = [0] * fs
    for L in range(nl):
        dw, fw = r["delay_width"][L], r["functions_width"][L]
        for j, i in enumerate(range(level_start[L], level_start[L + 1])):
            for k in range(dw):
                at = r["delay_start"][L] + j * dw + k
                e = arcs[i][k] if k < len(arcs[i]) else (-1, -1, -1, -1.0, -1.0)
                for key, x in zip(("host_delay_edges", "host_in_bit", "host_out_bit", "host_rise_val",
                                   "host_fall_val"), e):
                    d[key][at] = x
            h = len(rows[i])
            w = fw // h if h else 0
            for rr in range(h):
                for k in range(w):
                    f[r["functions_start"][L] + j * fw + rr * w + k] = rows[i][rr][k] if k < len(rows[i][rr]) else -1
            for k in range(w * h, fw):
                f[r["functions_start"][L] + j * fw + k] = -1
    r.update(d)
    r["host_functions"] = f
    return r


def random_design(seed, n_levels=9, max_level=40):
    rng = np.random.default_rng(seed)
    sizes = rng.integers(0, max_level + 1, n_levels)
    sizes[rng.integers(0, n_levels)] = 0          # an empty level
    level_start = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint32)
    n = int(level_start[-1])
    n_in = rng.integers(0, 7, n)
    n_out = rng.integers(1, 3, n)
    arcs, rows = [], []
    for i in range(n):
        na = int(rng.integers(0, 9)) if rng.random() > 0.15 else 0
        arcs.append([(int(rng.integers(0, 3)), int(rng.integers(0, n_in[i] + 1)), int(rng.integers(0, n_out[i] + 1)),
                      float(np.float32(rng.random() * 90)), float(np.float32(rng.random() * 90))) for _ in range(na)])
        nr = int(rng.integers(0, 5)) if rng.random() > 0.1 else 0
        rows.append([[int(x) for x in rng.integers(0, 12, rng.integers(1, 6))] for _ in range(nr)])
    return level_start, n_in, n_out, arcs, rows


def run_gpu(level_start, n_in, n_out, arcs, rows):
    arc_start = np.concatenate([[0], np.cumsum([len(a) for a in arcs])]).astype(np.uint32)
    flat = np.zeros(int(arc_start[-1]), PACK_ARC_DTYPE)
    k = 0
    for a in arcs:
        for e, ip, op, rs, fl in a:
            flat[k] = (e, ip, op, 0, rs, fl)
            k += 1
    row_start = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.uint32)
    all_rows = [row for r in rows for row in r]
    entry_start = np.concatenate([[0], np.cumsum([len(x) for x in all_rows])]).astype(np.uint32)
    entries = np.array([v for x in all_rows for v in x], np.int16)
    return pack_levels_gpu(level_start, n_in, n_out, arc_start, flat, row_start, entry_start, entries)


@pytest.mark.parametrize("seed", range(6))
def test_gpu_pack_matches_restatement(seed, gpu):
    case = random_design(seed, n_levels=3 + 4 * seed, max_level=10 + 60 * seed)
    exp = pack_ref(*case)
    got = run_gpu(*case)
    for key, want in exp.items():
        g = got[key]
        assert len(g) == len(want), key
        if key in ("host_rise_val", "host_fall_val"):
            assert np.array_equal(g, np.array(want, np.float32)), key
        else:
            assert np.array_equal(g.astype(np.int64), np.array(want, np.int64)), key


def test_gpu_pack_large_and_edge_shapes(gpu):
    """A level wider than one scan tile (4,096 instances) so that the tile
    offsets carry, and designs without any arc or function row."""
    case = random_design(99, n_levels=4, max_level=9000)
    exp, got = pack_ref(*case), run_gpu(*case)
    for key in ("val_num_start", "delay_start", "functions_start", "host_functions", "host_in_bit"):
        assert np.array_equal(got[key].astype(np.int64), np.array(exp[key], np.int64)), key
    ls = np.array([0, 3, 3, 5], np.uint32)
    bare = (ls, [1, 2, 0, 3, 1], [1, 1, 1, 2, 1], [[] for _ in range(5)], [[] for _ in range(5)])
    exp, got = pack_ref(*bare), run_gpu(*bare)
    assert len(got["host_functions"]) == 0 and len(got["host_delay_edges"]) == 0
    assert got["val_num_start"].tolist() == exp["val_num_start"] == [0, 1, 3, 0, 3]


@pytest.fixture(scope="module")
def tools(libgls):
    from gls import hostbuild
    return hostbuild.build()


def process(tools, d, out, *extra):
    r = subprocess.run([str(tools["gls_process"]), *extra, str(d / "lib.vlib"), str(d / "d.gv"), str(d / "d.sdf"),
                        str(d / out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    return (d / out).read_bytes(), r.stdout


@pytest.mark.parametrize("which", ["generated", "buses_aliases_open_output"])
def test_process_gpu_pack_writes_the_same_archive(which, tools, tmp_path):
    files.write_vlib(tmp_path / "lib.vlib")
    if which == "generated":
        cfg = synth.scaled(synth.CONFIGS["c1"], cells=3000, cycles=10, depth=14)
        nl = synth.make_netlist(cfg, 21)
        files.write_gv(tmp_path / "d.gv", nl)
        files.write_sdf(tmp_path / "d.sdf", nl)
    else:
        from test_gpu_cli import GV, SDF
        (tmp_path / "d.gv").write_text(GV)
        (tmp_path / "d.sdf").write_text(SDF)
    host, log_h = process(tools, tmp_path, "h.dat")
    gpu, log_g = process(tools, tmp_path, "g.dat", "--gpu-pack")
    both, _ = process(tools, tmp_path, "b.dat", "--gpu-levelize", "--gpu-pack")
    assert "level packing done on the host" in log_h and "level packing done on the GPU" in log_g
    assert host == gpu == both
