"""ctypes binding of the C ABI declared in include/gls.h.

This is the reference-facing boundary: `Simulator` mirrors the reference's
simulate stage (load the levelized netlist, take a stimulus window, run the
levels, read SAIF counts and waveforms).  There is no CPU fallback: if
libgls.so is missing or no CUDA device is present, calls raise.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .netlist import Netlist, Stimulus

LIB_PATH = Path(__file__).resolve().parent.parent / "lib" / "libgls.so"

GLS_OK, GLS_EINVAL, GLS_ECUDA, GLS_ENOMEM, GLS_ESTATE, GLS_ERANGE, GLS_EOVERFLOW = range(7)
CALC_FIXED, CALC_LITERAL = 0, 1
ALLOC_BOUND, ALLOC_EXACT, ALLOC_LEARNED = 0, 1, 2
MLP_IN, MLP_HID = 32, 128
MLP_PARAMS = MLP_HID * MLP_IN + MLP_HID + MLP_HID * MLP_HID + MLP_HID + MLP_HID + 1

# every symbol include/gls.h declares
EXPORTED = ["gls_create", "gls_destroy", "gls_last_error", "gls_load_netlist", "gls_add_window",
            "gls_clear_windows", "gls_run", "gls_saif_counts", "gls_saif_table", "gls_waveform_lengths", "gls_waveform",
            "gls_stats_get", "gls_cell_lut", "gls_abi_version", "gls_run_level_static",
            "gls_set_presize_model", "gls_presize_samples", "gls_presize_predict", "gls_trainer_create",
            "gls_trainer_destroy", "gls_trainer_error", "gls_trainer_set_data", "gls_trainer_fit",
            "gls_trainer_grad", "gls_trainer_get_params", "gls_trainer_set_params", "gls_run_batched",
            "gls_autotune", "gls_set_schedule", "gls_levelize", "gls_vcd_scan", "gls_vcd_free", "gls_pack_levels"]


class GlsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gls error {code}: {msg}")
        self.code = code


class Opts(C.Structure):
    _fields_ = [("device", C.c_int), ("calc_mode", C.c_int), ("alloc_mode", C.c_int),
                ("delay_factor", C.c_double), ("seg_events", C.c_uint32), ("pool_events", C.c_uint64),
                ("stream", C.c_void_p), ("profile", C.c_int)]


class NetlistC(C.Structure):
    _fields_ = [("n_nets", C.c_uint32), ("n_cells", C.c_uint32), ("cells", C.c_void_p),
                ("n_prims", C.c_uint32), ("prims", C.c_void_p), ("n_inst", C.c_uint32),
                ("n_levels", C.c_uint32), ("level_start", C.c_void_p), ("inst_cell", C.c_void_p),
                ("inst_pin_start", C.c_void_p), ("inst_pin_net", C.c_void_p),
                ("inst_arc_start", C.c_void_p), ("arcs", C.c_void_p)]


class StimulusC(C.Structure):
    _fields_ = [("n_nets", C.c_uint32), ("net", C.c_void_p), ("ev_start", C.c_void_p),
                ("time", C.c_void_p), ("value", C.c_void_p)]


class Stats(C.Structure):
    _fields_ = [("gate_events", C.c_uint64), ("output_events", C.c_uint64), ("segments", C.c_uint64),
                ("pool_events", C.c_uint64), ("pool_bytes", C.c_uint64), ("overflow_retries", C.c_uint64),
                ("kernel_ms", C.c_double), ("launches", C.c_uint32), ("n_windows", C.c_uint32),
                ("plan_ms", C.c_double), ("sim_ms", C.c_double), ("combine_ms", C.c_double),
                ("stim_ms", C.c_double), ("fanin_bytes", C.c_uint64), ("presize_overflows", C.c_uint64),
                ("pool_used", C.c_uint64), ("wide_windows", C.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchOpts(C.Structure):
    _fields_ = [("max_wave", C.c_uint32), ("use_graph", C.c_int), ("saif_only", C.c_int)]


class TuneResult(C.Structure):
    _fields_ = [("n", C.c_uint32), ("best", C.c_uint32), ("windows", C.c_uint32),
                ("seg_per_sm", C.c_uint32 * 32), ("warp_mask", C.c_uint32 * 32), ("flags", C.c_uint32 * 32),
                ("ms", C.c_float * 32)]


class PresizeModel(C.Structure):
    _fields_ = [("params", C.c_float * MLP_PARAMS), ("margin", C.c_float), ("slack", C.c_uint32)]


class TrainOpts(C.Structure):
    _fields_ = [("batch", C.c_uint32), ("epochs", C.c_uint32), ("lr", C.c_float), ("huber", C.c_float),
                ("seed", C.c_uint64)]


def presize_model(params: np.ndarray, margin: float = 0.25, slack: int = 8) -> PresizeModel:
    m = PresizeModel()
    p = np.ascontiguousarray(params, np.float32)
    if p.shape != (MLP_PARAMS,):
        raise ValueError(f"presize parameters: {MLP_PARAMS} floats expected, got {p.shape}")
    C.memmove(m.params, p.ctypes.data, p.nbytes)
    m.margin = margin
    m.slack = slack
    return m


_lib = None


def load_library(path: Path | None = None) -> C.CDLL:
    """Load libgls.so (raises if it was not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: run __graft_entry__.build() (libgls is required, no fallback)")
    lib = C.CDLL(str(p))
    lib.gls_last_error.restype = C.c_char_p
    lib.gls_last_error.argtypes = [C.c_void_p]
    lib.gls_create.argtypes = [C.POINTER(Opts), C.POINTER(C.c_void_p)]
    lib.gls_destroy.argtypes = [C.c_void_p]
    lib.gls_load_netlist.argtypes = [C.c_void_p, C.POINTER(NetlistC)]
    lib.gls_add_window.argtypes = [C.c_void_p, C.POINTER(StimulusC), C.c_uint64, C.c_uint64,
                                   C.POINTER(C.c_uint32)]
    lib.gls_clear_windows.argtypes = [C.c_void_p]
    lib.gls_run.argtypes = [C.c_void_p]
    lib.gls_saif_counts.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.gls_saif_table.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p]
    lib.gls_waveform_lengths.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p]
    lib.gls_waveform.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint64,
                                 C.POINTER(C.c_uint64)]
    lib.gls_stats_get.argtypes = [C.c_void_p, C.POINTER(Stats)]
    lib.gls_cell_lut.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_uint32]
    lib.gls_abi_version.restype = C.c_int
    lib.gls_run_level_static.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint64,
                                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint64]
    lib.gls_run_batched.argtypes = [C.c_void_p, C.POINTER(BatchOpts)]
    lib.gls_autotune.argtypes = [C.c_void_p, C.POINTER(BatchOpts), C.POINTER(TuneResult)]
    lib.gls_set_schedule.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32]
    lib.gls_levelize.argtypes = [C.c_int, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.gls_vcd_scan.argtypes = [C.c_int, C.c_char_p, C.c_uint64, C.c_void_p, C.c_void_p]
    lib.gls_vcd_free.argtypes = [C.c_void_p]
    lib.gls_vcd_free.restype = None
    lib.gls_set_presize_model.argtypes = [C.c_void_p, C.POINTER(PresizeModel)]
    lib.gls_presize_samples.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint64,
                                        C.POINTER(C.c_uint64)]
    lib.gls_presize_predict.argtypes = [C.c_void_p, C.POINTER(PresizeModel), C.c_void_p, C.c_uint64, C.c_void_p,
                                        C.c_int]
    lib.gls_trainer_create.argtypes = [C.c_int, C.c_uint64, C.POINTER(C.c_void_p)]
    lib.gls_trainer_destroy.argtypes = [C.c_void_p]
    lib.gls_trainer_error.restype = C.c_char_p
    lib.gls_trainer_error.argtypes = [C.c_void_p]
    lib.gls_trainer_set_data.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64]
    lib.gls_trainer_fit.argtypes = [C.c_void_p, C.POINTER(TrainOpts), C.c_void_p]
    lib.gls_trainer_grad.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_float, C.c_void_p, C.c_void_p]
    lib.gls_trainer_get_params.argtypes = [C.c_void_p, C.c_void_p]
    lib.gls_trainer_set_params.argtypes = [C.c_void_p, C.c_void_p]
    if path is None:
        _lib = lib
    return lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def cell_lut(cell_rec: np.ndarray, prims: np.ndarray, out: int, calc_mode: int) -> np.ndarray:
    """Truth table of one cell output (host helper, no GPU needed)."""
    from .netlist import CELL_DTYPE

    lib = load_library()
    rec = np.zeros(1, CELL_DTYPE)
    rec[0] = cell_rec
    rec["prim_start"] = 0
    n = 1 << (2 * int(rec["n_in"][0]))
    lut = np.zeros(n, np.uint8)
    rc = lib.gls_cell_lut(_ptr(rec), _ptr(np.ascontiguousarray(prims)), out, calc_mode, _ptr(lut), n)
    if rc:
        raise GlsError(rc, "gls_cell_lut")
    return lut


def levelize_gpu(pred_start: np.ndarray, pred: np.ndarray, device: int = 0):
    """Kahn levels on the GPU (gls_levelize): pred_start[n + 1] / pred[] list
    every instance's predecessor instances.  Returns (order, level_start):
    the instances level by level in instance order, and every level's first
    position followed by n.  Raises GlsError on a combinational loop."""
    lib = load_library()
    ps = np.ascontiguousarray(pred_start, np.uint64)
    pr = np.ascontiguousarray(pred, np.uint32)
    n = len(ps) - 1
    order = np.zeros(max(n, 1), np.uint32)
    level_start = np.zeros(n + 1, np.uint32)
    nl = C.c_uint32(0)
    rc = lib.gls_levelize(device, n, _ptr(ps), _ptr(pr) if len(pr) else None, _ptr(order), _ptr(level_start),
                          C.byref(nl))
    if rc:
        raise GlsError(rc, "gls_levelize: malformed predecessor table or combinational loop")
    return order[:n], level_start[: nl.value + 1]


PACK_ARC_DTYPE = np.dtype([("edge", "<i2"), ("in_pos", "<i2"), ("out_pos", "<i2"), ("pad", "<i2"),
                           ("rise", "<f4"), ("fall", "<f4")])


class PackIn(C.Structure):
    _fields_ = [("n_levels", C.c_uint32), ("n_inst", C.c_uint32)] + \
               [(f, C.c_void_p) for f in ("level_start", "n_in", "n_out", "arc_start", "arcs", "row_start",
                                          "entry_start", "entries")]


PACK_LEVEL = ("data_in_num_start", "data_out_num_start", "delay_start", "delay_width", "functions_start",
              "functions_width")
PACK_INST = (("data_in_num", np.int16), ("data_out_num", np.int16), ("val_num_start", np.uint32),
             ("delay_val_num", np.int16), ("functions_func_num", np.int16), ("functions_val_num", np.int16))
PACK_DELAY = (("delay_edges", np.int16), ("in_bit", np.int16), ("out_bit", np.int16), ("rise_val", np.float32),
              ("fall_val", np.float32))


class PackOut(C.Structure):
    _fields_ = [(f, C.c_void_p) for f in PACK_LEVEL] + [(f, C.c_void_p) for f, _ in PACK_INST] + \
               [(f, C.c_void_p) for f, _ in PACK_DELAY] + [("functions", C.c_void_p)] + \
               [(f, C.c_uint64) for f in ("delay_cap", "functions_cap", "delay_total", "functions_total")]


def pack_levels_gpu(level_start, n_in, n_out, arc_start, arcs, row_start, entry_start, entries, device: int = 0):
    """The reference's packed per-level arrays (gls_pack_levels) of
    instances in level order; returns a dict of numpy arrays named as the
    reference's fields (host_* for the padded tables).  The first call
    sizes the padded tables, the second fills them."""
    lib = load_library()
    lib.gls_pack_levels.argtypes = [C.c_int, C.POINTER(PackIn), C.POINTER(PackOut)]
    keep = dict(level_start=np.ascontiguousarray(level_start, np.uint32), n_in=np.ascontiguousarray(n_in, np.uint16),
                n_out=np.ascontiguousarray(n_out, np.uint16), arc_start=np.ascontiguousarray(arc_start, np.uint32),
                arcs=np.ascontiguousarray(arcs, PACK_ARC_DTYPE), row_start=np.ascontiguousarray(row_start, np.uint32),
                entry_start=np.ascontiguousarray(entry_start, np.uint32),
                entries=np.ascontiguousarray(entries, np.int16))
    nl, n = len(keep["level_start"]) - 1, len(keep["n_in"])
    pin = PackIn(nl, n, *[_ptr(keep[f]) if len(keep[f]) else None for f in
                          ("level_start", "n_in", "n_out", "arc_start", "arcs", "row_start", "entry_start",
                           "entries")])
    res = {f: np.zeros(max(nl, 1), np.uint32) for f in PACK_LEVEL}
    res.update({f: np.zeros(max(n, 1), t) for f, t in PACK_INST})
    out = PackOut()
    for f in PACK_LEVEL + tuple(f for f, _ in PACK_INST):
        setattr(out, f, _ptr(res[f]))
    rc = lib.gls_pack_levels(device, C.byref(pin), C.byref(out))
    if rc == GLS_EOVERFLOW:   # the padded tables' sizes are known now
        nd, nf = out.delay_total, out.functions_total
        for f, t in PACK_DELAY:
            res[f] = np.zeros(max(nd, 1), t)
            setattr(out, f, _ptr(res[f]))
        res["functions"] = np.zeros(max(nf, 1), np.int16)
        out.functions = _ptr(res["functions"])
        out.delay_cap, out.functions_cap = nd, nf
        rc = lib.gls_pack_levels(device, C.byref(pin), C.byref(out))
    if rc:
        raise GlsError(rc, "gls_pack_levels")
    nd, nf = out.delay_total, out.functions_total
    r = {f: res[f][:nl] for f in PACK_LEVEL}
    r.update({f: res[f][:n] for f, _ in PACK_INST})
    r.update({"host_" + f if f in ("delay_edges", "in_bit", "out_bit", "rise_val", "fall_val") else f:
              res[f][:nd] if f in res else np.zeros(0, t) for f, t in PACK_DELAY})
    r["host_functions"] = res["functions"][:nf] if "functions" in res else np.zeros(0, np.int16)
    return r


class VcdIds(C.Structure):
    _fields_ = [("n_ids", C.c_uint32), ("key", C.c_void_p), ("var_start", C.c_void_p), ("bit_start", C.c_void_p),
                ("bits", C.c_void_p), ("bus", C.c_void_p)]


class VcdChanges(C.Structure):
    _fields_ = [("n", C.c_uint64), ("signal", C.POINTER(C.c_uint32)), ("time", C.POINTER(C.c_uint64)),
                ("value", C.POINTER(C.c_uint8)), ("bus", C.POINTER(C.c_uint8)), ("fallback", C.c_int)]


def vcd_scan(body: bytes, codes: dict[str, list[tuple[list[int], bool]]], device: int = 0):
    """Bit changes of a VCD body on the GPU (gls_vcd_scan).  codes: identifier
    code -> declarations (bit signals msb first, bus flag).  Returns
    (signal, time, value, bus, fallback) in file order."""
    lib = load_library()
    keyed = []
    for code, decls in codes.items():
        b = code.encode()
        if not 0 < len(b) <= 8:
            raise ValueError("identifier codes of 1 to 8 bytes")
        keyed.append((int.from_bytes(b, "little"), decls))
    keyed.sort(key=lambda x: x[0])
    key = np.array([k for k, _ in keyed], np.uint64)
    var_start, bit_start, bits, bus = [0], [0], [], []
    for _, decls in keyed:
        for sig, is_bus in decls:
            bits.extend(sig)
            bit_start.append(len(bits))
            bus.append(1 if is_bus else 0)
        var_start.append(len(bus))
    arrs = [key, np.array(var_start, np.uint32), np.array(bit_start, np.uint32), np.array(bits, np.uint32),
            np.array(bus, np.uint8)]
    ids = VcdIds(len(key), *[_ptr(a) if len(a) else None for a in arrs])
    out = VcdChanges()
    buf = C.create_string_buffer(body, len(body))
    rc = lib.gls_vcd_scan(device, buf, len(body), C.byref(ids), C.byref(out))
    if rc:
        raise GlsError(rc, "gls_vcd_scan")
    try:
        n = int(out.n)
        take = lambda p, dt: np.ctypeslib.as_array(p, (n,)).astype(dt) if n else np.zeros(0, dt)
        return (take(out.signal, np.uint32), take(out.time, np.uint64), take(out.value, np.uint8),
                take(out.bus, np.uint8), bool(out.fallback))
    finally:
        lib.gls_vcd_free(C.byref(out))


def netlist_preds(in_nets: list[list[int]], out_nets: list[list[int]]):
    """Predecessor table of an instance list: the instances driving each
    instance's input nets (the edges of src/process.cpp:90-114)."""
    driver: dict[int, int] = {}
    for i, outs in enumerate(out_nets):
        for net in outs:
            driver[net] = i
    starts, preds = [0], []
    for ins in in_nets:
        ps = sorted({driver[n] for n in ins if n in driver})
        preds.extend(ps)
        starts.append(len(preds))
    return np.array(starts, np.uint64), np.array(preds, np.uint32)


class Simulator:
    """One libgls context on one GPU: the simulate stage behind a C ABI."""

    def __init__(self, device: int = 0, calc_mode: int = CALC_FIXED, seg_events: int = 0,
                 pool_events: int = 0, delay_factor: float = 1.0, stream: int | None = None,
                 alloc_mode: int = ALLOC_BOUND, profile: bool = False):
        self.lib = load_library()
        o = Opts(device, calc_mode, alloc_mode, delay_factor, seg_events, pool_events, stream or None,
                 1 if profile else 0)
        h = C.c_void_p()
        rc = self.lib.gls_create(C.byref(o), C.byref(h))
        if rc:
            raise GlsError(rc, "gls_create failed (no CUDA device?)")
        self.h = h
        self.n_nets = 0
        self._keep = []

    def _check(self, rc: int, what: str):
        if rc:
            raise GlsError(rc, f"{what}: {self.lib.gls_last_error(self.h).decode()}")

    def close(self):
        if self.h:
            self.lib.gls_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def load(self, nl: Netlist):
        cells, prims = nl.cell_arrays()
        arrs = dict(
            cells=np.ascontiguousarray(cells), prims=np.ascontiguousarray(prims),
            level_start=np.ascontiguousarray(nl.level_start, np.uint32),
            inst_cell=np.ascontiguousarray(nl.inst_cell, np.uint32),
            pin_start=np.ascontiguousarray(nl.pin_start, np.uint32),
            pin_net=np.ascontiguousarray(nl.pin_net, np.uint32),
            arc_start=np.ascontiguousarray(nl.arc_start, np.uint32),
            arcs=np.ascontiguousarray(nl.arcs) if len(nl.arcs) else np.zeros(1, nl.arcs.dtype),
        )
        c = NetlistC(nl.n_nets, len(cells), _ptr(arrs["cells"]), len(prims), _ptr(arrs["prims"]), nl.n_inst,
                     nl.n_levels, _ptr(arrs["level_start"]), _ptr(arrs["inst_cell"]), _ptr(arrs["pin_start"]),
                     _ptr(arrs["pin_net"]), _ptr(arrs["arc_start"]), _ptr(arrs["arcs"]))
        self._check(self.lib.gls_load_netlist(self.h, C.byref(c)), "load_netlist")
        self.n_nets = nl.n_nets

    def add_window(self, st: Stimulus, t_begin: int, t_end: int) -> int:
        nets = np.ascontiguousarray(st.nets, np.uint32)
        evs = np.ascontiguousarray(st.ev_start, np.uint64)
        tm = np.ascontiguousarray(st.time, np.uint32)
        vl = np.ascontiguousarray(st.value, np.uint8)
        s = StimulusC(len(nets), _ptr(nets), _ptr(evs), _ptr(tm) if len(tm) else None,
                      _ptr(vl) if len(vl) else None)
        wid = C.c_uint32()
        self._check(self.lib.gls_add_window(self.h, C.byref(s), t_begin, t_end, C.byref(wid)), "add_window")
        return wid.value

    def clear_windows(self):
        self._check(self.lib.gls_clear_windows(self.h), "clear_windows")

    def run(self):
        self._check(self.lib.gls_run(self.h), "run")

    def run_batched(self, max_wave: int = 0, use_graph: bool = True, saif_only: bool = False):
        """All added windows in waves, each level one launch per kernel over a wave."""
        o = BatchOpts(max_wave, 1 if use_graph else 0, 1 if saif_only else 0)
        self._check(self.lib.gls_run_batched(self.h, C.byref(o)), "run_batched")

    def autotune(self, max_wave: int = 0, use_graph: bool = True, saif_only: bool = False) -> dict:
        """Time the candidate schedules on the first wave; keep the fastest."""
        o = BatchOpts(max_wave, 1 if use_graph else 0, 1 if saif_only else 0)
        r = TuneResult()
        self._check(self.lib.gls_autotune(self.h, C.byref(o), C.byref(r)), "autotune")
        cands = [{"seg_per_sm": r.seg_per_sm[k], "warp_mask": r.warp_mask[k], "flags": r.flags[k], "ms": r.ms[k]}
                 for k in range(r.n)]
        return {"best": cands[r.best], "windows": r.windows, "candidates": cands}

    def set_schedule(self, seg_per_sm: int, warp_mask: int, flags: int = 0):
        self._check(self.lib.gls_set_schedule(self.h, seg_per_sm, warp_mask, flags), "set_schedule")

    def saif(self, window: int = 0) -> np.ndarray:
        """(n_nets, 3) uint64: T0, T1, TX; UINT64_MAX rows were not produced."""
        t3 = np.empty((self.n_nets, 3), np.uint64)
        self._check(self.lib.gls_saif_table(self.h, window, _ptr(t3)), "saif_table")
        return t3

    def saif_counts(self, window: int = 0):
        """T0, T1, TX as three arrays (the reference-shaped call)."""
        t0 = np.empty(self.n_nets, np.uint64)
        t1 = np.empty(self.n_nets, np.uint64)
        tx = np.empty(self.n_nets, np.uint64)
        self._check(self.lib.gls_saif_counts(self.h, window, _ptr(t0), _ptr(t1), _ptr(tx)), "saif_counts")
        return t0, t1, tx

    def lengths(self, window: int = 0) -> np.ndarray:
        ln = np.zeros(self.n_nets, np.uint32)
        self._check(self.lib.gls_waveform_lengths(self.h, window, _ptr(ln)), "waveform_lengths")
        return ln

    def waveform(self, net: int, window: int = 0):
        n = C.c_uint64()
        self._check(self.lib.gls_waveform(self.h, window, net, None, None, 0, C.byref(n)), "waveform")
        if n.value == 2**64 - 1:
            return None
        t = np.zeros(n.value, np.uint32)
        v = np.zeros(n.value, np.uint8)
        self._check(self.lib.gls_waveform(self.h, window, net, _ptr(t), _ptr(v), n.value, C.byref(n)), "waveform")
        return t, v

    def run_level_static(self, level: int, first: int, count: int, d_pool: int, pool_cap: int, d_top: int,
                         d_net_off: int, d_net_len: int, d_saif: int, t_begin: int, t_end: int):
        """One level's gate outputs on caller-owned device buffers (device
        pointers as integers), with no device allocation by the library."""
        self._check(self.lib.gls_run_level_static(self.h, level, first, count, d_pool, pool_cap, d_top, d_net_off,
                                                  d_net_len, d_saif, t_begin, t_end), "run_level_static")

    def stats(self) -> dict:
        s = Stats()
        self._check(self.lib.gls_stats_get(self.h, C.byref(s)), "stats")
        return s.as_dict()

    # ---------------------------------------------------------- presize
    def set_presize_model(self, params: np.ndarray, margin: float = 0.25, slack: int = 8):
        """Install the MLP used by ALLOC_LEARNED (FP32 parameters, flat)."""
        self._model = presize_model(params, margin, slack)
        self._check(self.lib.gls_set_presize_model(self.h, C.byref(self._model)), "set_presize_model")

    def presize_samples(self, window: int = 0):
        """(features (n, 32) float32, output-list lengths (n,) uint32) of every gate output."""
        n = C.c_uint64()
        self._check(self.lib.gls_presize_samples(self.h, window, None, None, 0, C.byref(n)), "presize_samples")
        feat = np.zeros((n.value, MLP_IN), np.float32)
        cnt = np.zeros(n.value, np.uint32)
        self._check(self.lib.gls_presize_samples(self.h, window, _ptr(feat), _ptr(cnt), n.value, C.byref(n)),
                    "presize_samples")
        return feat, cnt

    def presize_predict(self, params: np.ndarray, feat: np.ndarray, tensor_cores: bool = True) -> np.ndarray:
        """Network output y for host feature rows (tensor-core or FP32 kernel)."""
        m = presize_model(params)
        f = np.ascontiguousarray(feat, np.float32)
        y = np.zeros(len(f), np.float32)
        self._check(self.lib.gls_presize_predict(self.h, C.byref(m), _ptr(f), len(f), _ptr(y),
                                                 1 if tensor_cores else 0), "presize_predict")
        return y


class Trainer:
    """GPU training of the presize MLP (FP32, Adam, Huber loss on log lengths)."""

    def __init__(self, device: int = 0, seed: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        rc = self.lib.gls_trainer_create(device, seed, C.byref(h))
        if rc:
            raise GlsError(rc, "gls_trainer_create failed (no CUDA device?)")
        self.h = h

    def _check(self, rc: int, what: str):
        if rc:
            raise GlsError(rc, f"{what}: {self.lib.gls_trainer_error(self.h).decode()}")

    def close(self):
        if self.h:
            self.lib.gls_trainer_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_data(self, feat: np.ndarray, target: np.ndarray):
        self._feat = np.ascontiguousarray(feat, np.float32)
        self._target = np.ascontiguousarray(target, np.float32)
        self._check(self.lib.gls_trainer_set_data(self.h, _ptr(self._feat), _ptr(self._target), len(self._target)),
                    "set_data")

    def fit(self, epochs: int, batch: int = 8192, lr: float = 1e-3, huber: float = 1.0, seed: int = 0) -> np.ndarray:
        loss = np.zeros(epochs, np.float32)
        o = TrainOpts(batch, epochs, lr, huber, seed)
        self._check(self.lib.gls_trainer_fit(self.h, C.byref(o), _ptr(loss)), "fit")
        return loss

    def grad(self, first: int, n: int, huber: float = 1.0):
        g = np.zeros(MLP_PARAMS, np.float32)
        loss = np.zeros(1, np.float32)
        self._check(self.lib.gls_trainer_grad(self.h, first, n, huber, _ptr(g), _ptr(loss)), "grad")
        return g, float(loss[0])

    def params(self) -> np.ndarray:
        p = np.zeros(MLP_PARAMS, np.float32)
        self._check(self.lib.gls_trainer_get_params(self.h, _ptr(p)), "get_params")
        return p

    def set_params(self, p: np.ndarray):
        self._p = np.ascontiguousarray(p, np.float32)
        self._check(self.lib.gls_trainer_set_params(self.h, _ptr(self._p)), "set_params")
