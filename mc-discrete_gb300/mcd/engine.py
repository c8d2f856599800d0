"""Host engine: builds mcd_sim structs from input.file parameters, owns the
device buffers (torch tensors) and calls the C ABI on the current stream.

    run(input_par, num_el, seed)          one simulation, one launch
    Batch(sims).run(tune)                 many simulations, one persistent launch

Everything is device-resident; results are copied back only when asked.
"""
import ctypes as C

import numpy as np

from . import _lib
from .config import with_defaults
from .tables import ds_tables, sigma_table, sigma_table_fits

DEFAULT_HIST_E = (200, 100.0)   # 200 bins of 100 eV
DEFAULT_HIST_T = (90, 1.0)      # 90 bins of 1 degree

_DTYPE = {_lib.FP32: np.float32, _lib.FP64: np.float64}


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("mcd needs a CUDA device (there is no CPU path)")
    return torch


def mode_of(input_par):
    return _lib.MODE_DS if "DS" in input_par.get("mode", "DS") else _lib.MODE_CONT


def elastic_model(elastic, mode, dispatch="reference"):
    """The MCD_ELASTIC_* code of an input.file 'elastic' value.

    dispatch="reference" follows the reference's string tests:
      DS (MC/tools/scattering.py:483-493): 'Ruth_vanilla' exactly; any name
        containing 'vanilla_wDefl' calls ruther_sigma_wDefl, which that module
        never imports (:14), so it raises NameError; 'Ruth_nigram' exactly;
        any name containing 'nigram_wDefl'.
      continuous (:781-790): any name containing 'vanilla', then any name
        containing 'nigram' -- so both wDefl variants fall back to their
        base models.
    dispatch="intended" maps the four names one to one.  Names containing
    'Ruth' that match no rule (the reference then runs without an elastic
    channel) raise ValueError; other names select Mott scattering, whose
    tabulated cross sections (ioffe data) are not part of the reference."""
    if "Ruth" not in elastic:
        raise NotImplementedError("elastic %r: Mott tables (ioffe data) are not available" % elastic)
    if dispatch == "intended":
        if elastic not in _lib.ELASTIC:
            raise ValueError("unknown elastic model %r" % elastic)
        return _lib.ELASTIC[elastic]
    if mode == _lib.MODE_DS:
        if elastic == "Ruth_vanilla":
            return _lib.ELASTIC_RUTH
        if "vanilla_wDefl" in elastic:
            raise NameError("name 'ruther_sigma_wDefl' is not defined")
        if elastic == "Ruth_nigram":
            return _lib.ELASTIC_NIGRAM
        if "nigram_wDefl" in elastic:
            return _lib.ELASTIC_NIGRAM_WDEFL
    else:
        if "vanilla" in elastic:
            return _lib.ELASTIC_RUTH
        if "nigram" in elastic:
            return _lib.ELASTIC_NIGRAM
    raise ValueError("elastic %r selects no elastic cross section" % elastic)


def make_sim(input_par, num_el, seed=0, first_electron=0, precision=_lib.FP32, sim_id=0,
             hist_E=DEFAULT_HIST_E, hist_T=DEFAULT_HIST_T, quirks=_lib.QUIRKS_REFERENCE,
             tally_flags=0, J_scale=1.0, n_scale=1.0, elastic_dispatch="reference"):
    p = with_defaults(input_par)
    s = _lib.Sim()
    s.mode = mode_of(p)
    s.bethe_model = _lib.BETHE[p.get("Bethe_model", "classical")]
    s.precision = precision
    s.quirks = quirks
    s.tally_flags = tally_flags
    s.sim_id = sim_id
    s.E0 = float(p["E0"])
    s.Emin = float(p["Emin"])
    s.s_tilt = float(p["s_tilt"])
    s.Wc = float(p["Wc"])
    s.thickness = float(p["thickness"])
    s.max_scatt = int(p["maxScatt"])
    s.num_el = int(num_el)
    s.first_electron = int(first_electron)
    s.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    s.hist_E_bins, s.hist_E_width = int(hist_E[0]), float(hist_E[1])
    s.hist_T_bins, s.hist_T_width = int(hist_T[0]), float(hist_T[1])
    s.J_scale = float(J_scale)
    s.n_scale = float(n_scale)
    s.elastic = elastic_model(p.get("elastic", "Ruth_vanilla"), s.mode, elastic_dispatch)
    s.diff_mfp = 0
    if p.get("diffMFP") and s.mode == _lib.MODE_DS:
        # the channel reads the material's extinction distance
        # (MC/tools/material.py:225-226 defines it for Si only)
        if not _lib.material(p["material"]).xip_g > 0:
            raise KeyError("xip_g")
        s.diff_mfp = 1
    return s


def use_sigma_table(sim, mat, device="cuda"):
    """Point a DS simulation at its cross-section table for its precision
    (FP32: linear in log E; FP64: cubic on octave grids), built once per
    parameter set and kept alive by the cache; returns the table, or None
    when the simulation evaluates its cross sections inline (continuous
    mode, or an FP64 energy range too wide for the table)."""
    if sim.mode != _lib.MODE_DS:
        return None
    if sim.precision == _lib.FP64 and not sigma_table_fits(sim, mat):
        return None
    t = sigma_table(sim, mat, device)
    sim.sigma_table = t.data_ptr()
    return t


def tally_to_dict(t):
    out = {k: int(t.outcome[i]) for i, k in enumerate(_lib.OUTCOME_NAMES)}
    for k in ("events", "double_rows", "nan_events", "clamped", "long_path", "table_range"):
        out[k] = int(getattr(t, k))
    out["channel"] = np.array(t.channel[:], dtype=np.int64)
    out["sum_E_bks"] = float(t.sum_E_bks)
    out["sum_E2_bks"] = float(t.sum_E2_bks)
    out["sum_steps2"] = float(t.sum_steps2)
    out["hist_E"] = np.array(t.hist_E[:], dtype=np.int64)
    out["hist_T"] = np.array(t.hist_T[:], dtype=np.int64)
    return out


def tally_from_bytes(buf):
    t = _lib.Tally.from_buffer_copy(bytes(buf))
    return tally_to_dict(t)


def _device_rows(n, fdt, device):
    """Per-electron row arrays on the device (the mcd_electron_out layout)."""
    torch = _torch()
    return dict(
        outcome=torch.zeros(n, dtype=torch.uint8, device=device),
        flags=torch.zeros(n, dtype=torch.uint8, device=device),
        final_E=torch.zeros(n, dtype=fdt, device=device),
        dir=torch.zeros(3 * n, dtype=fdt, device=device),
        last_pos=torch.zeros(3 * n, dtype=fdt, device=device),
        max_z=torch.zeros(n, dtype=fdt, device=device),
        n_events=torch.zeros(n, dtype=torch.int32, device=device),
    )


def _rows_struct(e):
    return _lib.ElectronOut(e["outcome"].data_ptr(), e["flags"].data_ptr(), e["final_E"].data_ptr(),
                            e["dir"].data_ptr(), e["last_pos"].data_ptr(), e["max_z"].data_ptr(),
                            e["n_events"].data_ptr())


def _host_rows(el, n):
    """Per-electron rows copied to the host (dir and last_pos as (n, 3))."""
    e = {k: v.cpu().numpy() for k, v in el.items()}
    return dict(outcome=e["outcome"], flags=e["flags"], final_E=e["final_E"],
                dir=e["dir"].reshape(3, n).T.copy(), last_pos=e["last_pos"].reshape(3, n).T.copy(),
                max_z=e["max_z"], n_events=e["n_events"])


class RunBuffers:
    """Device buffers of one simulation (re-usable across launches)."""

    def __init__(self, num_el, precision=_lib.FP32, electrons=True, ring_capacity=0, device="cuda", ring_fields=0):
        torch = _torch()
        self.device = torch.device(device)
        self.num_el = int(num_el)
        self.precision = precision
        tsz = C.sizeof(_lib.Tally)
        self.tally = torch.zeros(tsz, dtype=torch.uint8, device=self.device)
        self.status = torch.zeros(1, dtype=torch.int32, device=self.device)
        fdt = torch.float32 if precision == _lib.FP32 else torch.float64
        self.el = _device_rows(self.num_el, fdt, self.device) if electrons else None
        self.ring = None
        self.ring_fields = int(ring_fields)
        if ring_capacity:
            self.ring = torch.zeros((int(ring_capacity), event_bytes(self.ring_fields)), dtype=torch.uint8,
                                    device=self.device)
            self.cursor = torch.zeros(1, dtype=torch.int64, device=self.device)

    def zero(self):
        self.tally.zero_()
        self.status.zero_()
        if self.ring is not None:
            self.cursor.zero_()

    def electron_struct(self):
        return _rows_struct(self.el) if self.el is not None else None

    def ring_struct(self):
        if self.ring is None:
            return None
        return _lib.EventRing(self.ring.data_ptr(), self.ring.shape[0], self.cursor.data_ptr(), self.ring_fields, 0)


class RunResult:
    def __init__(self, tally, status, electrons=None, events=None, events_total=0):
        self.tally = tally
        self.status = status
        self.electrons = electrons
        self.events = events
        self.events_total = events_total

    @property
    def eta(self):
        n = sum(self.tally[k] for k in _lib.OUTCOME_NAMES)
        return self.tally["bks"] / n if n else float("nan")


EVENT_DTYPE = np.dtype([("electron", "<u4"), ("step_chan", "<u4"), ("E", "<f4"), ("W", "<f4"),
                        ("pathl", "<f4"), ("c2", "<f4"), ("half_phi", "<f4"), ("x", "<f4"),
                        ("y", "<f4"), ("z", "<f4")])
_EV_NAMES = ((_lib.EV_E, ("E",)), (_lib.EV_W, ("W",)), (_lib.EV_PATHL, ("pathl",)), (_lib.EV_C2, ("c2",)),
             (_lib.EV_PHI, ("half_phi",)), (_lib.EV_POS, ("x", "y", "z")))


def event_dtype(fields=0):
    """Record dtype of a ring written with an MCD_EV_* field mask (columns,
    0 = all; with EV_PACKED_HEAD the header is one word 'head')."""
    f = int(fields) & _lib.EV_ALL
    packed = bool(int(fields) & _lib.EV_PACKED_HEAD)
    if f in (0, _lib.EV_ALL) and not packed:
        return EVENT_DTYPE
    f = f or _lib.EV_ALL
    names = [("head", "<u4")] if packed else [("electron", "<u4"), ("step_chan", "<u4")]
    for bit, cols in _EV_NAMES:
        if f & bit:
            names += [(c, "<f4") for c in cols]
    return np.dtype(names)


def event_bytes(fields=0):
    return event_dtype(fields).itemsize


def unpack_events(rec, fields):
    """Records of a packed-header ring (in ring order) as records with the
    'electron' and 'step_chan' header, sorted by electron and event.  An
    electron's records keep their order in the ring, so its n-th record is
    its event n; a ring that overflowed has lost records and cannot be
    unpacked."""
    fields = int(fields)
    if not fields & _lib.EV_PACKED_HEAD:
        return rec
    out_dt = event_dtype(fields & ~_lib.EV_PACKED_HEAD)
    head = rec["head"]
    e = head >> 4
    order = np.argsort(e, kind="stable")
    es = e[order]
    n = es.size
    first = np.ones(n, dtype=bool)
    first[1:] = es[1:] != es[:-1]
    starts = np.flatnonzero(first)
    step = np.arange(n, dtype=np.int64) - np.repeat(starts, np.diff(np.append(starts, n)))
    out = np.empty(n, dtype=out_dt)
    out["electron"] = es
    out["step_chan"] = (step.astype(np.uint32) << 5) | (head[order] & 15)
    for name in out_dt.names[2:]:
        out[name] = rec[name][order]
    return out


def launch(sim, mat, tables, bufs, block_size=0, stream=None):
    """Enqueue one mcd_run on `stream` (torch's current stream by default)."""
    torch = _torch()
    st = stream if stream is not None else torch.cuda.current_stream(bufs.device)
    tm = tables[0].struct if tables else None
    tg = tables[1].struct if tables else None
    el = bufs.electron_struct()
    rg = bufs.ring_struct()
    code = _lib.lib().mcd_run(C.byref(sim), C.byref(mat), C.byref(tm) if tm else None,
                              C.byref(tg) if tg else None, bufs.tally.data_ptr(),
                              C.byref(el) if el else None, C.byref(rg) if rg else None,
                              bufs.status.data_ptr(), int(block_size), st.cuda_stream)
    _lib.check("mcd_run", code)


def collect(bufs):
    """Copy the results of the last launch back to the host (synchronises)."""
    tally = tally_from_bytes(bufs.tally.cpu().numpy())
    status = int(bufs.status.item())
    electrons = _host_rows(bufs.el, bufs.num_el) if bufs.el is not None else None
    events, total = None, 0
    if bufs.ring is not None:
        total = int(bufs.cursor.item())
        k = min(total, bufs.ring.shape[0])
        events = bufs.ring[:k].cpu().numpy().view(event_dtype(bufs.ring_fields)).reshape(-1)
        if total > bufs.ring.shape[0]:
            status |= _lib.FLAG_RING_FULL
        else:
            events = unpack_events(events, bufs.ring_fields)
    return RunResult(tally, status, electrons, events, total)


def run(input_par, num_el=None, seed=0, first_electron=0, precision="fp32", electrons=True, ring_capacity=0,
        tally_channels=False, hist_E=DEFAULT_HIST_E, hist_T=DEFAULT_HIST_T, quirks=_lib.QUIRKS_REFERENCE,
        J_scale=1.0, n_scale=1.0, block_size=0, device="cuda", tables=None, ring_fields=0, tabulated=False):
    """Run one simulation to completion and return its results on the host.
    tabulated: DS transport reads the channel cross sections from a table
    for its precision (use_sigma_table) instead of evaluating them."""
    _torch()
    p = with_defaults(input_par)
    n = int(p["num_el"] if num_el is None else num_el)
    prec = _lib.FP64 if precision in ("fp64", _lib.FP64) else _lib.FP32
    mat = _lib.material(p["material"])
    sim = make_sim(p, n, seed, first_electron, prec, 0, hist_E, hist_T, quirks,
                   _lib.TALLY_CHANNELS if tally_channels else 0, J_scale, n_scale)
    if sim.mode == _lib.MODE_DS and tables is None:
        tables = ds_tables(mat, p["E0"], p["Emin"], p["Wc"], p["tol_E"], p["tol_W"], device)
    if tabulated:
        use_sigma_table(sim, mat, device)
    bufs = RunBuffers(n, prec, electrons, ring_capacity, device, ring_fields)
    bufs.zero()
    launch(sim, mat, tables if sim.mode == _lib.MODE_DS else None, bufs, block_size)
    return collect(bufs)


# ---------------------------------------------------------------------------
# batched persistent launch
# ---------------------------------------------------------------------------
class Batch:
    """Many simulations run by one persistent kernel.

    sims: list of input_par dicts (each with num_el).  Tables are built once
    per distinct (material, E0, Emin, Wc, tol) and shared.  electrons=True
    keeps every simulation's per-electron rows (electrons(k)).
    """

    def __init__(self, sims, seed=0, device="cuda", hist_E=DEFAULT_HIST_E, hist_T=DEFAULT_HIST_T,
                 quirks=_lib.QUIRKS_REFERENCE, tally_channels=False, first_electron=0, electrons=False):
        torch = _torch()
        self.device = torch.device(device)
        self.inputs = [with_defaults(s) for s in sims]
        self.n = len(self.inputs)
        mats, mat_index = [], {}
        tabs, tab_index = [], {}
        sim_mat, sim_m, sim_g = [], [], []
        self.structs = []
        for k, p in enumerate(self.inputs):
            sp = p["material"]
            if sp not in mat_index:
                mat_index[sp] = len(mats)
                mats.append(_lib.material(sp))
            mi = mat_index[sp]
            sim_mat.append(mi)
            if mode_of(p) == _lib.MODE_DS:
                key = (sp, p["E0"], p["Emin"], p["Wc"], p["tol_E"], p["tol_W"])
                if key not in tab_index:
                    tm, tg = ds_tables(mats[mi], *key[1:], device=device)
                    tab_index[key] = len(tabs)
                    tabs += [tm, tg]
                sim_m.append(tab_index[key])
                sim_g.append(tab_index[key] + 1)
            else:
                sim_m.append(0)
                sim_g.append(0)
            self.structs.append(make_sim(p, p["num_el"], seed, first_electron, _lib.FP32, k, hist_E, hist_T, quirks,
                                         _lib.TALLY_CHANNELS if tally_channels else 0))
        self.tables = tabs
        self.el, self._el_structs = None, []
        if electrons:
            self.el = [_device_rows(int(p["num_el"]), torch.float32, self.device) for p in self.inputs]
            self._el_structs = [_rows_struct(e) for e in self.el]   # read when the batch is packed
            for s_, eo in zip(self.structs, self._el_structs):
                s_.electrons = C.addressof(eo)
        self.mats = (_lib.Material * len(mats))(*mats)
        self._sims_arr = (_lib.Sim * self.n)(*self.structs)
        self._tarr = (_lib.Table * max(1, len(tabs)))(*[t.struct for t in tabs]) if tabs else None
        ia = lambda v: (C.c_int32 * self.n)(*v)  # noqa: E731
        self._idx = (ia(sim_mat), ia(sim_m), ia(sim_g))
        nbytes = _lib.lib().mcd_batch_workspace_bytes(self.n)
        if nbytes == 0:
            raise _lib.MCDError("mcd_batch_workspace_bytes", _lib.ETOOBIG)
        self.workspace = torch.empty(nbytes + 256, dtype=torch.uint8, device=self.device)
        off = (-self.workspace.data_ptr()) % 256
        self.ws_ptr = self.workspace.data_ptr() + off
        self.ws_bytes = nbytes
        self.prepare()
        self.tallies = torch.zeros((self.n, C.sizeof(_lib.Tally)), dtype=torch.uint8, device=self.device)
        self.status = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.total_electrons = sum(int(p["num_el"]) for p in self.inputs)

    def prepare(self, stream=None):
        """Pack the simulations into the device workspace (host-to-device copy)."""
        torch = _torch()
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        code = _lib.lib().mcd_batch_prepare(self._sims_arr, self.n, self.mats, self._idx[0], self._tarr,
                                            self._idx[1], self._idx[2], self.ws_ptr, self.ws_bytes,
                                            st.cuda_stream)
        _lib.check("mcd_batch_prepare", code)

    def launch(self, tune=None, stream=None):
        torch = _torch()
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        t = tune if tune is not None else _lib.Tune(256, 0, 1, 0, 0)
        code = _lib.lib().mcd_run_batched(self.ws_ptr, self.n, self.tallies.data_ptr(), C.byref(t),
                                          self.status.data_ptr(), st.cuda_stream)
        _lib.check("mcd_run_batched", code)

    def zero(self):
        self.tallies.zero_()
        self.status.zero_()

    def run_events(self, capacity, fields=0, tune=None, stream=None):
        """One run with every event appended to a device ring of `capacity`
        records (mcd_run_batched_ring; `fields` as for RunBuffers).  Returns
        (tallies, status, events, events_total): the events on the host in
        the 8-byte-header form, or None when they outgrew the ring
        (status has FLAG_RING_FULL; a re-run with a larger ring is exact)."""
        torch = _torch()
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        rb = event_bytes(fields)
        ring = torch.empty(int(capacity) * rb, dtype=torch.uint8, device=self.device)
        cursor = torch.zeros(1, dtype=torch.int64, device=self.device)
        t = tune if tune is not None else _lib.Tune(256, 0, 1, 0, 0)
        rs = _lib.EventRing(ring.data_ptr(), int(capacity), cursor.data_ptr(), int(fields), 0)
        self.zero()
        code = _lib.lib().mcd_run_batched_ring(self.ws_ptr, self.n, self.tallies.data_ptr(), C.byref(t), C.byref(rs),
                                               self.status.data_ptr(), st.cuda_stream)
        _lib.check("mcd_run_batched_ring", code)
        tallies, status = self.collect()
        total = int(cursor.item())
        if total > capacity:
            return tallies, status | _lib.FLAG_RING_FULL, None, total
        rec = ring[:total * rb].cpu().numpy().view(event_dtype(fields)).reshape(-1)
        return tallies, status, unpack_events(rec, fields), total

    def run(self, tune=None):
        self.zero()
        self.launch(tune)
        return self.collect()

    def collect(self):
        host = self.tallies.cpu().numpy()
        return [tally_from_bytes(host[k]) for k in range(self.n)], int(self.status.item())

    def electrons(self, k):
        """Simulation k's per-electron rows on the host (electrons=True)."""
        if self.el is None:
            raise RuntimeError("the batch keeps no per-electron rows (electrons=False)")
        return _host_rows(self.el[k], int(self.inputs[k]["num_el"]))
