"""Benchmark: batched persistent kernel vs one plain launch per simulation.

Workload (one step): 64 DS simulations {Al, Si, Cu, Au} x E0 {5, 10, 20, 30}
keV x tilt {0, 20, 45, 70} deg, Emin 1 keV, Wc 100 eV, tol_E = tol_W = 1e-3,
num_el = round(10^U[3,6]) drawn from numpy.random.default_rng(0) in that
nested order (8,927,966 electrons).  A step transports every electron to
its end: the persistent kernel runs the whole batch in one launch; the plain
path makes 64 launches of one thread per electron.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl mcd|reference]

Prints one JSON line (rank 0).  Under torchrun each rank runs the whole
workload on its own electron indices (weak scaling, no data-path
collective): the ranks meet at the timing barrier, and after the timed
region one sum of the tallies gives the whole job's event counts.
--impl reference times the CPU restatement of the reference (the C oracle)
on all host cores over a bounded, num_el-weighted sample of the same
workload, on the reference's own W/E grids, without loading the library.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "mc-discrete_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

MATERIALS = ("Al", "Si", "Cu", "Au")
ENERGIES = (5000.0, 10000.0, 20000.0, 30000.0)
TILTS = (0.0, 20.0, 45.0, 70.0)
N_SHELLS = {"Al": 3, "Si": 3, "Cu": 4, "Au": 8}
# Algorithmic work per DS event (inline cross sections for 3 + n_shells
# channels, channel pick, step, move, angle, quaternion update): FP32 FLOP
# (FMA = 2) and special-function (MUFU) operations.
FLOP_PER_EVENT = {k: 176 + 18 * n for k, n in N_SHELLS.items()}   # Si 230, Au 320
MUFU_PER_EVENT = {k: 17 + 4 * n for k, n in N_SHELLS.items()}     # Si 29, Au 49
# electrons of the bounded CPU sample, spread over the 64 simulations in
# proportion to num_el, so that its mix of trajectory lengths is the workload's
CPU_SAMPLE_ELECTRONS = 40000
# DRAM bytes (read + write) of one batched launch of the 64-simulation step,
# from an ncu capture of that launch (tables and workspace read about once;
# the figure does not grow with the electrons)
BATCHED_DRAM_BYTES = 55.48e6 + 0.47e6
# warp instructions issued per event by the batched kernel on this workload
# in its tuned shape (two blocks of 576 per SM, 56 registers), from an ncu
# capture of a quarter-size launch (2.0065e10 instructions for 1.3855e9
# events); the issue peak is one warp instruction per scheduler per cycle,
# 4 schedulers per SM
WARP_INST_PER_EVENT = 14.48
# the same capture's unit fractions (of peak sustained): issue-active cycles,
# threads per warp instruction / 32, the L1/TEX unit, its shared-memory
# wavefronts, and L2
BATCHED_NCU = {"issue_active": 0.770, "warp_execution_efficiency": 0.714, "l1tex_throughput": 0.747,
               "shared_wavefronts": 0.301, "l2_throughput": 0.029,
               "capture": "ncu --set full of k_batched_lr (2 x 576, 56 registers) on a quarter of the workload "
                          "(1.3855e9 events)"}


def workload(scale=1.0):
    rng = np.random.default_rng(0)
    sims = []
    for m in MATERIALS:
        for E0 in ENERGIES:
            for t in TILTS:
                n = int(round(10 ** rng.uniform(3, 6)))
                if scale != 1.0:
                    n = max(32, int(round(n * scale)))
                sims.append(dict(material=m, E0=E0, Emin=1000.0, s_tilt=t, Wc=100.0, tol_E=1e-3, tol_W=1e-3,
                                 mode="DS", num_el=n))
    return sims


WORKLOAD_NAME = ("64 DS sims {Al,Si,Cu,Au} x E0 {5,10,20,30} keV x tilt {0,20,45,70} deg, Emin 1 keV, "
                 "Wc 100 eV, tol 1e-3, num_el round(10^U[3,6]) rng(0)")


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples of the SM clock and throttle reasons."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        """Start sampling every 100 ms; returns once the first sample is in
        (at most 3 s), so that the samples kept cover the timed region from
        its start."""
        self.n0 = 0
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
            return
        t0 = time.perf_counter()
        while not self.lines and self.proc.poll() is None and time.perf_counter() - t0 < 3.0:
            time.sleep(0.005)
        self.n0 = len(self.lines)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        # the samples taken inside the timed region (the one before it when
        # the region was shorter than a sampling interval)
        for ln in self.lines[self.n0:] or self.lines[-1:]:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


# ---------------------------------------------------------------------------
def sample_sizes(sims, electrons=CPU_SAMPLE_ELECTRONS):
    """Electrons of each simulation in a bounded CPU sample weighted like the
    workload: num_el x (electrons / total electrons), at least one."""
    total = sum(s["num_el"] for s in sims)
    return [max(1, int(round(s["num_el"] * electrons / total))) for s in sims]


_GOLDEN_TABLES = {}


def oracle_tables(s):
    """The oracle's CDF tables of a workload simulation, on the W and E grids
    the reference's own grid search chose for it (tests/golden/tables.npz,
    written by tests/golden/gen_golden.py from the reference).  The CPU legs
    load nothing of the library under test."""
    import coracle
    import mcd_oracle as O
    mat = O.Material(s["material"])
    if "T" not in _GOLDEN_TABLES:
        _GOLDEN_TABLES["T"] = np.load(os.path.join(ROOT, "tests", "golden", "tables.npz"))
    T = _GOLDEN_TABLES["T"]
    key = "cfg4_%s_%d" % (s["material"], int(s["E0"] / 1000))
    spec = T[key + "/Moller/spec"]
    assert (spec[1], spec[2], spec[3]) == (s["Emin"], s["Wc"], s["tol_E"]), key
    return mat, [coracle.HostTable.build(kind, mat, T["%s/%s/Ws" % (key, kind)], T["%s/%s/Es" % (key, kind)])
                 for kind in ("Moller", "Gryz")]


def cpu_sample(sims, sizes, steps=1, seed=0):
    """The C oracle over the first sizes[k] electrons of simulation k (the
    GPU's Philox electron indices and sim ids), on every host thread."""
    import coracle
    threads = os.cpu_count() or 1
    prepared = []
    for s, n in zip(sims, sizes):
        mat, ht = oracle_tables(s)
        prepared.append((mat, ht, min(n, s["num_el"])))
    times, events, electrons, bks, ns = [], 0, 0, [], []
    for _ in range(steps):
        t0 = time.perf_counter()
        ev = el = 0
        bks, ns = [], []
        for k, (s, (mat, ht, n)) in enumerate(zip(sims, prepared)):
            r = coracle.run(mat, s["E0"], s["Emin"], s["s_tilt"], n, seed=seed, mode="DS", Wc=s["Wc"],
                            tables=ht, sim_id=k, nthreads=threads)
            ev += int(r["n_events"].sum())
            el += n
            bks.append(int((r["outcome"] == 1).sum()))
            ns.append(n)
        times.append(time.perf_counter() - t0)
        events, electrons = ev, el
    return {"times": times, "events": events, "electrons": electrons, "threads": threads, "bks": bks, "n": ns}


CFG1_WORKLOAD = ("DS Si, E0 10 keV, Emin 1 keV, tilt 0 deg, Wc 100 eV, tol 1e-3, 1000 electrons, FP64 "
                 "transport with per-electron rows")


def cfg1_bench(args, dev):
    """The small plain configuration in full on both sides: one FP64 launch
    (automatic block size) against the C oracle on 1 core and on all host
    cores (same Philox stream, so the two follow the same trajectories).
    The GPU reads the simulation's FP64 cross-section table (cubic on octave
    grids); the launch that evaluates every cross section per event is timed
    beside it, and the FP32 launch with its FP32 table."""
    import torch
    import coracle
    import mcd_oracle as O
    from mcd import _lib, engine, tables
    p = dict(material="Si", E0=10000.0, Emin=1000.0, s_tilt=0.0, Wc=100.0, tol_E=1e-3, tol_W=1e-3, mode="DS")
    n = 1000
    mat = _lib.material("Si")
    dt = tables.ds_tables(mat, 10000.0, 1000.0, 100.0, 1e-3, 1e-3, dev)
    stream = torch.cuda.current_stream(dev)

    def timed(sim, prec):
        bufs = engine.RunBuffers(n, prec, True, 0, device=dev)
        ms = []
        for k in range(args.warmup + max(3, args.steps)):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            bufs.zero()
            e0.record(stream)
            engine.launch(sim, mat, dt, bufs)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            if k >= args.warmup:
                ms.append(e0.elapsed_time(e1))
        return statistics.median(ms), engine.collect(bufs)

    sim = engine.make_sim(p, n, seed=args.seed, precision=_lib.FP64)
    engine.use_sigma_table(sim, mat, dev)
    ms, g = timed(sim, _lib.FP64)
    ms_inline, gi = timed(engine.make_sim(p, n, seed=args.seed, precision=_lib.FP64), _lib.FP64)
    sim32 = engine.make_sim(p, n, seed=args.seed, precision=_lib.FP32)
    engine.use_sigma_table(sim32, mat, dev)
    ms32, _ = timed(sim32, _lib.FP32)
    om = O.Material("Si")
    ht = [coracle.HostTable(t.Ws.cpu().numpy(), t.Es.cpu().numpy(), t.cdf.cpu().numpy()) for t in dt]
    cpu = {}
    for th in (1, os.cpu_count() or 1):
        best = float("inf")
        for _ in range(3 if th > 1 else 1):
            t0 = time.perf_counter()
            c = coracle.run(om, 10000.0, 1000.0, 0.0, n, seed=args.seed, mode="DS", Wc=100.0, tables=ht, nthreads=th)
            best = min(best, time.perf_counter() - t0)
        cpu[th] = best
    ev = int(g.tally["events"])

    def same(r):
        return float(np.mean((r.electrons["outcome"] == c["outcome"]) & (r.electrons["n_events"] == c["n_events"])))

    return {"workload": CFG1_WORKLOAD, "num_el": n, "events": ev, "gpu_ms": ms, "gpu_events_per_s": ev / ms * 1e3,
            "cross_sections": "FP64 table, cubic on octave grids (exact in cells that straddle a threshold)",
            "gpu_inline_ms": ms_inline, "gpu_fp32_ms": ms32,
            "longest_electron_events": int(g.electrons["n_events"].max()),
            "note": "the launch lasts as long as its longest trajectory, a chain of dependent instructions "
                    "(FP64 ones the longest); the automatic size runs two electrons per warp (at most one "
                    "warp per scheduler), each on a half-warp whose lanes compute the next 16 events' "
                    "trajectory-independent values (Philox block, step logarithm, azimuth, uniforms)",
            "cpu_1core_s": cpu[1], "cpu_all_cores_s": cpu[os.cpu_count() or 1], "cpu_cores": os.cpu_count() or 1,
            "cpu_timing": "best of 3 on all cores, one run on 1 core",
            "eta_gpu_fp64": g.tally["bks"] / n, "eta_oracle": float(np.mean(c["outcome"] == 1)),
            "identical_trajectories": same(g), "identical_trajectories_inline": same(gi),
            "gpu_launches": 3 * (args.warmup + max(3, args.steps))}


def bench_config(sims):
    """The workload as both arms name it (identical dicts)."""
    return {"workload": WORKLOAD_NAME, "sims": len(sims),
            "electrons_per_replica": sum(s["num_el"] for s in sims),
            "l2": "GPU arm: flushed between timed steps (256 MB write)"}


def reference_python_record():
    """The reference's own Python DS worker (multiTraj_DS), timed where the
    reference is installed (tests/golden/time_reference.py writes the
    record); it cannot run on a host without the reference."""
    try:
        with open(os.path.join(ROOT, "tests", "golden", "reference_timing.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


def sample_note(r):
    return ("num_el-weighted sample: %d electrons over the 64 sims (num_el x %.3g, at least 1), %d events per "
            "step, first electrons of each sim on the GPU's Philox indices"
            % (r["electrons"], CPU_SAMPLE_ELECTRONS / max(1, r["total"]), r["events"]))


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    sims = workload()
    sizes = sample_sizes(sims)
    # warm-up steps run a smaller slice of the same sample
    if args.warmup:
        cpu_sample(sims[:8], sizes[:8], steps=args.warmup)
    r = cpu_sample(sims, sizes, steps=args.steps)
    r["total"] = sum(s["num_el"] for s in sims)
    t = sum(r["times"])
    v = r["events"] * len(r["times"]) / t
    sample = sample_note(r)
    line = {
        "impl": "reference", "metric": "scatter events/s", "value": v, "unit": "events/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / len(r["times"]),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": bench_config(sims),
        "cpu_baseline": {"value": v, "unit": "events/s", "cores": r["threads"], "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "electrons_per_s": r["electrons"] * len(r["times"]) / t,
        "reference_python": reference_python_record(),
        "note": "C restatement of the reference's DS trajectory loop (oracle/mcd_oracle.c), FP64, all host "
                "threads, on the reference's own W/E grids; the reference itself is Python and is not present "
                "on the GPU host (reference_python: its worker timed where it is installed)",
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
ADJ_WORKLOAD = ("continuous classical Bethe, Al, E0 15 keV, Emin 1 keV, tilt 70 deg, 1e6 electrons, FP32; "
                "L2 loss of 64 Gaussian-soft exit-energy bins (sigma 50 eV) against a target made with J x 1.1")


def adjoint_bench(args, dev):
    """Forward and adjoint times of the differentiable continuous-mode workload."""
    import torch
    from mcd.adjoint import ExitEnergyModel
    p = dict(material="Al", E0=15000.0, Emin=1000.0, s_tilt=70.0, mode="cont", Bethe_model="classical")
    n = max(1000, int(round(1e6 * args.scale)))
    m = ExitEnergyModel(p, n, seed=args.seed, precision="fp32", device=dev)
    t, _, _ = m.forward(1.1, 1.0)
    h, _, _ = m.forward(1.0, 1.0)
    g = 2.0 * (h - t)
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        m.launch_forward(1.0, 1.0)
        m.launch_backward(g, 0.0)
    torch.cuda.synchronize(dev)
    tf = tb = 0.0
    for _ in range(args.steps):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        m.launch_forward(1.0, 1.0)
        e1.record(stream)
        m.launch_backward(g, 0.0)
        e2.record(stream)
        torch.cuda.synchronize(dev)
        tf += e0.elapsed_time(e1)
        tb += e1.elapsed_time(e2)
    h, _, _ = m.forward(1.0, 1.0)
    L = float(np.sum((h - t) ** 2))
    dJ, dn = m.backward(2.0 * (h - t), 0.0)
    d = 1e-3
    Lp = float(np.sum((m.chain(1 + d, 1.0)[0] - t) ** 2))
    Lm = float(np.sum((m.chain(1 - d, 1.0)[0] - t) ** 2))
    fd = (Lp - Lm) / (2 * d)
    h, _, _ = m.forward(1.0, 1.0)     # restore the checkpoints of J = 1
    # the re-simulated central difference with common random numbers
    # (every electron free to change its event sequence), split into the
    # electrons whose exit event stayed and the jump part of the others
    from mcd.adjoint import resimulated_fd
    r = resimulated_fd(m, t, h=d)
    crn = {"dL_dJscale": r["fd"], "rel_err": abs(dJ - r["fd"]) / abs(r["fd"]),
           "z": (r["fd"] - dJ) / r["jump_se"], "same_sequence_dL_dJscale": r["fd_same_sequence"],
           "same_sequence_rel_err": abs(dJ - r["fd_same_sequence"]) / abs(dJ), "jump_part": r["fd_jump"],
           "jump_se_rel": r["jump_se"] / abs(dJ), "electrons_changed": r["changed"],
           "note": "the jump part is noise of standard error ~ 1/sqrt(N h) (16 seeds: mean 1.3% +- 2.9% of the "
                   "gradient), so agreement is measured by z = (FD - adjoint) / its standard error"}
    depth = adjoint_depth_bench(args, dev, p, n)
    return {"workload": ADJ_WORKLOAD, "num_el": n, "fwd_ms": tf / args.steps, "bwd_ms": tb / args.steps,
            "bwd_over_fwd": tb / tf, "loss": L, "dL_dJscale": dJ, "dL_dnscale": dn,
            "fd_frozen_dL_dJscale": fd, "fd_frozen_rel_err": abs(dJ - fd) / abs(fd) if fd else None,
            "fd_crn": crn, "fd_crn_rel_err": crn["rel_err"],
            "fd_step": d, "max_depth": depth, "gpu_launches": 2 * args.steps + depth["gpu_launches"] + 3}


def adjoint_depth_bench(args, dev, p, n):
    """The same workload with the deepest z of backscattered electrons binned
    (64 Gaussian-soft bins over 0-20000 A, sigma 300 A; target made with
    J x 1.1): the adjoint runs through every deflection."""
    import torch
    from mcd.adjoint import ExitEnergyModel
    m = ExitEnergyModel(p, n, seed=args.seed, precision="fp32", device=dev, quantity="max_depth", lo=0.0,
                        hi=20000.0, sigma=300.0)
    t, _, _ = m.forward(1.1, 1.0)
    h, _, _ = m.forward(1.0, 1.0)
    g = 2.0 * (h - t)
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        m.launch_forward(1.0, 1.0)
        m.launch_backward(g, 0.0)
    torch.cuda.synchronize(dev)
    tf = tb = 0.0
    for _ in range(args.steps):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        m.launch_forward(1.0, 1.0)
        e1.record(stream)
        m.launch_backward(g, 0.0)
        e2.record(stream)
        torch.cuda.synchronize(dev)
        tf += e0.elapsed_time(e1)
        tb += e1.elapsed_time(e2)
    h, _, _ = m.forward(1.0, 1.0)
    dJ, dn = m.backward(2.0 * (h - t), 0.0)
    d = 1e-3
    fdJ = (float(np.sum((m.chain(1 + d, 1.0)[0] - t) ** 2)) - float(np.sum((m.chain(1 - d, 1.0)[0] - t) ** 2))) / (2 * d)
    fdn = (float(np.sum((m.chain(1.0, 1 + d)[0] - t) ** 2)) - float(np.sum((m.chain(1.0, 1 - d)[0] - t) ** 2))) / (2 * d)
    # dL/dJ is about 40 times smaller than dL/dn here, and an FP32 chain
    # resolves a difference in J only to about 1e-2 of it (step 1e-3:
    # rounding; step 1e-2: the curvature of the chain); the FP64 model on
    # the first 1e5 electrons, adjoint against its own step-1e-5 difference
    n64 = min(n, 100000)
    m64 = ExitEnergyModel(p, n64, seed=args.seed, precision="fp64", device=dev, quantity="max_depth", lo=0.0,
                          hi=20000.0, sigma=300.0)
    t64, _, _ = m64.forward(1.1, 1.0)
    h64, _, _ = m64.forward(1.0, 1.0)
    dJ64, _ = m64.backward(2.0 * (h64 - t64), 0.0)
    d64 = 1e-5
    fdJ64 = (float(np.sum((m64.chain(1 + d64, 1.0)[0] - t64) ** 2)) -
             float(np.sum((m64.chain(1 - d64, 1.0)[0] - t64) ** 2))) / (2 * d64)
    return {"fwd_ms": tf / args.steps, "bwd_ms": tb / args.steps, "bwd_over_fwd": tb / tf,
            "dL_dJscale": dJ, "dL_dnscale": dn, "fd_frozen_rel_err_J": abs(dJ - fdJ) / abs(fdJ) if fdJ else None,
            "fd_frozen_rel_err_n": abs(dn - fdn) / abs(fdn) if fdn else None, "fd_step": d,
            "fp64_electrons": n64, "fp64_fd_frozen_rel_err_J": abs(dJ64 - fdJ64) / abs(fdJ64) if fdJ64 else None,
            "gpu_launches": 2 * args.steps + 6}


TABLES_WORKLOAD = ("the sampled-loss table pairs (Moller, outermost-shell Gryzinski) of the 16 (material, E0) "
                   "pairs of the 64-simulation workload (tol 1e-3), and of Au 30 keV, Emin 0.5 keV, Wc 50 eV, "
                   "tol 1e-4: host grid search (QUADPACK reference integral, float32 trapezoid scans) and GPU FP64 "
                   "fill with guide tables")


def tables_bench(args, dev):
    """Wall time of building the DS tables from scratch for a fresh parameter
    set: the grid search on the host and the fill on the GPU (grid copies,
    allocation and mcd_build_table, CUDA events), each table built twice and
    the second build timed.  Beside them, the reference's own table build
    (tests/golden/reference_timing.json: probTable grid search + computeBlock
    per table, where the reference is installed)."""
    import torch
    from mcd import _lib, tables
    stream = torch.cuda.current_stream(dev)

    def build(sp, E0, Emin, Wc, tol):
        m = _lib.material(sp)
        t0 = time.perf_counter()
        grids = [tables.find_grids(kind, m, E0, Emin, Wc, tol, tol) for kind in ("Moller", "Gryz")]
        host = time.perf_counter() - t0
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t1 = time.perf_counter()
        e0.record(stream)
        dts = [tables.DeviceTable(kind, m, W, E, dev) for kind, (W, E) in zip(("Moller", "Gryz"), grids)]
        e1.record(stream)
        torch.cuda.synchronize(dev)
        wall = time.perf_counter() - t1
        cells = sum(d.nE * (d.nW - 1) for d in dts)
        return host, e0.elapsed_time(e1) * 1e-3, wall, cells

    pairs = sorted({(s["material"], s["E0"]) for s in workload()})
    for sp, E0 in pairs[:2]:
        build(sp, E0, 1000.0, 100.0, 1e-3)          # warm-up: imports, allocator
    res = [build(sp, E0, 1000.0, 100.0, 1e-3) for sp, E0 in pairs]
    au = build("Au", 30000.0, 500.0, 50.0, 1e-4)
    au = build("Au", 30000.0, 500.0, 50.0, 1e-4)
    ref = reference_python_record()
    rt = ref["tables"] if ref else None
    out = {"workload": TABLES_WORKLOAD,
           "workload_16_pairs": {"host_search_ms": 1e3 * sum(r[0] for r in res),
                                 "gpu_fill_ms": 1e3 * sum(r[1] for r in res),
                                 "fill_wall_ms": 1e3 * sum(r[2] for r in res),
                                 "total_ms": 1e3 * sum(r[0] + r[2] for r in res),
                                 "cdf_cells": sum(r[3] for r in res),
                                 "reference_s": rt["workload_total_s"] if rt else None},
           "au30_tol1e-4": {"host_search_ms": 1e3 * au[0], "gpu_fill_ms": 1e3 * au[1], "fill_wall_ms": 1e3 * au[2],
                            "total_ms": 1e3 * (au[0] + au[2]), "cdf_cells": au[3],
                            "reference_s": rt["au30_tol1e-4_total_s"] if rt else None},
           "reference_note": ("the reference's probTable grid search + computeBlock + memmap per table, one core of "
                              "%s (%s)" % (ref["host"]["processor"], ref["date"])) if ref else None,
           "gpu_launches": 2 * (len(res) + 2 + 2)}
    return out


CONT_WORKLOAD = ("continuous JL Bethe, Cu, E0 20 keV, Emin 1 keV, tilt 70 deg, 1e6 electrons, FP32; "
                 "exit-energy histogram 200 x 100 eV and polar exit-angle histogram 90 x 1 deg")


def cont_bench(args, dev):
    """Events/s and electrons/s of the continuous-mode histogram workload:
    one persistent batched launch and one plain launch per step."""
    import torch
    from mcd import _lib, engine
    n = max(1000, int(round(1e6 * args.scale)))
    p = dict(material="Cu", E0=20000.0, Emin=1000.0, s_tilt=70.0, mode="cont", Bethe_model="JL", num_el=n)
    b = engine.Batch([p], seed=args.seed, device=dev)
    from mcd import autotune
    tune, _ = autotune.tune(b)
    sim = engine.make_sim(p, n, seed=args.seed)
    mat = _lib.material("Cu")
    bufs = engine.RunBuffers(n, _lib.FP32, False, 0, device=dev)
    stream = torch.cuda.current_stream(dev)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize(dev)
        tot = 0.0
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize(dev)
            tot += e0.elapsed_time(e1)
        return tot / args.steps

    def batched():
        b.zero()
        b.launch(tune)

    def plain():
        bufs.zero()
        engine.launch(sim, mat, None, bufs, block_size=args.plain_block)

    ms_b = timed(batched)
    t = b.collect()[0][0]
    ms_p = timed(plain)
    tp = engine.collect(bufs).tally
    ev = int(t["events"])
    hE = np.asarray(t["hist_E"][:200], dtype=np.float64)
    mids = (np.arange(200) + 0.5) * 100.0
    return {"workload": CONT_WORKLOAD, "num_el": n, "events": ev, "ms": ms_b, "events_per_s": ev / ms_b * 1e3,
            "electrons_per_s": n / ms_b * 1e3, "plain_ms": ms_p, "plain_events_per_s": int(tp["events"]) / ms_p * 1e3,
            "eta": t["bks"] / n, "mean_exit_E_eV": float((hE * mids).sum() / max(1.0, hE.sum())),
            "tune": {"block": tune.block_size, "refill": tune.refill, "variant": tune.variant},
            "cpu_baseline": None if args.no_cpu else oracle_eta_check(
                args, t["bks"] / n, n, _oracle_material("Cu"), 20000.0, 1000.0, 70.0, min(n, 20000),
                mode="cont", bethe="JL", max_scatt=10 ** 6),
            "gpu_launches": 2 * args.steps}


def _oracle_material(sp):
    import mcd_oracle as O
    return O.Material(sp)


def oracle_eta_check(args, eta_gpu, n_gpu, om, E0, Emin, tilt, n, **kw):
    """CPU baseline of a section: the FP64 C oracle on all host threads over
    the first n electrons of the same workload (same Philox electron indices),
    its events/s, and the section's backscatter yield against the oracle's
    (z of the difference; FP32 and FP64 trajectories diverge, so the
    comparison is statistical)."""
    import coracle
    t0 = time.perf_counter()
    c = coracle.run(om, E0, Emin, tilt, n, seed=args.seed, **kw)
    dt = time.perf_counter() - t0
    eta_o = float(np.mean(c["outcome"] == 1))
    var = eta_gpu * (1 - eta_gpu) / n_gpu + eta_o * (1 - eta_o) / n
    return {"kind": "port", "cores": os.cpu_count() or 1, "electrons": n,
            "events_per_s": float(c["n_events"].sum()) / dt, "eta_oracle": eta_o,
            "z": abs(eta_gpu - eta_o) / max(math.sqrt(var), 1e-12)}


DET_WORKLOAD = ("projection of 2^27 float32 exit directions (three planes, 1.61 GB) onto the EBSD detector "
                "(two planes, 1.07 GB out), reference geometry")


def detector_bench(args, dev):
    """HBM roofline of the detector projection map: 20 algorithmic bytes per
    direction (12 read, 8 written), inputs far larger than L2."""
    import torch
    from mcd import detector
    n = max(1 << 20, int(round((1 << 27) * args.scale)))
    g = torch.Generator(device=dev).manual_seed(args.seed)
    dirs = torch.randn((3, n), generator=g, device=dev, dtype=torch.float32)
    dirs /= dirs.norm(dim=0, keepdim=True)
    out = torch.empty((2, n), device=dev, dtype=torch.float32)
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        detector.project(dirs, out=out)
    torch.cuda.synchronize(dev)
    times = []
    for _ in range(max(3, args.steps)):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        detector.project(dirs, out=out)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        times.append(e0.elapsed_time(e1) * 1e-3)
    t = statistics.median(times)
    pk = measured_peaks()
    peak = float(pk.get("hbm_gbs", 6800.0))
    peak_note = ("measured copy bandwidth (MEASURED_PEAKS.json)" if "hbm_gbs" in pk else
                 "fallback 6.8 TB/s: no measured-peaks file on this host")
    gbs = 20.0 * n / t / 1e9
    cpu = None
    if not args.no_cpu:
        # CPU baseline: the FP64 restatement of projOnDetector (one core, numpy)
        # on the first 2^20 directions, and the FP32 kernel's error against it
        import mcd_oracle as O
        k = 1 << 20
        v = dirs[:, :k].double().T.cpu().numpy()
        t0 = time.perf_counter()
        ref = O.proj_on_detector(v, detector.ALPHA, detector.XY_PC, detector.L)
        dt = time.perf_counter() - t0
        err = np.abs(out[:, :k].double().T.cpu().numpy() - ref)
        cpu = {"kind": "port", "cores": 1, "directions": k, "directions_per_s": k / dt,
               "max_abs_err_um": float(err.max()), "max_rel_err": float((err / np.maximum(np.abs(ref), 1.0)).max())}
    return {"workload": DET_WORKLOAD, "n": n, "ms": t * 1e3, "directions_per_s": n / t,
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         "bytes_per_direction": 20, "peak_note": peak_note},
            "cpu_baseline": cpu, "gpu_launches": max(3, args.steps)}


STREAM_WORKLOAD = ("DS Au, E0 30 keV, Emin 0.5 keV, tilt 70 deg, Wc 50 eV, tol 1e-4, every event streamed "
                   "with its electron, channel, step length, W, polar angle and position (28-byte records, "
                   "one-word header) through two device rings to pinned host memory")


def stream_bench(args, dev):
    """Events/s of the streamed DS run, device rings drained to the host."""
    import torch
    from mcd.stream import EventStream
    n = max(10000, int(round(1e7 * args.scale * args.stream_fraction)))
    p = dict(material="Au", E0=30000.0, Emin=500.0, s_tilt=70.0, Wc=50.0, tol_E=1e-4, tol_W=1e-4, mode="DS",
             num_el=n)
    chunk = min(n, 1_000_000)
    from mcd import _lib
    fields = _lib.EV_PATHL | _lib.EV_W | _lib.EV_C2 | _lib.EV_POS | _lib.EV_PACKED_HEAD
    es = EventStream(p, chunk=chunk, seed=args.seed, events_per_electron=950.0, device=dev, fields=fields)
    seen = [0]

    def consumer(rec, c):            # the host side only counts what arrives
        seen[0] += rec.size

    es.run(consumer)                  # warm-up pass (tables, rings, pinned buffers)
    seen[0] = 0
    torch.cuda.synchronize(dev)
    st = es.run(consumer)
    eta = sum(t["bks"] for t in st["tallies"]) / n
    cpu = None
    if not args.no_cpu:
        import coracle
        from mcd import tables
        dt = tables.ds_tables(_lib.material("Au"), 30000.0, 500.0, 50.0, 1e-4, 1e-4, dev)
        ht = [coracle.HostTable(t.Ws.cpu().numpy(), t.Es.cpu().numpy(), t.cdf.cpu().numpy()) for t in dt]
        cpu = oracle_eta_check(args, eta, n, _oracle_material("Au"), 30000.0, 500.0, 70.0, min(n, 2000),
                               mode="DS", Wc=50.0, tables=ht, max_scatt=10 ** 6)
    # the device-to-host link the drain is bound by, on this machine: copies of
    # one piece into the stream's own pinned host piece, timed alone, the
    # best of three trials of four (one trial on a freshly pinned buffer
    # once read 69 GB/s on a box whose stream had just drained 153 GB/s)
    dst = es.host[0]
    piece = dst.numel()
    src = torch.empty(piece, dtype=torch.uint8, device=dev)
    side = torch.cuda.Stream(dev)
    rates = []
    with torch.cuda.stream(side):
        dst.copy_(src, non_blocking=True)
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(side)
            for _ in range(4):
                dst.copy_(src, non_blocking=True)
            e1.record(side)
            side.synchronize()
            rates.append(4 * piece / (e0.elapsed_time(e1) * 1e-3) / 1e9)
    link = max(rates)
    del src
    drain = st["bytes"] / st["wall_s"] / 1e9
    return {"workload": STREAM_WORKLOAD, "num_el": n, "chunk": chunk, "events": st["events"],
            "records_received": seen[0], "wall_s": st["wall_s"], "events_per_s": st["events"] / st["wall_s"],
            "drain_GB_per_s": drain, "d2h_link_GB_per_s": link, "drain_frac_of_link": drain / link,
            "record_bytes": es.rec_bytes,
            "ring_GB": es.cap * es.rec_bytes / 1e9, "eta": eta, "cpu_baseline": cpu,
            "reruns": st["reruns"], "gpu_launches": len(es.batches)}


def run_mcd(args):
    import torch
    from mcd import _lib, autotune, engine, shard

    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if ws > 1 else 0)
    torch.cuda.set_device(dev)
    sims = workload(args.scale)
    first = shard.replica_offset(rank)     # disjoint Philox electron indices per rank

    batch = engine.Batch(sims, seed=args.seed, device=dev, first_electron=first)
    if args.block or args.refill:
        tune = _lib.Tune(args.block or 256, args.blocks_per_sm, args.refill or 1, args.variant, 0)
        tune_table = None
    else:
        tune, tune_table = autotune.tune(batch)
    graph = autotune.BatchGraph(batch, tune)
    # plain path: one launch and buffer set per simulation, no per-electron
    # output; with a cross-section table per simulation (as the batched
    # kernel reads) and with the cross sections evaluated inline
    plain, plain_inline = [], []
    for k, s in enumerate(sims):
        mat = _lib.material(s["material"])
        tabs = batch.tables[2 * (k // len(TILTS)): 2 * (k // len(TILTS)) + 2]
        sim = engine.make_sim(s, s["num_el"], args.seed, first, _lib.FP32, k)
        engine.use_sigma_table(sim, mat, dev)
        plain.append((sim, mat, tabs, engine.RunBuffers(s["num_el"], _lib.FP32, False, 0, dev)))
        sim = engine.make_sim(s, s["num_el"], args.seed, first, _lib.FP32, k)
        plain_inline.append((sim, mat, tabs, engine.RunBuffers(s["num_el"], _lib.FP32, False, 0, dev)))

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def batched_step():                   # zero tallies, reset queue, launch: one graph
        graph.replay()

    def plain_step(arm=plain):
        for sim, mat, tabs, bufs in arm:
            bufs.zero()
            engine.launch(sim, mat, tabs, bufs, block_size=args.plain_block)

    def plain_inline_step():
        plain_step(plain_inline)

    def timed(step, k):
        total = 0.0
        for _ in range(k):
            flush.fill_(1.0)                       # evict L2 between timed steps
            torch.cuda.synchronize(dev)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step()
            b.record(stream)
            torch.cuda.synchronize(dev)
            total += a.elapsed_time(b) * 1e-3
        return total

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(dev)

    for _ in range(args.warmup):
        batched_step()
        if not args.no_plain:
            plain_step()
            plain_inline_step()
    torch.cuda.synchronize(dev)
    tallies, status = batch.collect()
    events = sum(t["events"] for t in tallies)
    electrons = batch.total_electrons

    clocks = ClockSampler(dev.index)
    barrier()
    clocks.start()
    t_batched = timed(batched_step, args.steps)
    barrier()
    clk = clocks.stop()
    k_plain = max(1, args.steps // 2)
    if args.no_plain:
        t_plain, t_plain_inline, ptallies, pitallies = float("nan"), float("nan"), tallies, tallies
    else:
        t_plain = timed(plain_step, k_plain)
        ptallies = [engine.collect(b[3]).tally for b in plain]
        t_plain_inline = timed(plain_inline_step, k_plain)
        pitallies = [engine.collect(b[3]).tally for b in plain_inline]
    barrier()

    # end to end through the public API: host-side inputs packed and copied
    # in, tallies copied out to pinned host memory, every step
    host_t = torch.empty(batch.tallies.shape, dtype=torch.uint8, pin_memory=True)
    t_e2e = 0.0
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        batch.prepare()
        batch.zero()
        batch.launch(tune)
        host_t.copy_(batch.tallies, non_blocking=True)
        torch.cuda.synchronize(dev)
        t_e2e += time.perf_counter() - t0
    e2e_tallies = [engine.tally_from_bytes(host_t[k].numpy()) for k in range(batch.n)]
    assert sum(t["events"] for t in e2e_tallies) == events

    def summed(tl):
        """Tallies summed over the ranks (each rank transported its own
        electrons): one collective of the integer counts, one of the FP64 sums."""
        return tl if dist is None else shard.allreduce_tallies(tl, dist, dev)

    tallies, ptallies, pitallies = summed(tallies), summed(ptallies), summed(pitallies)
    if dist is not None:
        tt = torch.tensor([t_batched, t_plain, t_plain_inline, t_e2e], dtype=torch.float64, device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_batched, t_plain, t_plain_inline, t_e2e = tt.tolist()
        dist.destroy_process_group()
    if rank != 0:
        return

    K = args.steps
    # every count below is the sum over all ranks; times are the slowest rank's
    events = sum(t["events"] for t in tallies)
    electrons = sum(sum(t[o] for o in ("bks", "abs", "trsm", "trdf", "long")) for t in tallies)
    value = events * K / t_batched
    plain_value = sum(t["events"] for t in ptallies) * k_plain / t_plain
    plain_inline_value = sum(t["events"] for t in pitallies) * k_plain / t_plain_inline
    # eta: batched vs plain (same counters) and vs the reference's samples
    zs = []
    for t, p in zip(tallies, ptallies):
        n = sum(t[o] for o in ("bks", "abs", "trsm", "long"))
        zs.append(abs(t["bks"] - p["bks"]) / max(1.0, math.sqrt(max(t["bks"], 1) * (1 - t["bks"] / n))))
    ref = {}
    try:
        S = np.load(os.path.join(ROOT, "tests", "golden", "ref_stats.npz"))
        for tag, key in (("si10", ("Si", 10000.0, 0.0)), ("cu20t45", ("Cu", 20000.0, 45.0)),
                         ("al5", ("Al", 5000.0, 0.0))):
            k = next(i for i, s in enumerate(sims) if (s["material"], s["E0"], s["s_tilt"]) == key)
            t = tallies[k]
            n = sum(t[o] for o in ("bks", "abs", "trsm", "long"))
            ro = S[tag + "/outcome"]
            k1, n1 = int((ro == 1).sum()), ro.size
            pp = (k1 + t["bks"]) / (n1 + n)
            z = abs(k1 / n1 - t["bks"] / n) / math.sqrt(pp * (1 - pp) * (1 / n1 + 1 / n))
            ref[tag] = {"eta": t["bks"] / n, "eta_reference": k1 / n1, "z": z}
    except (OSError, KeyError, StopIteration):
        ref = None

    # roofline: FP32 issue (FLOP) and special-function (MUFU) rates
    props = torch.cuda.get_device_properties(dev)
    sms = props.multi_processor_count
    peaks = measured_peaks()
    fmax = float(peaks.get("sm_max_mhz", 2070.0)) * 1e6
    flop = sum(t["events"] * FLOP_PER_EVENT[s["material"]] for t, s in zip(tallies, sims))
    mufu = sum(t["events"] * MUFU_PER_EVENT[s["material"]] for t, s in zip(tallies, sims))
    kt = t_batched / K
    fp32_peak = sms * 128 * 2 * fmax / 1e12
    mufu_peak = sms * 16 * fmax / 1e12
    ach = flop / kt / ws / 1e12          # per GPU
    ach_mufu = mufu / kt / ws / 1e12
    # the binding limit is the larger of the two fractions; both peaks are
    # nominal formulas (the measured-peaks file holds HBM and bf16 GEMM rates)
    fp32 = {"achieved": ach, "peak": fp32_peak, "unit": "TFLOP/s", "frac": ach / fp32_peak,
            "per_event": "176 + 18 n_shells FLOP (FMA = 2)"}
    mufu_ = {"achieved": ach_mufu, "peak": mufu_peak, "unit": "Tops/s", "frac": ach_mufu / mufu_peak,
             "per_event": "17 + 4 n_shells MUFU operations"}
    top, name = (mufu_, "mufu-issue") if mufu_["frac"] >= fp32["frac"] else (fp32, "fp32-issue")
    roofline = {"bound": name, "achieved": top["achieved"], "peak": top["peak"], "unit": top["unit"],
                "frac": top["frac"], "traffic": BATCHED_DRAM_BYTES if args.scale == 1.0 else None,
                "traffic_note": "DRAM bytes per launch from an ncu capture of the full step",
                "fp32": fp32, "mufu": mufu_,
                "issue": {"achieved": value * WARP_INST_PER_EVENT / 1e9 / ws,
                          "peak": sms * 4 * fmax / 1e9, "unit": "G warp instructions/s",
                          "frac": value * WARP_INST_PER_EVENT / ws / (sms * 4 * fmax),
                          "inst_per_event_note": "warp instructions per event from an ncu capture"},
                "ncu": BATCHED_NCU,
                "peak_note": "nominal peaks, not measured: %d SMs x 128 FP32 lanes x 2 FLOP (MUFU: x16 ops) per "
                             "cycle at sm_max_mhz %.0f; frac is the larger of the FP32 and MUFU fractions"
                             % (sms, fmax / 1e6)}

    adj = None if args.no_adjoint else adjoint_bench(args, dev)
    stream = None if args.no_stream else stream_bench(args, dev)
    cont = None if args.no_cont else cont_bench(args, dev)
    det = None if args.no_detector else detector_bench(args, dev)
    tabs = None if args.no_tables else tables_bench(args, dev)
    if args.no_cpu:
        cpu = {"events": 0, "electrons": 0, "times": [float("nan")], "threads": 0, "total": 1}
    else:
        cpu = cpu_sample(sims, sample_sizes(sims), steps=1, seed=args.seed)
        cpu["total"] = sum(s["num_el"] for s in sims)
    cpu_v = cpu["events"] / cpu["times"][0]
    # eta against the FP64 oracle's sample of the first electrons of each
    # simulation: pooled over the (num_el-weighted) sample, and per simulation
    # where the sample holds at least 100 electrons
    vs_oracle = None
    if not args.no_cpu:
        def z2(k1, n1, k2, n2):
            pp = (k1 + k2) / (n1 + n2)
            return abs(k1 / n1 - k2 / n2) / math.sqrt(max(pp * (1 - pp), 1e-12) * (1 / n1 + 1 / n2))
        zo = []
        for k, t in enumerate(tallies):
            if cpu["n"][k] >= 100:
                zo.append(z2(t["bks"], sum(t[o] for o in ("bks", "abs", "trsm", "long")), cpu["bks"][k], cpu["n"][k]))
        ng = sum(sum(t[o] for o in ("bks", "abs", "trsm", "long")) for t in tallies)
        vs_oracle = {"pooled_z": z2(sum(t["bks"] for t in tallies), ng, sum(cpu["bks"]), sum(cpu["n"])),
                     "eta_gpu": sum(t["bks"] for t in tallies) / ng, "eta_oracle": sum(cpu["bks"]) / sum(cpu["n"]),
                     "max_z": max(zo) if zo else None, "sims_with_100": len(zo),
                     "oracle_sample": sample_note(cpu)}
    c1 = None if args.no_cfg1 else cfg1_bench(args, dev)

    line = {
        "metric": "scatter events/s", "value": value, "unit": "events/s", "n_gpus": ws, "steps": K,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_batched / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(sims),
        "electrons_per_step": electrons, "events_per_step": events,
        "parallelism": "%d replicas, counts summed over ranks" % ws if ws > 1 else "1 GPU",
        "tune": {"block": tune.block_size, "refill": tune.refill, "variant": tune.variant,
                 "blocks_per_sm": tune.blocks_per_sm, "autotuned_ms": tune_table, "cuda_graph": True},
        "electrons_per_s": electrons * K / t_batched,
        "plain": {"value": plain_value, "unit": "events/s", "ms_per_step": 1e3 * t_plain / k_plain,
                  "launches_per_step": len(sims), "cross_sections": "one table per simulation"},
        "plain_inline": {"value": plain_inline_value, "unit": "events/s",
                         "ms_per_step": 1e3 * t_plain_inline / k_plain, "launches_per_step": len(sims),
                         "cross_sections": "evaluated per event"},
        "batched_over_plain": value / plain_value,
        "batched_over_plain_inline": value / plain_inline_value,
        "eta": {"batched_vs_plain_max_z": max(zs), "vs_reference": ref, "vs_oracle_fp64": vs_oracle},
        "e2e": {"value": events * K / t_e2e, "unit": "events/s", "h2d_bytes_per_step": int(_lib.lib().mcd_batch_upload_bytes(batch.n)),
                "d2h_bytes_per_step": int(batch.tallies.numel())},
        "roofline": roofline,
        "cpu_baseline": {"value": cpu_v, "unit": "events/s", "cores": cpu["threads"], "kind": "port",
                         "sample": "C oracle, " + sample_note(cpu) if cpu["electrons"] else None},
        "reference_python": reference_python_record(),
        "clocks": clk,
        "adjoint": adj,
        "stream": stream,
        "cont": cont,
        "cfg1": c1,
        "detector": det,
        "tables": tabs,
        "gpu_launches": K,
        "status": status,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=12)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mcd", choices=("mcd", "reference"))
    ap.add_argument("--block", type=int, default=0, help="batched block size (0: autotune)")
    ap.add_argument("--refill", type=int, default=0, help="batched refill granularity (0: autotune)")
    ap.add_argument("--blocks-per-sm", type=int, default=0)
    ap.add_argument("--variant", type=int, default=0, help="batched tune variant bits, with --block")
    ap.add_argument("--plain-block", type=int, default=0, help="plain launch block size (0: automatic)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--scale", type=float, default=1.0,
                    help="multiply every num_el (profiling of small cases); 1 = the benchmark workload")
    ap.add_argument("--no-plain", action="store_true", help="skip the 64-launch plain path")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline sample")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint (bwd/fwd) measurement")
    ap.add_argument("--no-stream", action="store_true", help="skip the streamed-event measurement")
    ap.add_argument("--no-cont", action="store_true", help="skip the continuous-mode histogram measurement")
    ap.add_argument("--no-detector", action="store_true", help="skip the detector-projection measurement")
    ap.add_argument("--no-cfg1", action="store_true", help="skip the small FP64 configuration")
    ap.add_argument("--no-tables", action="store_true", help="skip the table-build timing")
    ap.add_argument("--stream-fraction", type=float, default=1.0,
                    help="fraction of the 1e7-electron streaming workload to run (1 = all of it)")
    ap.add_argument("--section", default="", choices=("", "cfg1", "cont", "adjoint", "stream", "detector", "tables"),
                    help="run one section alone on cuda:0 and print its JSON (for profiling); not the bench line")
    args = ap.parse_args()
    if args.section:
        import torch
        dev = torch.device("cuda", 0)
        torch.cuda.set_device(dev)
        fn = {"cfg1": cfg1_bench, "cont": cont_bench, "adjoint": adjoint_bench, "stream": stream_bench,
              "detector": detector_bench, "tables": tables_bench}[args.section]
        print(json.dumps({args.section: fn(args, dev)}), flush=True)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_mcd(args)


if __name__ == "__main__":
    main()
