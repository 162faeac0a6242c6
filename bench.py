#!/usr/bin/env python3
"""Throughput of the per-tick physics step on GB300 (cell-steps/s, voxel-steps/s).

Default workload (the plain step at README scale): a 4 mm cubic chamber with
25,000 cells uniform in a 550 um-wide slab, lognormal charge (median 3 %,
sigma_ln 0.5, clipped at 0.2), 128^3 temperature and CO2 grids, light along +x,
division at a stored-energy threshold with compaction every 10 ticks, dt = 1 ms.
Inputs are synthetic and seeded (the engine's own PCG32 spawn).

One bench step is one tick of the whole world, replayed as a CUDA graph. The
L2 cache is flushed (a 256 MB write) between timed steps, outside the timed
intervals, which are CUDA events on the stream the tick runs on.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the reference algorithm on the host cores instead: the
C oracle (a restatement of the reference's kernel bodies, pinned to the
reference's own outputs) over the same world with all host threads.
"""
import argparse
import datetime
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import helpers as H  # noqa: E402  (engine bindings; the oracle only for the CPU legs)

agb = H.agb
METRIC = "cell-steps/s & voxel-steps/s, 1 GB300: plain vs batched+surrogate @<=0.01 K err"
EMAX = agb.CELL_ENERGY_MAX


# ---------------------------------------------------------------------------
# Workloads
# ---------------------------------------------------------------------------
def _grid3(n, D, init, scale, bc, face=None):
    return agb.grid(n, n, D, init, scale, bc, face_value=face)


def workload(name, seed=1):
    """(desc, spawn, description) for the plain-step configurations."""
    if name == "slab25k":
        d = agb.default_desc(capacity=50000, seed=seed, co2_init=1.0)
        d.chamber_w = d.chamber_h = d.chamber_d = 4.0e-3
        d.grid[agb.FIELD_T] = _grid3(128, agb.WATER_THERMAL_DIFFUSIVITY, agb.AMBIENT_TEMP_DEFAULT, 1e9, agb.BC_ROBIN)
        d.grid[agb.FIELD_CO2] = _grid3(128, agb.CO2_DIFFUSIVITY_WATER, 1.0, 1e15, agb.BC_NEUMANN)
        d.grid[agb.FIELD_N2] = agb.GridDesc()
        d.grid[agb.FIELD_IRR] = _grid3(128, agb.IRRADIANCE_NOMINAL_DIFFUSIVITY, 0.0, 1e18, agb.BC_NEUMANN)
        d.taxis_enabled = 0
        d.light = agb.Light(1.0, 0.0, 0.0, 1.0e4, 0.0, 1)
        d.division_predicate = agb.DIVIDE_ENERGY
        d.division_energy = 0.16 * EMAX
        d.compaction_enabled = 1
        d.compaction_period = 10
        d.biology_rate = 1.0e5
        sp = agb.spawn(25000, placement=agb.PLACE_SLAB_X, place_radius=275e-6, charge_dist=agb.DIST_LOGNORMAL,
                       charge_a=0.03, charge_b=0.5, charge_max=0.2, awake=True)
        return d, sp, dict(cells=25000, grid=128, chamber_mm=4.0, light="+x", division="energy>=0.16*Emax",
                           compaction_period=10, hash_cell_um=22.0)
    if name == "cube2k":
        d = agb.default_desc(capacity=4000, seed=seed, co2_init=1.0)
        d.chamber_w = d.chamber_h = d.chamber_d = 400e-6
        face = [373.15, 293.15, 293.15, 293.15, 293.15, 293.15]
        bc = [agb.BC_DIRICHLET] + [agb.BC_NEUMANN] * 5
        d.grid[agb.FIELD_T] = _grid3(64, agb.WATER_THERMAL_DIFFUSIVITY, agb.AMBIENT_TEMP_DEFAULT, 1e9, bc, face)
        d.grid[agb.FIELD_CO2] = _grid3(64, agb.CO2_DIFFUSIVITY_WATER, 1.0, 1e15, agb.BC_NEUMANN)
        d.grid[agb.FIELD_N2] = agb.GridDesc()
        d.grid[agb.FIELD_IRR] = _grid3(64, agb.IRRADIANCE_NOMINAL_DIFFUSIVITY, 0.0, 1e18, agb.BC_NEUMANN)
        d.taxis_enabled = 0
        d.hash_cell_size = 10e-6
        d.light = agb.Light(0.0, 0.0, 1.0, 1.0e4, 0.0, 1)
        sp = agb.spawn(2000, charge_dist=agb.DIST_UNIFORM, charge_a=0.0, charge_b=0.2, awake=True)
        return d, sp, dict(cells=2000, grid=64, chamber_mm=0.4, light="+z", hash_cell_um=10.0)
    if name == "clusters1m":
        d = agb.default_desc(capacity=2000000, seed=seed, co2_init=1.5)
        d.chamber_w = d.chamber_h = d.chamber_d = 4.0e-3
        d.grid[agb.FIELD_T] = _grid3(256, agb.WATER_THERMAL_DIFFUSIVITY, agb.AMBIENT_TEMP_DEFAULT, 1e9, agb.BC_ROBIN)
        d.grid[agb.FIELD_CO2] = _grid3(256, agb.CO2_DIFFUSIVITY_WATER, 1.5, 1e15, agb.BC_NEUMANN)
        d.grid[agb.FIELD_N2] = agb.GridDesc()
        d.grid[agb.FIELD_IRR] = _grid3(256, agb.IRRADIANCE_NOMINAL_DIFFUSIVITY, 0.0, 1e18, agb.BC_NEUMANN)
        d.taxis_enabled = 0
        d.light = agb.Light(0.0, 0.0, 1.0, 1.0e4, 0.0, 1)
        d.compaction_enabled = 1
        d.biology_rate = 1.38e5
        d.hash_cell_size = 10e-6
        # Dormant: awake cells packed ~60 to a 15.6 um voxel overdrive the lumped
        # thermostat exchange past the lethal temperature within a few ticks.
        sp = agb.spawn(1000000, placement=agb.PLACE_CLUSTERS, place_radius=40e-6, clusters=64,
                       cluster_extent=3e-3, charge_dist=agb.DIST_UNIFORM, charge_a=0.0, charge_b=0.2, awake=False)
        return d, sp, dict(cells=1000000, grid=256, chamber_mm=4.0, light="+z", clusters=64, hash_cell_um=10.0,
                           awake=False)
    raise SystemExit("unknown workload " + name)


def batch_workload(n=64, seed=1):
    """The batched ensemble: n independent 4 mm chambers with seeds seed..seed+n-1,
    cell counts log-uniform in [1e3, 2e5], temperature/CO2/irradiance grid edge
    drawn from {64, 96, 128, 192}, charge uniform in [0, q] with q swept
    linearly up to 0.20 over the chambers. Otherwise the slab25k recipe: light
    +x at 1e4 W/m^2, division at 0.16 Emax, compaction every 10 ticks, awake
    cells placed uniformly. Draws come from a numpy generator seeded with seed."""
    rng = np.random.default_rng(seed)
    counts = np.rint(np.exp(rng.uniform(np.log(1.0e3), np.log(2.0e5), n))).astype(int)
    edges = rng.choice([64, 96, 128, 192], n)
    descs, spawns = [], []
    for i in range(n):
        d = agb.default_desc(capacity=int(2 * counts[i]), seed=seed + i, co2_init=1.0)
        d.chamber_w = d.chamber_h = d.chamber_d = 4.0e-3
        e = int(edges[i])
        d.grid[agb.FIELD_T] = _grid3(e, agb.WATER_THERMAL_DIFFUSIVITY, agb.AMBIENT_TEMP_DEFAULT, 1e9, agb.BC_ROBIN)
        d.grid[agb.FIELD_CO2] = _grid3(e, agb.CO2_DIFFUSIVITY_WATER, 1.0, 1e15, agb.BC_NEUMANN)
        d.grid[agb.FIELD_N2] = agb.GridDesc()
        d.grid[agb.FIELD_IRR] = _grid3(e, agb.IRRADIANCE_NOMINAL_DIFFUSIVITY, 0.0, 1e18, agb.BC_NEUMANN)
        d.taxis_enabled = 0
        d.light = agb.Light(1.0, 0.0, 0.0, 1.0e4, 0.0, 1)
        d.division_predicate = agb.DIVIDE_ENERGY
        d.division_energy = 0.16 * EMAX
        d.compaction_enabled = 1
        d.compaction_period = 10
        d.biology_rate = 1.0e5
        q = 0.20 * (i + 1) / n
        descs.append(d)
        spawns.append(agb.spawn(int(counts[i]), charge_dist=agb.DIST_UNIFORM, charge_a=0.0, charge_b=q,
                                awake=True))
    info = dict(chambers=n, cells=int(counts.sum()), cells_min=int(counts.min()), cells_max=int(counts.max()),
                grid_edges={str(k): int((edges == k).sum()) for k in (64, 96, 128, 192)}, chamber_mm=4.0)
    return descs, spawns, info


def run_batch(args, stream, l2_flush, dist=None, rank=0, ws=1):
    """Time the batched ensemble: one graph launch per step for all chambers.
    With several ranks the chambers are sharded (heaviest first onto the
    least-loaded rank); the rate is the sum over ranks over the slowest rank."""
    import torch
    descs, spawns, info = batch_workload(args.batch_chambers, seed=1)
    if ws > 1:
        costs = [sp.count * 200.0 + 8.0 * voxel_steps_per_tick(d) for d, sp in zip(descs, spawns)]
        mine = MR.lpt_shards(costs, ws)[rank]
        descs = [descs[i] for i in mine]
        spawns = [spawns[i] for i in mine]
    t0 = time.perf_counter()
    b = agb.Batch(descs, spawns, agb.batch_opts(autotune=True, lanes=args.batch_lanes,
                                                 staged=bool(args.batch_staged)))
    setup_s = time.perf_counter() - t0
    sh = stream.cuda_stream
    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 20)):           # two compaction periods: every graph captured
            b.step(1, stream=sh)
        torch.cuda.synchronize()
        n0 = sum(c.count() for c in b.chambers)
        k0 = b.graph_kernels()
        ms = []
        for _ in range(args.batch_steps):
            l2_flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            b.step(1, stream=sh)
            e1.record(stream)
            ms.append((e0, e1))
        torch.cuda.synchronize()
        n1 = sum(c.count() for c in b.chambers)
        launches = b.graph_kernels() - k0
    total_s = MR.reduce_max(dist, sum(a.elapsed_time(z) for a, z in ms) / 1e3)
    vox = MR.reduce_sum(dist, sum(voxel_steps_per_tick(d) for d in descs))
    n0 = MR.reduce_sum(dist, n0)
    n1 = MR.reduce_sum(dist, n1)
    classes = {}
    for i in range(b.n):
        t = b.tuning(i).as_dict()
        classes.setdefault(t["size_class"], {"hash_cell_um": round(t["hash_cell_size"] * 1e6, 2),
                                             "ftcs_T": t["ftcs"][0], "chambers": 0})["chambers"] += 1
    peak, _kind = measured_peaks()
    out = {"roofline_step": step_roofline(0.5 * (n0 + n1) * args.batch_steps / total_s,
                                          vox * args.batch_steps / total_s, peak),
           "cell_steps_per_s": 0.5 * (n0 + n1) * args.batch_steps / total_s,
           "voxel_steps_per_s": vox * args.batch_steps / total_s,
           "ms_per_step": total_s * 1e3 / args.batch_steps, "steps": args.batch_steps,
           "cells_start_end": [n0, n1], "gpu_launches": launches, "setup_s": setup_s,
           "lanes": args.batch_lanes or min(args.batch_chambers, 16), "staged": b.staged(),
           "config": dict(info, workload="batch%d" % args.batch_chambers,
                          step="one tick of every chamber, one graph launch"),
           "autotune": classes}
    b.close()
    return out


def surrogate_for(desc, seed=1):
    """A surrogate descriptor matching a world's 3-D temperature and CO2 grids
    (one FTCS pass per tick), trained on windows with heat sources and
    temperature excursions of the size the 25,000-cell run produces."""
    gT, gC = desc.grid[agb.FIELD_T], desc.grid[agb.FIELD_CO2]
    sd = agb.surrogate_desc(nx=gT.nx, ny=gT.ny, nz=gT.nz, extent=desc.chamber_w, dt=agb.DT_PHYSICS * desc.physics_rate,
                            seed=seed)
    sd.diffusivity[0], sd.diffusivity[1] = gT.diffusivity, gC.diffusivity
    sd.init[0], sd.init[1] = gT.init, gC.init
    for k in range(6):
        sd.bc[0][k], sd.face[0][k] = gT.bc[k], gT.face_value[k]
        sd.bc[1][k], sd.face[1][k] = gC.bc[k], gC.face_value[k]
    sd.train_temperature_amplitude = 20.0
    sd.train_heat_per_step = 2.0
    sd.train_source_density = 0.01
    sd.train_uptake_per_step = 1.0e-5
    return sd


def run_surrogate(args, stream):
    """The learned field surrogate on the 25,000-cell setup: train it on the
    GPU, time one network window against the FTCS window it replaces, then
    drive the world's temperature and CO2 grids with it (FTCS judge every 8th
    window, fallback past 0.01 K or 1e-6 energy drift)."""
    import torch
    desc, sp, _info = workload("slab25k", seed=1)
    sd = surrogate_for(desc)
    sg = agb.Surrogate(sd)
    sh = stream.cuda_stream
    t0 = time.perf_counter()
    losses = sg.train(args.surrogate_windows, stream=sh)
    train_s = time.perf_counter() - t0
    shape = (sd.nz, sd.ny, sd.nx)
    T, Cf, qT, qC = [torch.zeros(shape, dtype=torch.float32, device="cuda") for _ in range(4)]

    def timed(fn, reps=10):
        with torch.cuda.stream(stream):
            for _ in range(2):
                fn()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    sg.window(10 ** 7, T.data_ptr(), Cf.data_ptr(), qT.data_ptr(), qC.data_ptr(), stream=sh)
    net_ms = timed(lambda: sg.advance(T.data_ptr(), Cf.data_ptr(), qT.data_ptr(), qC.data_ptr(), judge=-1, stream=sh))
    ftcs_ms = timed(lambda: sg.reference(T.data_ptr(), Cf.data_ptr(), qT.data_ptr(), qC.data_ptr(), stream=sh))
    # Held-out accuracy against the FTCS window, and the do-nothing baseline.
    errs, pers = [], []
    for idx in range(3):
        sg.window(10 ** 8 + idx, T.data_ptr(), Cf.data_ptr(), qT.data_ptr(), qC.data_ptr(), stream=sh)
        rT, rC = T.clone(), Cf.clone()
        sg.reference(rT.data_ptr(), rC.data_ptr(), qT.data_ptr(), qC.data_ptr(), stream=sh)
        pers.append(float((rT - T).abs().max()))
        sg.advance(T.data_ptr(), Cf.data_ptr(), qT.data_ptr(), qC.data_ptr(), judge=-1, stream=sh)
        errs.append(float((T - rT).abs().max()))
    # The world, driven by the surrogate.
    w = agb.World(desc)
    w.spawn(sp)
    steps = sd.steps
    w.attach_surrogate(sg, stream=sh)
    with torch.cuda.stream(stream):
        w.step(steps, stream=sh)                          # one warm-up window
        torch.cuda.synchronize()
        r0 = sg.report()
        n0 = w.count(stream=sh)
        ticks = steps * args.surrogate_windows_run
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        w.step(ticks, stream=sh)
        e1.record(stream)
        torch.cuda.synchronize()
        n1 = w.count(stream=sh)
    el = e0.elapsed_time(e1) / 1e3
    r1 = sg.report()
    vox = 2 * sd.nx * sd.ny * sd.nz
    out = {"train_windows": args.surrogate_windows, "train_s": train_s,
           "loss_first_last": [float(losses[:20].mean()), float(losses[-20:].mean())] if len(losses) >= 20 else None,
           "network_ms_per_window": net_ms, "ftcs_ms_per_window": ftcs_ms,
           "held_out_max_err_K": max(errs), "persistence_max_err_K": max(pers),
           "world": {"workload": "slab25k", "ticks": ticks, "ms_per_step": el * 1e3 / ticks,
                     "cell_steps_per_s": 0.5 * (n0 + n1) * ticks / el, "voxel_steps_per_s": vox * ticks / el,
                     "windows": int(r1.calls - r0.calls), "judged": int(r1.judged - r0.judged),
                     "fallbacks": int(r1.fallbacks - r0.fallbacks),
                     "last_judged_err_K": r1.last_err_temperature, "last_energy_drift": r1.last_energy_drift},
           "note": "voxel-steps counted as the T and CO2 FTCS passes the windows stand for"}
    w.attach_surrogate(None, stream=sh)
    w.close()
    sg.close()
    return out


CELL_STEP_BYTES = 200.0       # algorithmic bytes of one cell-step (state read + written, key, sort, ranges)
VOXEL_STEP_BYTES = 8.0        # one FTCS pass over one FP32 voxel (read + write)


def step_roofline(cell_steps_per_s, voxel_steps_per_s, peak):
    """Whole-step HBM roofline: (cell-steps x 200 B + voxel-steps x 8 B) per
    second against the measured copy bandwidth (moved cells of divisions and
    compactions are not counted)."""
    gbs = (cell_steps_per_s * CELL_STEP_BYTES + voxel_steps_per_s * VOXEL_STEP_BYTES) / 1e9
    return {"achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
            "formula": "(cell_steps/s * 200 B + voxel_steps/s * 8 B) / peak"}


def substeps(desc, f):
    """FTCS passes per tick of field f (src/fields/grid.cuh:51-53; 1/6 bound in 3-D)."""
    g = desc.grid[f]
    if g.nx <= 0:
        return 0
    dx = desc.chamber_w / g.nx
    lim = 6.0 if g.nz > 1 else 4.0
    return int(agb.DT_PHYSICS * desc.physics_rate / (dx * dx / (lim * g.diffusivity))) + 1


def voxel_steps_per_tick(desc):
    """FTCS voxel-steps of one tick: substeps x voxels for T, CO2 and N2."""
    total = 0
    for f in (agb.FIELD_T, agb.FIELD_CO2, agb.FIELD_N2):
        g = desc.grid[f]
        if g.nx > 0:
            total += substeps(desc, f) * g.nx * g.ny * g.nz
    return total


# ---------------------------------------------------------------------------
# Instrumentation
# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region.

    The sampler is started and its first row awaited before the timed region
    opens (nvidia-smi takes a while to start); rows are stamped, and those
    inside [mark_start, mark_end] (widened by one sampling period) are the
    ones reported."""
    PERIOD_MS = 50
    Q = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.out = tempfile.TemporaryFile(mode="w+")

    def start(self):
        self.t0 = self.t1 = None
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", str(self.PERIOD_MS)],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        deadline = time.time() + 5.0
        while time.time() < deadline and self.proc.poll() is None and os.fstat(self.out.fileno()).st_size == 0:
            time.sleep(0.01)

    def mark_start(self):
        self.t0 = datetime.datetime.now()

    def mark_end(self):
        self.t1 = datetime.datetime.now()

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.seek(0)
        rows = [r.split(",") for r in self.out.read().strip().splitlines() if r.strip()]
        if self.t0 is not None and self.t1 is not None:
            slack = datetime.timedelta(milliseconds=self.PERIOD_MS)
            inside = []
            for r in rows:
                try:
                    t = datetime.datetime.strptime(r[0].strip(), "%Y/%m/%d %H:%M:%S.%f")
                except ValueError:
                    continue
                if self.t0 - slack <= t <= self.t1 + slack:
                    inside.append(r)
            if inside:
                rows = inside
        rows = [r[1:] for r in rows]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
            except (ValueError, IndexError):
                continue
            for k, n in enumerate(names):
                if len(r) > 4 + k and r[4 + k].strip().lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(key):
    """DRAM bytes per launch from the committed ncu summary, if present."""
    p = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(p):
        return None
    with open(p) as fh:
        for line in fh:
            parts = line.split()
            if len(parts) >= 2 and parts[0] == key:
                return float(parts[1])
    return None


# ---------------------------------------------------------------------------
# Distributed plumbing (one process per GPU; replicas of independent chambers)
# ---------------------------------------------------------------------------
def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        return rank, ws, local, dist
    return rank, ws, local, None


def _load_multirank():
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "multirank", os.path.join(ROOT, "astrophage-microscope_gb300", "multirank.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


MR = _load_multirank()


def allreduce_max(dist, v):
    return MR.reduce_max(dist, v)


def allreduce_sum(dist, v):
    return MR.reduce_sum(dist, v)


# ---------------------------------------------------------------------------
# Arms
# ---------------------------------------------------------------------------
def cpu_oracle_rate(desc, sp, seconds, threads, state=None):
    """Cell-steps/s of the C oracle on this host's cores over a bounded sample."""
    orc = H.OracleWorld(desc, threads=threads)
    if state is None:
        orc.spawn(sp)
    else:
        cells, nid, fields = state
        orc.import_cells(cells, nid)
        for f, arr in fields.items():
            orc.import_field(f, arr)
    orc.step(1)                               # warm-up tick
    ticks, t0 = 0, time.perf_counter()
    cell_ticks = 0
    while True:
        n = orc.count()
        orc.step(1)
        ticks += 1
        cell_ticks += n
        el = time.perf_counter() - t0
        if el >= seconds or ticks >= 2000:
            break
    orc.close()
    return cell_ticks / el, ticks, el


def run_reference(args, wl):
    rank, ws, _, dist = (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), 0, None)
    if rank != 0:
        return 0
    desc, sp, info = wl
    threads = os.cpu_count() or 1
    orc = H.OracleWorld(desc, threads=threads)
    orc.spawn(sp)
    orc.step(args.warmup)
    cell_ticks, t0 = 0, time.perf_counter()
    for _ in range(args.steps):
        cell_ticks += orc.count()
        orc.step(1)
    el = time.perf_counter() - t0
    value = cell_ticks / el
    vox = voxel_steps_per_tick(desc) * args.steps / el
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded PCG32 spawn)",
            "config": dict({"workload": args.workload}, **info),
            "voxel_steps_per_s": vox,
            "cpu_baseline": {"value": value, "unit": "cell-steps/s", "cores": threads, "kind": "port",
                             "sample": "%d ticks of the full workload (C oracle of the reference algorithm, "
                                       "OpenMP over cells and voxels)" % args.steps},
            "e2e": {"value": value, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def profile_batch(steps, staged=True, chambers=64):
    """The batch (64 chambers unless asked otherwise) after 20 warm-up steps,
    then `steps` steps inside an NVTX range named "timed" (ncu --nvtx
    --nvtx-include "timed/" selects them)."""
    import torch
    descs, spawns, _info = batch_workload(chambers, seed=1)
    b = agb.Batch(descs, spawns, agb.batch_opts(autotune=True, staged=staged))
    st = torch.cuda.Stream()
    sh = st.cuda_stream
    with torch.cuda.stream(st):
        for _ in range(20):
            b.step(1, stream=sh)
        torch.cuda.synchronize()
        k0 = b.graph_kernels()
        torch.cuda.nvtx.range_push("timed")
        for _ in range(steps):
            b.step(1, stream=sh)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
    print("profile-batch: %d steps, %d kernels, staged %s" % (steps, b.graph_kernels() - k0, b.staged()))
    b.close()
    return 0


def profile_stencil(n, passes=6):
    """A world holding one n^3 temperature grid (no cells): `passes` FTCS passes."""
    d = agb.default_desc(capacity=16, seed=1)
    d.taxis_enabled = 0
    d.chamber_w = d.chamber_h = d.chamber_d = 4.0e-3
    d.grid[agb.FIELD_T] = _grid3(n, agb.WATER_THERMAL_DIFFUSIVITY, agb.AMBIENT_TEMP_DEFAULT, 1e9, agb.BC_ROBIN)
    for f in (agb.FIELD_CO2, agb.FIELD_N2, agb.FIELD_IRR):
        d.grid[f] = agb.GridDesc()
    w = agb.World(d)
    rng = np.random.default_rng(5)
    w.import_field(agb.FIELD_T, (290.0 + 80.0 * rng.random((n, n, n))).astype(np.float32))
    dx = d.chamber_w / n
    dt_pass = 0.9 * dx * dx / (6.0 * agb.WATER_THERMAL_DIFFUSIVITY)   # one pass per call
    for _ in range(passes):
        w.diffuse(agb.FIELD_T, dt_pass)
    w.export_field(agb.FIELD_T)
    assert w.counters()[3] == 0
    print("profile-stencil %d^3: %d passes ok" % (n, passes))
    return 0


def profile_surrogate(calls):
    """The surrogate on a 128^3 window: `calls` network windows and one training
    step (small case for ncu: the convolution and weight-gradient kernels)."""
    import torch
    sd = agb.surrogate_desc(seed=1)
    sg = agb.Surrogate(sd)
    shape = (sd.nz, sd.ny, sd.nx)
    T, Cf, qT, qC = [torch.zeros(shape, dtype=torch.float32, device="cuda") for _ in range(4)]
    sg.window(1, T.data_ptr(), Cf.data_ptr(), qT.data_ptr(), qC.data_ptr())
    for _ in range(calls):
        sg.advance(T.data_ptr(), Cf.data_ptr(), qT.data_ptr(), qC.data_ptr(), judge=-1)
    sg.train(1)
    torch.cuda.synchronize()
    assert sg.error_word() == 0
    print("profile-surrogate: %d windows + 1 training step ok" % calls)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--workload", default="slab25k", choices=["slab25k", "cube2k", "clusters1m"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--batch-steps", type=int, default=30,
                    help="timed steps of the batched ensemble reported beside the plain step (0: skip)")
    ap.add_argument("--batch-chambers", type=int, default=64)
    ap.add_argument("--batch-lanes", type=int, default=0)
    ap.add_argument("--batch-staged", type=int, default=1,
                    help="1: one launch per stage over every chamber; 0: each chamber's tick on the lanes")
    ap.add_argument("--batch-only", action="store_true",
                    help="run only the batched ensemble and print its result (profiling)")
    ap.add_argument("--surrogate-windows", type=int, default=1500,
                    help="training windows of the learned field surrogate (0: skip the surrogate leg)")
    ap.add_argument("--surrogate-windows-run", type=int, default=16)
    ap.add_argument("--profile-batch", type=int, default=0,
                    help="only run N steps of the batched ensemble inside an NVTX range (small case for ncu)")
    ap.add_argument("--profile-stencil", type=int, default=0,
                    help="only run a few FTCS passes on an N^3 temperature grid (small case for ncu)")
    ap.add_argument("--profile-surrogate", type=int, default=0,
                    help="only run N surrogate windows and one training step (small case for ncu)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.profile_batch:
        return profile_batch(args.profile_batch, staged=bool(args.batch_staged), chambers=args.batch_chambers)
    if args.profile_stencil:
        return profile_stencil(args.profile_stencil)
    if args.profile_surrogate:
        return profile_surrogate(args.profile_surrogate)

    if args.impl == "reference":
        return run_reference(args, workload(args.workload, seed=1))
    if args.batch_only:
        import torch
        stream = torch.cuda.Stream()
        l2_flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
        print(json.dumps(run_batch(args, stream, l2_flush)))
        return 0

    import torch
    rank, ws, local, dist = dist_init()
    torch.cuda.set_device(local)
    desc, sp, info = workload(args.workload, seed=1 + rank)
    lib = agb.load()
    world = agb.World(desc, lib)
    world.spawn(sp)
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    l2_flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    # Initial state for the CPU baseline (before any tick).
    state0 = None
    if rank == 0 and not args.no_cpu:
        cells0, nid0 = world.export_cells()
        state0 = (cells0, nid0, {f: world.export_field(f) for f in range(4) if desc.grid[f].nx > 0})

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            world.step(1, graph=True, stream=sh)
        torch.cuda.synchronize()
        n_start = world.count(stream=sh)
        kernels_before = world.graph_kernels()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        sampler = ClockSampler(local)
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        sampler.start()
        sampler.mark_start()
        for k in range(args.steps):
            l2_flush.zero_()                           # L2 flush, outside the timed interval
            starts[k].record(stream)
            world.step(1, graph=True, stream=sh)
            ends[k].record(stream)
        torch.cuda.synchronize()
        sampler.mark_end()
        clocks = sampler.stop()
        if dist is not None:
            dist.barrier()
        n_end = world.count(stream=sh)
        launches = world.graph_kernels() - kernels_before
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_s = allreduce_max(dist, sum(step_ms) / 1e3)
    cells_mean = 0.5 * (n_start + n_end)
    cell_steps = allreduce_sum(dist, cells_mean * args.steps)
    vox_steps = allreduce_sum(dist, float(voxel_steps_per_tick(desc)) * args.steps)
    value = cell_steps / total_s

    # Dominant-kernel roofline: the 3-D FTCS pass on the temperature grid. The
    # passes of `reps` diffusion calls are captured in one CUDA graph (so host
    # launch cost is not counted) and each replay, after an L2 flush, is timed
    # with events on the stream it runs on.
    peak, peak_kind = measured_peaks()
    gT = desc.grid[agb.FIELD_T]
    vox_T = gT.nx * gT.ny * gT.nz
    reps, replays = 20, 5
    ftcs_graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        world.diffuse(agb.FIELD_T, agb.DT_PHYSICS, stream=sh)
        torch.cuda.synchronize()
    with torch.cuda.graph(ftcs_graph, stream=stream):
        for _ in range(reps):
            world.diffuse(agb.FIELD_T, agb.DT_PHYSICS, stream=torch.cuda.current_stream().cuda_stream)
    ftcs_ms = 0.0
    with torch.cuda.stream(stream):
        for _ in range(replays):
            l2_flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ftcs_graph.replay()
            e1.record(stream)
            torch.cuda.synchronize()
            ftcs_ms += e0.elapsed_time(e1)
    ftcs_s = ftcs_ms / 1e3 / (replays * reps * substeps(desc, agb.FIELD_T))   # per pass
    algo_bytes = 8.0 * vox_T
    achieved = algo_bytes / ftcs_s / 1e9
    traffic = profile_traffic("ftcs3d_%d" % gT.nx)

    # End to end through the C ABI with host buffers: pinned state in, one tick,
    # state out, every step.
    e2e = None
    if rank == 0:
        n = world.count()
        pinned = agb.CellArrays(n)
        for name, t in agb.CELL_FIELDS:
            pinned.a[name] = torch.empty(max(n, 1), dtype=getattr(torch, np.dtype(t).name),
                                         pin_memory=True).numpy()
        cells, nid = world.export_cells()
        for name, _t in agb.CELL_FIELDS:
            pinned.a[name][:n] = cells[name]
        bytes_state = sum(np.dtype(t).itemsize for _n, t in agb.CELL_FIELDS) * n
        e2e_steps = max(30, args.steps)
        # Untimed warm-up of each loop over a whole compaction period, so that
        # every tick phase has its graph captured before timing starts.
        e2e_warm = max(args.warmup, desc.compaction_period if desc.compaction_period > 0 else 1)

        def fused(k, pinned, nid):
            for _ in range(k):
                pinned, nid = world.step_host(pinned, nid, 1, stream=sh)
            return pinned, nid

        def separate(k, pinned, nid):
            for _ in range(k):
                world.import_cells(pinned, nid, stream=sh)
                world.step(1, graph=True, stream=sh)
                pinned, nid = world.export_cells(stream=sh, into=pinned)
            return pinned, nid

        pinned, nid = fused(e2e_warm, pinned, nid)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pinned, nid = fused(e2e_steps, pinned, nid)
        torch.cuda.synchronize()
        el_fused = time.perf_counter() - t0
        pinned, nid = separate(e2e_warm, pinned, nid)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pinned, nid = separate(e2e_steps, pinned, nid)
        torch.cuda.synchronize()
        el_sep = time.perf_counter() - t0
        e2e = {"value": n * e2e_steps / min(el_fused, el_sep), "unit": "cell-steps/s",
               "h2d_bytes_per_step": bytes_state, "d2h_bytes_per_step": bytes_state,
               "fused_call": n * e2e_steps / el_fused, "separate_calls": n * e2e_steps / el_sep,
               "path": "pinned host SoA in, one graph tick, pinned host SoA out, every step: agb_world_step_host "
                       "(one call) and agb_world_import_cells + agb_world_step_graph + agb_world_export_cells"}

    batched = None
    if args.batch_steps > 0:
        world.close()
        batched = run_batch(args, stream, l2_flush, dist, rank, ws)

    surrogate = None
    if rank == 0 and args.surrogate_windows > 0:
        surrogate = run_surrogate(args, stream)
        surrogate["vs_plain_voxel_steps"] = surrogate["world"]["voxel_steps_per_s"] / (vox_steps / total_s)

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        rate, ticks, el = cpu_oracle_rate(desc, sp, args.cpu_seconds, threads, state0)
        cpu = {"value": rate, "unit": "cell-steps/s", "cores": threads, "kind": "port",
               "sample": "%d ticks (%.1f s) of the same workload from the same initial state, C oracle "
                         "(FP64, OpenMP over cells and voxels)" % (ticks, el)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_s * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 compute, f64 state",
            "data": "synthetic (seeded PCG32 spawn of the workload's distributions)",
            "config": dict({"workload": args.workload, "step": "one tick of the whole chamber",
                            "l2": "flushed between timed steps (256 MB write, untimed)",
                            "parallelism": "replicas (independent chambers per GPU)" if ws > 1 else "single GPU"},
                           **info),
            "voxel_steps_per_s": vox_steps / total_s,
            "cells_start_end": [n_start, n_end],
            "roofline_step": step_roofline(value, vox_steps / total_s, peak),
            "roofline": {"bound": "hbm", "kernel": "ftcs3d (temperature, %d^3)" % gT.nx,
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_source": peak_kind, "algorithmic_bytes_per_launch": algo_bytes,
                         "launch_us": ftcs_s * 1e6, "traffic": traffic,
                         "timing": "mean pass of %d graph-captured back-to-back passes after an L2 flush; "
                                   "field %.0f MB (%s L2)" % (reps * substeps(desc, agb.FIELD_T), 4.0 * vox_T / 1e6,
                                                              "inside" if 8.0 * vox_T < 100e6 else "larger than")},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clocks,
            "batched": batched,
            "surrogate": surrogate,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
