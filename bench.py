#!/usr/bin/env python3
"""Throughput of the per-tick physics step on GB300 (cell-steps/s, voxel-steps/s).

Headline workload (the plain step at README scale, slab25k): a 4 mm cubic
chamber with 25,000 cells uniform in a 550 um-wide slab, lognormal charge
(median 3 %, sigma_ln 0.5, clipped at 0.2), 128^3 temperature and CO2 grids,
light along +x, division at a stored-energy threshold with compaction every 10
ticks, dt = 1 ms. Inputs are synthetic and seeded (the engine's own PCG32
spawn); the workloads live in astrophage-microscope_gb300/workloads.py.

One bench step is one tick of the whole world, replayed as a CUDA graph; every
tick phase's graph is captured during setup, before warm-up. The L2 cache is
flushed (a 256 MB write) between timed steps, outside the timed intervals,
which are CUDA events on the stream the tick runs on. Beside the headline the
line carries: per-step statistics, the duration of each section of the tick
(in-graph timing events) and the roofline of the longest one, one FTCS pass's
roofline, the end-to-end loop through the C ABI with pinned host buffers, the
CPU baseline, the 1M-cell cluster workload (`scaled`, the HBM-graded
configuration), the 64-chamber batch and the learned surrogate.

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
# Workloads (shared with the parity tests)
# ---------------------------------------------------------------------------
W = H.load_workloads()
workload = W.workload
batch_workload = W.batch_workload
substeps = W.substeps
voxel_steps_per_tick = W.voxel_steps_per_tick


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


def run_surrogate(args, stream):
    """The learned field surrogate on the 25,000-cell setup: train it on the GPU
    on windows cut from runs of the plain-step workloads (fields and the cells'
    rasterised heat and uptake sources, on the 128^3 grid), measure it on
    held-out windows against the plain FTCS window and against persistence,
    time a network window against the FTCS window it replaces, repeat for
    longer windows (the error-vs-cost curve), then drive the world's
    temperature and CO2 grids with it (FTCS judge every 8th window, fallback
    past 0.01 K or 1e-6 energy drift)."""
    import torch
    SD = H.load_surrogate_data()
    desc, sp, _info = workload("slab25k", seed=1)
    sh = stream.cuda_stream
    held = list(SD.world_windows(SD.surrogate_desc_for(desc), 9, seed=900, every=7))

    def trained(steps, windows):
        sd = SD.surrogate_desc_for(desc, steps=steps)
        sg = agb.Surrogate(sd)
        t0 = time.perf_counter()
        losses = [sg.train_on(*[x.data_ptr() for x in win], stream=sh)
                  for win in SD.world_windows(sd, windows, seed=100)]
        return sd, sg, np.array(losses, np.float32), time.perf_counter() - t0

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

    def costs(sg, sd):
        T, Cf, qT, qC = [x.clone() for x in held[0]]
        net = timed(lambda: sg.advance(T.data_ptr(), Cf.data_ptr(), qT.data_ptr(), qC.data_ptr(), judge=-1,
                                       stream=sh))
        ftcs = timed(lambda: sg.reference(T.data_ptr(), Cf.data_ptr(), qT.data_ptr(), qC.data_ptr(), stream=sh))
        return net, ftcs

    sd, sg, losses, train_s = trained(16, args.surrogate_windows)
    net_ms, ftcs_ms = costs(sg, sd)
    ev_world = SD.evaluate(sg, held)
    shape = (sd.nz, sd.ny, sd.nx)
    synth = []
    for idx in range(3):
        f = [torch.zeros(shape, dtype=torch.float32, device="cuda") for _ in range(4)]
        sg.window(10 ** 8 + idx, *[x.data_ptr() for x in f], stream=sh)
        synth.append(f)
    ev_synth = SD.evaluate(sg, synth)
    curve = [{"steps": 16, "network_ms": net_ms, "ftcs_ms": ftcs_ms, "speedup_vs_ftcs": ftcs_ms / net_ms,
              "train_windows": args.surrogate_windows, **ev_world}]
    for steps in args.surrogate_curve:
        sd2, sg2, _l2, _t2 = trained(steps, args.surrogate_curve_windows)
        n2, f2 = costs(sg2, sd2)
        curve.append({"steps": steps, "network_ms": n2, "ftcs_ms": f2, "speedup_vs_ftcs": f2 / n2,
                      "train_windows": args.surrogate_curve_windows, **SD.evaluate(sg2, held)})
        sg2.close()
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
           "training_data": "windows cut every tick from seeded runs of cube2k (64^3, resampled), slab25k "
                            "(128^3) and clusters20k (64^3, resampled): T, CO2 and the cells' rasterised heat "
                            "and uptake sources",
           "loss_first_last": [float(losses[:20].mean()), float(losses[-20:].mean())] if len(losses) >= 20 else None,
           "network_ms_per_window": net_ms, "ftcs_ms_per_window": ftcs_ms,
           "held_out_world": ev_world, "held_out_synthetic": ev_synth,
           "held_out_max_err_K": ev_world["net_max_K"], "persistence_max_err_K": ev_world["persistence_max_K"],
           "error_vs_cost": curve,
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


def config_for(args, info, ws):
    """The workload description both arms print (identical keys and values)."""
    return dict({"workload": args.workload, "step": "one tick of the whole chamber",
                 "l2": "flushed between timed steps (256 MB write, untimed)",
                 "parallelism": "replicas (independent chambers per GPU)" if ws > 1 else "single GPU"}, **info)


def run_reference(args, wl):
    rank, ws = int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))
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
            "data": "synthetic (seeded PCG32 spawn of the workload's distributions)",
            "config": config_for(args, info, ws),
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
    d.grid[agb.FIELD_T] = W.grid3(n, agb.WATER_THERMAL_DIFFUSIVITY, agb.AMBIENT_TEMP_DEFAULT, 1e9, agb.BC_ROBIN)
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


# Algorithmic bytes per tick of each section of the tick (the data the section
# must move at least once; neighbour candidates, halo planes and re-reads are
# not counted). n = cells, v(f) = voxels of field f, p(f) = its passes.
#   hash        per cell: position 24 + flags 4 + key/slot written 8, each radix
#               pass 16 (key and slot read and written), ranges and snapshot
#               (sorted key/slot 8, position gather 24, snapshot 16, range 8)
#   cell_pass   per cell: position 24, flags 4, energy 8, biomass 8, emission
#               state 16, own snapshot record 16, trilinear samples of the
#               temperature, CO2 and irradiance fields 3 x 32 read; forces 12,
#               samples 12, irradiance 4, energy 8 written
#   integrate   per cell: position 24, velocity 24, force 12, energy 8,
#               biomass 8, t_local 4, rng 8, id 8, flags 4, co2_local 4 read;
#               position 24, velocity 24, rng 8, flags 4, age 4, CO2 demand 8
#               written
#   lifecycle   per cell: flags 4, co2_local 4, co2_held 8, energy 8, t_local 4
#               read, co2_held 8 and flags 4 written (+ moved cells, not counted)
#   thermal     per cell and substep: position 24, flags 4, energy 8, a voxel
#               4 read; energy 8, temp_cell 4, deposit 8 written
#   t_diffuse   8 B per temperature voxel (the last pass) + 8 B per cell (flush)
#   slow_fields 8 B per CO2/N2 voxel and pass
#   irradiance  per cell 36 B (position, flags, stamp) + 4 B per irradiance voxel
SECTION_BYTES = {
    "hash": lambda n, d, p: n * (92.0 + 16.0 * p),
    "cell_pass": lambda n, d, p: n * (200.0 + 36.0),
    "integrate": lambda n, d, p: n * (176.0),
    "lifecycle": lambda n, d, p: n * 40.0,
    "thermal": lambda n, d, p: n * 60.0 * max(substeps(d, agb.FIELD_T), 1),
    "t_diffuse": lambda n, d, p: 8.0 * _vox(d, agb.FIELD_T) + 8.0 * n,
    "slow_fields": lambda n, d, p: 8.0 * (_vox(d, agb.FIELD_CO2) * substeps(d, agb.FIELD_CO2) +
                                          _vox(d, agb.FIELD_N2) * substeps(d, agb.FIELD_N2)),
    "irradiance": lambda n, d, p: 36.0 * n + 4.0 * _vox(d, agb.FIELD_IRR),
}


def _vox(desc, f):
    g = desc.grid[f]
    return g.nx * g.ny * g.nz if g.nx > 0 else 0


def radix_passes(buckets):
    """Digit passes of the hash sort: 8-bit digits, 9-bit where that saves a
    pass (17-18 and 25-27-bit keys)."""
    bits = max(1, int(buckets).bit_length())
    return -(-bits // 9) if bits in (17, 18, 25, 26, 27) else -(-bits // 8)


def step_stats(ms):
    ms = sorted(ms)
    return {"mean": sum(ms) / len(ms), "median": statistics.median(ms), "min": ms[0], "max": ms[-1]}


def time_sections(world, stream, l2_flush, ticks):
    """Mean duration of each section of the tick over `ticks` graph replays with
    the in-graph section timers on (each replay after an L2 flush)."""
    import torch
    sh = stream.cuda_stream
    world.set_timing(True)
    world.prepare_graphs(1, stream=sh)
    acc = {}
    with torch.cuda.stream(stream):
        for _ in range(ticks):
            l2_flush.zero_()
            world.step(1, graph=True, stream=sh)
            for k, v in world.section_times().items():
                acc.setdefault(k, []).append(v)
    world.set_timing(False)
    return {k: 1e3 * sum(v) / len(v) for k, v in acc.items()}       # microseconds


def dominant_roofline(sections_us, desc, cells, passes, peak, peak_kind):
    """The roofline of the section that takes longest inside the tick."""
    cand = {k: v for k, v in sections_us.items() if k in SECTION_BYTES}
    k = max(cand, key=cand.get)
    algo = SECTION_BYTES[k](cells, desc, passes)
    t = cand[k] * 1e-6
    achieved = algo / t / 1e9
    return {"bound": "hbm", "kernel": k, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind, "algorithmic_bytes_per_launch": algo,
            "launch_us": cand[k], "traffic": None,
            "timing": "mean over timed graph replays of the section's in-graph timing events (L2 flushed "
                      "before each tick); DRAM traffic is in the committed ncu summaries, not measured here"}


def ftcs_pass_roofline(world, desc, stream, l2_flush, peak, peak_kind, reps=20, replays=5):
    """One FTCS pass over the temperature field: the passes of `reps` diffusion
    calls captured in one CUDA graph, each replay after an L2 flush, timed with
    events on the replay stream."""
    import torch
    sh = stream.cuda_stream
    gT = desc.grid[agb.FIELD_T]
    vox = gT.nx * gT.ny * gT.nz
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        world.diffuse(agb.FIELD_T, agb.DT_PHYSICS, stream=sh)
        torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=stream):
        for _ in range(reps):
            world.diffuse(agb.FIELD_T, agb.DT_PHYSICS, stream=torch.cuda.current_stream().cuda_stream)
    tot = 0.0
    with torch.cuda.stream(stream):
        for _ in range(replays):
            l2_flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            g.replay()
            e1.record(stream)
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
    per_pass = tot / 1e3 / (replays * reps * substeps(desc, agb.FIELD_T))
    algo = 8.0 * vox
    ach = algo / per_pass / 1e9
    return {"kernel": "ftcs3d (temperature, %d^3)" % gT.nx, "achieved": ach, "peak": peak, "unit": "GB/s",
            "frac": ach / peak, "peak_source": peak_kind, "algorithmic_bytes_per_launch": algo,
            "launch_us": per_pass * 1e6,
            "timing": "mean pass of %d graph-captured back-to-back passes after an L2 flush; field %.0f MB (%s L2)"
                      % (reps * substeps(desc, agb.FIELD_T), 4.0 * vox / 1e6,
                         "inside" if 8.0 * vox < 100e6 else "larger than")}


def run_plain(name, args, stream, l2_flush, dist, rank, ws, local, warmup, steps, e2e=False, cpu=False):
    """One plain-step leg: setup (spawn, every graph phase captured), `warmup`
    untimed ticks, `steps` timed ticks (one graph replay each, L2 flushed
    between them, outside the timed intervals), then section timers, the FTCS
    pass, and optionally the end-to-end loop and the CPU baseline."""
    import torch
    desc, sp, info = workload(name, seed=1 + rank)
    world = agb.World(desc)
    world.spawn(sp)
    sh = stream.cuda_stream
    state0 = None
    if cpu:
        cells0, nid0 = world.export_cells()
        state0 = (cells0, nid0, {f: world.export_field(f) for f in range(4) if desc.grid[f].nx > 0})
    world.prepare_graphs(1, stream=sh)             # setup: no capture inside warm-up or timing
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            world.step(1, graph=True, stream=sh)
        torch.cuda.synchronize()
        n_start = world.count(stream=sh)
        kernels_before = world.graph_kernels()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        sampler = ClockSampler(local)
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        sampler.start()
        sampler.mark_start()
        for k in range(steps):
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
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    total_s = allreduce_max(dist, sum(step_ms) / 1e3)
    cell_steps = allreduce_sum(dist, 0.5 * (n_start + n_end) * steps)
    vox_steps = allreduce_sum(dist, float(voxel_steps_per_tick(desc)) * steps)
    peak, peak_kind = measured_peaks()
    out = {"workload": name, "config": config_for(argparse.Namespace(workload=name), info, ws),
           "cell_steps_per_s": cell_steps / total_s, "voxel_steps_per_s": vox_steps / total_s,
           "ms_per_step": total_s * 1e3 / steps, "step_ms": step_stats(step_ms),
           "cells_start_end": [n_start, n_end], "gpu_launches": launches, "clocks": clocks,
           "roofline_step": step_roofline(cell_steps / total_s, vox_steps / total_s, peak)}
    cell = desc.hash_cell_size
    buckets = 1
    for extent in (desc.chamber_w, desc.chamber_h, desc.chamber_d):
        buckets *= int(np.ceil(extent / cell - 1e-9))
    passes = radix_passes(buckets)
    sections = time_sections(world, stream, l2_flush, max(10, min(steps, 40)))
    out["sections_us"] = sections
    out["roofline"] = dominant_roofline(sections, desc, 0.5 * (n_start + n_end), passes, peak, peak_kind)
    out["ftcs_pass"] = ftcs_pass_roofline(world, desc, stream, l2_flush, peak, peak_kind)
    if e2e:
        out["e2e"] = e2e_leg(world, desc, args, stream)
    world.close()
    if cpu:
        threads = os.cpu_count() or 1
        rate, ticks, el = cpu_oracle_rate(desc, sp, args.cpu_seconds, threads, state0)
        out["cpu_baseline"] = {"value": rate, "unit": "cell-steps/s", "cores": threads, "kind": "port",
                               "sample": "%d ticks (%.1f s) of the same workload from the same initial state, C "
                                         "oracle (FP64, OpenMP over cells and voxels)" % (ticks, el)}
    return out


def e2e_leg(world, desc, args, stream):
    """End to end through the C ABI with host buffers: pinned state in, one
    tick, state out, every step; the faster of the one-call and the
    separate-calls loop is the value, both are reported."""
    import torch
    sh = stream.cuda_stream
    n = world.count()
    pinned = agb.CellArrays(n)
    for name, t in agb.CELL_FIELDS:
        pinned.a[name] = torch.empty(max(n, 1), dtype=getattr(torch, np.dtype(t).name), pin_memory=True).numpy()
    cells, nid = world.export_cells()
    for name, _t in agb.CELL_FIELDS:
        pinned.a[name][:n] = cells[name]
    bytes_state = sum(np.dtype(t).itemsize for _n, t in agb.CELL_FIELDS) * n
    e2e_steps = max(30, args.steps)
    warm = max(args.warmup, 3)

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

    world.prepare_graphs(1, stream=sh)
    pinned, nid = fused(warm, pinned, nid)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pinned, nid = fused(e2e_steps, pinned, nid)
    torch.cuda.synchronize()
    el_fused = time.perf_counter() - t0
    pinned, nid = separate(warm, pinned, nid)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pinned, nid = separate(e2e_steps, pinned, nid)
    torch.cuda.synchronize()
    el_sep = time.perf_counter() - t0
    return {"value": n * e2e_steps / min(el_fused, el_sep), "unit": "cell-steps/s",
            "h2d_bytes_per_step": bytes_state, "d2h_bytes_per_step": bytes_state,
            "fused_call": n * e2e_steps / el_fused, "separate_calls": n * e2e_steps / el_sep,
            "path": "pinned host SoA in, one graph tick, pinned host SoA out, every step: agb_world_step_host "
                    "(one call) and agb_world_import_cells + agb_world_step_graph + agb_world_export_cells"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--workload", default="slab25k", choices=list(W.PLAIN))
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--scaled", default="clusters1m", choices=list(W.PLAIN) + ["none"],
                    help="second plain-step leg reported beside the headline (the HBM-graded configuration)")
    ap.add_argument("--scaled-steps", type=int, default=20)
    ap.add_argument("--ref200k-steps", type=int, default=50,
                    help="timed ticks of the reference's own 200,000-cell throughput configuration (0: skip)")
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
    ap.add_argument("--surrogate-curve", type=int, nargs="*", default=[32, 64],
                    help="window lengths (FTCS steps) of the error-vs-cost curve beside the 16-step network")
    ap.add_argument("--surrogate-curve-windows", type=int, default=600)
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
    agb.load()
    stream = torch.cuda.Stream()
    l2_flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    head = run_plain(args.workload, args, stream, l2_flush, dist, rank, ws, local, args.warmup, args.steps,
                     e2e=(rank == 0), cpu=(rank == 0 and not args.no_cpu))

    scaled = None
    if args.scaled != "none" and args.scaled != args.workload:
        scaled = run_plain(args.scaled, args, stream, l2_flush, dist, rank, ws, local, 3, args.scaled_steps)
        scaled.pop("config", None)

    ref200k = None
    if args.ref200k_steps > 0:
        # The configuration the reference publishes its hash rebuild and tick
        # rate at (RTX 4070 Ti SUPER): measured here the same way as the headline.
        ref200k = run_plain("ref200k", args, stream, l2_flush, dist, rank, ws, local, 3, args.ref200k_steps)
        ref200k.pop("config", None)
        ref200k["published"] = {"hash_rebuild_ms": 0.110, "ticks_per_s": 281, "hardware": "RTX 4070 Ti SUPER",
                                "source": "reference README.md:110-112"}
        ref200k["hash_rebuild_ms"] = ref200k["sections_us"].get("hash", 0.0) / 1e3
        ref200k["ticks_per_s"] = 1e3 / ref200k["ms_per_step"]

    batched = None
    if args.batch_steps > 0:
        batched = run_batch(args, stream, l2_flush, dist, rank, ws)

    surrogate = None
    if rank == 0 and args.surrogate_windows > 0:
        surrogate = run_surrogate(args, stream)
        surrogate["vs_plain_voxel_steps"] = surrogate["world"]["voxel_steps_per_s"] / head["voxel_steps_per_s"]

    if rank == 0:
        line = {
            "metric": METRIC, "value": head["cell_steps_per_s"], "unit": "cell-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms_per_step"],
            "ms_per_step_median": head["step_ms"]["median"], "ms_per_step_min": head["step_ms"]["min"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 compute, f64 state",
            "data": "synthetic (seeded PCG32 spawn of the workload's distributions)",
            "config": head["config"],
            "voxel_steps_per_s": head["voxel_steps_per_s"],
            "cells_start_end": head["cells_start_end"],
            "roofline": head["roofline"],
            "roofline_step": head["roofline_step"],
            "sections_us": head["sections_us"],
            "ftcs_pass": head["ftcs_pass"],
            "cpu_baseline": head.get("cpu_baseline"),
            "e2e": head.get("e2e"),
            "gpu_launches": head["gpu_launches"],
            "clocks": head["clocks"],
            "setup": "every tick phase's graph captured before warm-up (agb_world_prepare_graphs)",
            "scaled": scaled,
            "ref200k": ref200k,
            "batched": batched,
            "surrogate": surrogate,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
