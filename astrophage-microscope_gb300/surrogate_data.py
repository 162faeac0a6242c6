"""Training and evaluation windows for the learned field surrogate, cut from
runs of the engine's own worlds.

A window is the temperature and CO2 fields of a world at some tick, moved to
the surrogate's grid (trilinear), together with the per-step sources that the
world's cells put into those fields while the surrogate drives them: the
fields stay frozen over a window and the cells' exchange accumulates, so the
sources are constant over it. Each cell is placed in the surrogate's chamber
(its position scaled by the ratio of the chamber sizes) and rasterised into
the voxel that holds it:

  q_T  (T_set - T_voxel) * (1 - exp(-G dt / C)) per awake live cell, in kelvin
       per step, with C = rho c_p dx^3 of the surrogate's voxel: the lumped
       exchange of the thermal stage (thermal.cuh:80-86);
  q_C  -co2_uptake_rate(c_voxel) * dt * biology_rate / voxel volume per live
       cell, in kg/m^3 per step (lifecycle.cuh:24-28, the demand of
       lifecycle.cu:41-57).

The worlds are the plain-step workloads (astrophage-microscope_gb300/
workloads.py): the 2,000-cell 64^3 cube, the 25,000-cell 128^3 slab and the
20,000-cell 64^3 cluster world (the 1M-cell workload's density at a size whose
cells can be exported every tick). torch is used for the resampling only.
"""
import os
import re

import numpy as np

import agb
import workloads as W

HERE = os.path.dirname(os.path.abspath(__file__))
WORKLOADS = ("cube2k", "slab25k", "clusters20k")


def canon(name):
    """A constant of the engine's canon table (include/agb_canon.h)."""
    with open(os.path.join(os.path.dirname(HERE), "include", "agb_canon.h")) as fh:
        m = re.search(r"#define AGB_%s ([-0-9.eE+]+)" % name, fh.read())
    return float(m.group(1))


def _nearest(pos, n, dx):
    i = np.floor((pos.astype(np.float32) + np.float32(0.5 * n * dx)) / np.float32(dx)).astype(np.int64)
    return np.clip(i, 0, n - 1)


def cell_sources(sd, desc, cells, T, Cf):
    """(q_T, q_C) on the surrogate's grid (descriptor sd) from one tick's cells
    of a world (descriptor desc) and the fields T, Cf already on that grid."""
    shape = (sd.nz, sd.ny, sd.nx)
    qT = np.zeros(shape, np.float32)
    qC = np.zeros(shape, np.float32)
    flags = cells["flags"]
    alive = ((flags & agb.FLAG_OCCUPIED) != 0) & ((flags & agb.FLAG_ALIVE) != 0)
    awake = alive & ((flags & agb.FLAG_AWAKE) != 0)
    dx = sd.extent / sd.nx
    span = (sd.nx * dx, sd.ny * dx, sd.nz * dx)
    scale = (span[0] / desc.chamber_w, span[1] / desc.chamber_h, span[2] / desc.chamber_d)
    vol = dx ** 3

    def voxels(mask):
        i = _nearest(cells["x"][mask] * scale[0], sd.nx, dx)
        j = _nearest(cells["y"][mask] * scale[1], sd.ny, dx)
        k = _nearest(cells["z"][mask] * scale[2], sd.nz, dx)
        return k, j, i
    if desc.thermal_enabled:
        cap = canon("WATER_DENSITY") * canon("WATER_SPECIFIC_HEAT") * vol
        relax = -np.expm1(-canon("CONDUCTION_COEFF") * sd.dt / cap)
        k, j, i = voxels(awake)
        dT = relax * (canon("CELL_TEMP_SETPOINT") - T[k, j, i].astype(np.float64))
        np.add.at(qT, (k, j, i), dT.astype(np.float32))
    k, j, i = voxels(alive)
    c = np.maximum(Cf[k, j, i].astype(np.float64), 0.0)
    rate = canon("LIFE_CO2_UPTAKE_MAX") * c / (c + canon("LIFE_CO2_HALF_SATURATION"))
    np.add.at(qC, (k, j, i), (-rate * sd.dt * desc.biology_rate / vol).astype(np.float32))
    return qT, qC


def _to_grid(torch, a, shape):
    """A (nz, ny, nx) field on the device, trilinearly resampled to `shape`."""
    t = torch.as_tensor(a, device="cuda", dtype=torch.float32)[None, None]
    if tuple(a.shape) == tuple(shape):
        return t[0, 0].contiguous()
    return torch.nn.functional.interpolate(t, size=shape, mode="trilinear", align_corners=False)[0, 0].contiguous()


def world_windows(sd, count, seed, names=WORKLOADS, every=2, runs_per_workload=2, warm=3):
    """`count` windows (T, C, q_T, q_C: device tensors on the surrogate grid of
    `sd`) from seeded runs of the workloads (runs_per_workload runs each, seeds
    seed, seed + 1, ...), taken in turn from every run, one window every
    `every` ticks of a run, so that consecutive windows come from different
    worlds."""
    import torch
    shape = (sd.nz, sd.ny, sd.nx)
    runs = []
    for r in range(runs_per_workload):
        for name in names:
            desc, sp, _ = W.workload(name, seed=seed + len(runs))
            w = agb.World(desc)
            w.spawn(sp)
            w.step(warm, graph=True)
            runs.append((desc, w))
    try:
        for made in range(count):
            desc, w = runs[made % len(runs)]
            T = _to_grid(torch, w.export_field(agb.FIELD_T), shape)
            Cf = _to_grid(torch, w.export_field(agb.FIELD_CO2), shape)
            cells, _nid = w.export_cells()
            qT, qC = cell_sources(sd, desc, cells, T.cpu().numpy(), Cf.cpu().numpy())
            yield T, Cf, torch.as_tensor(qT, device="cuda"), torch.as_tensor(qC, device="cuda")
            w.step(every, graph=True)
    finally:
        for _desc, w in runs:
            w.close()


def surrogate_desc_for(desc, seed=1, steps=16):
    """A surrogate descriptor matching a world's 3-D temperature and CO2 grids
    (one FTCS pass per tick), normalised for the temperature excursions and
    cell heat sources of the 25,000-cell run."""
    gT, gC = desc.grid[agb.FIELD_T], desc.grid[agb.FIELD_CO2]
    sd = agb.surrogate_desc(nx=gT.nx, ny=gT.ny, nz=gT.nz, extent=desc.chamber_w,
                            dt=agb.DT_PHYSICS * desc.physics_rate, seed=seed)
    sd.steps = steps
    sd.diffusivity[0], sd.diffusivity[1] = gT.diffusivity, gC.diffusivity
    sd.init[0], sd.init[1] = gT.init, gC.init
    for k in range(6):
        sd.bc[0][k], sd.face[0][k] = gT.bc[k], gT.face_value[k]
        sd.bc[1][k], sd.face[1][k] = gC.bc[k], gC.face_value[k]
    sd.train_temperature_amplitude = 20.0
    sd.train_heat_per_step = 2.0
    sd.train_source_density = 0.01
    sd.train_uptake_per_step = 1.0e-5
    sd.learning_rate = 3.0e-4
    return sd


def evaluate(sg, windows):
    """Largest and RMS temperature error of the network's window against the
    plain FTCS window, and the same for persistence (leaving the fields as
    they are), over the given windows."""
    import torch
    net_max = net_rms = per_max = per_rms = 0.0
    n = 0
    for T, Cf, qT, qC in windows:
        rT, rC = T.clone(), Cf.clone()
        sg.reference(rT.data_ptr(), rC.data_ptr(), qT.data_ptr(), qC.data_ptr())
        xT, xC = T.clone(), Cf.clone()
        sg.advance(xT.data_ptr(), xC.data_ptr(), qT.data_ptr(), qC.data_ptr(), judge=-1)
        e, p = (xT - rT).abs(), (T - rT).abs()
        net_max, per_max = max(net_max, float(e.max())), max(per_max, float(p.max()))
        net_rms += float(e.pow(2).mean())
        per_rms += float(p.pow(2).mean())
        n += 1
    torch.cuda.synchronize()
    return {"net_max_K": net_max, "net_rms_K": (net_rms / max(n, 1)) ** 0.5,
            "persistence_max_K": per_max, "persistence_rms_K": (per_rms / max(n, 1)) ** 0.5, "windows": n}
