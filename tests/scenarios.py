"""Seeded parity scenarios shared by the golden-fixture generator and the tests.

Every scenario is expressible by the reference (depth-averaged nz = 1 grids,
one boundary condition per field, in-plane light), so the reference itself
(run on the CPU) can produce its expected outputs. Inputs are synthetic and
seeded: PCG32 spawn from the world seed, then a numpy-seeded mutation that
pushes cells across the division, starvation, overheating and wall thresholds.
"""
import hashlib

import numpy as np

from helpers import agb

STAGES = [(agb.STAGE_HASH, "hash"), (agb.STAGE_THERMAL, "thermal"), (agb.STAGE_EMISSION, "emission"),
          (agb.STAGE_MOTION, "motion"), (agb.STAGE_SLOW_FIELDS, "slow_fields"),
          (agb.STAGE_LIFECYCLE, "lifecycle"), (agb.STAGE_CLOCK, "clock")]


def stages_for(desc):
    """world_step's stage order for this world: taxis (stage 3) runs between
    emission and motion only when the world enables it (src/sim/step.cu:161-162)."""
    out = list(STAGES)
    if desc.taxis_enabled:
        out.insert(3, (agb.STAGE_TAXIS, "taxis"))
    return out


def slab_desc(n_t=64, n_c=64, n_n=32, n_i=64, cap=3000, co2=1.0, bio=1e5, bc_t=agb.BC_ROBIN,
              light=(1.0, 0.0, 1e4, 0.0), compaction=0, seed=20260802):
    """The reference's default world (4 mm x 4 mm x 60 um slab) with smaller grids."""
    d = agb.default_desc(capacity=cap, seed=seed, co2_init=co2)
    d.grid[agb.FIELD_T] = agb.grid(n_t, 1, agb.WATER_THERMAL_DIFFUSIVITY, agb.AMBIENT_TEMP_DEFAULT,
                                   agb.DEPOSIT_SCALE[0], bc_t)
    d.grid[agb.FIELD_CO2] = agb.grid(n_c, 1, agb.CO2_DIFFUSIVITY_WATER, co2, agb.DEPOSIT_SCALE[1], agb.BC_NEUMANN)
    d.grid[agb.FIELD_N2] = agb.grid(n_n, 1, agb.N2_DIFFUSIVITY, 0.0, agb.DEPOSIT_SCALE[2], agb.BC_NEUMANN)
    d.grid[agb.FIELD_IRR] = agb.grid(n_i, 1, agb.IRRADIANCE_NOMINAL_DIFFUSIVITY, 0.0, agb.DEPOSIT_SCALE[3],
                                     agb.BC_NEUMANN)
    d.taxis_enabled = 0
    d.compaction_enabled = compaction
    d.biology_rate = bio
    if light is not None:
        d.light = agb.Light(light[0], light[1], 0.0, light[2], light[3], 1)
    return d


def _mut_lifecycle(cells, desc):
    n = cells.n
    rng = np.random.default_rng(1)
    idx = rng.choice(n, n // 4, replace=False)
    cells.a["co2_held"][idx] = agb.CO2_MASS_PER_DIVISION * (1 - 1e-9)
    cells.a["flags"][idx[: n // 10]] |= agb.FLAG_AWAKE
    cells.a["energy"][idx[: n // 20]] = 1e-9
    cells.a["x"][idx[n // 20: n // 16]] = 0.5 * desc.chamber_w - 5.0e-6 + 1e-9


def _fields_hot(desc):
    n = desc.grid[agb.FIELD_T].nx
    t = np.full((1, n, n), agb.AMBIENT_TEMP_DEFAULT, np.float32)
    t[0, n // 4: n // 4 + 6, n // 4: n // 4 + 6] = 600.0   # overheating: > CELL_LETHAL_TEMP
    t[0, n // 2: n // 2 + 8, :] = 372.0                      # ignition band: > setpoint
    return {agb.FIELD_T: t}


def _collinear(cells, desc):
    # tests/physics/test_emission.cu:73-133 (T13): two cells 15 um apart on the
    # light axis; the rear one must see exactly zero irradiance.
    cells.a["x"][:2] = [-7.5e-6, 7.5e-6]
    cells.a["y"][:2] = 0.0
    cells.a["z"][:2] = 0.0
    cells.a["energy"][:2] = 0.0


def _mut_taxis(cells, desc):
    # Force both tumble triggers (run timer past TAXIS_RUN_MAX; a remembered
    # signal above the current one) and mix in dormant and dark cells.
    n = cells.n
    cells.a["run_timer"][0:n:3] = 0.45
    cells.a["taxis_memory"][1:n:3] = 1.0e9
    cells.a["flags"][2:n:7] &= np.uint32(0xFFFFFFFF ^ agb.FLAG_AWAKE)
    cells.a["energy"][5:n:11] = 0.0


def scenarios():
    """name -> dict(desc, spawn, mutate, fields, ticks)."""
    s = {}
    s["slab_uniform"] = dict(
        desc=slab_desc(), ticks=3,
        spawn=agb.spawn(1500, charge_dist=agb.DIST_UNIFORM, charge_a=0.0, charge_b=0.2, awake=True))
    d = slab_desc(bio=1e6, bc_t=agb.BC_DIRICHLET, compaction=1)
    d.boundary_x = agb.WALL_ABSORBING
    s["lifecycle_compaction"] = dict(
        desc=d, ticks=4, mutate=_mut_lifecycle,
        spawn=agb.spawn(1200, placement=agb.PLACE_GAUSSIAN, place_radius=6e-4, charge_dist=agb.DIST_NORMAL,
                        charge_a=0.05, charge_b=0.05))
    s["diagonal_light_dormant"] = dict(
        desc=slab_desc(light=(0.3, -1.0, 5e3, 2.0)), ticks=3,
        spawn=agb.spawn(1000, placement=agb.PLACE_DISC, place_radius=1e-3, charge_dist=agb.DIST_UNIFORM,
                        charge_a=0.0, charge_b=1.0))
    d = slab_desc(n_t=96, n_i=96, light=(-1.0, 0.0, 2e4, 0.0))
    d.store_disposition = 2
    s["hot_field"] = dict(
        desc=d, ticks=3, fields=_fields_hot,
        spawn=agb.spawn(2000, placement=agb.PLACE_GRID, charge_dist=agb.DIST_CONSTANT, charge_a=0.5))
    d = slab_desc(cap=2)
    d.thermal_noise = 0
    d.thermal_enabled = 0
    d.contact_enabled = 0
    d.adhesion_enabled = 0
    s["collinear_shadow"] = dict(desc=d, ticks=1, mutate=_collinear, spawn=agb.spawn(2))
    d = slab_desc(cap=4000, n_t=128, light=(0.0, 1.0, 1e4, 0.0))
    d.contact_enabled = 1
    s["dense_cluster"] = dict(
        desc=d, ticks=2,
        spawn=agb.spawn(4000, placement=agb.PLACE_GAUSSIAN, place_radius=6e-5, charge_dist=agb.DIST_UNIFORM,
                        charge_a=0.0, charge_b=0.2, awake=True))
    d = slab_desc(light=(1.0, 0.0, 1e4, 0.0))
    d.taxis_enabled = 1
    s["taxis_seek"] = dict(
        desc=d, ticks=4, mutate=_mut_taxis,
        spawn=agb.spawn(1500, charge_dist=agb.DIST_UNIFORM, charge_a=0.9, charge_b=1.0, awake=True))
    return s


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:24]


def cells_digest(w):
    cells, nid = w.export_cells()
    out = {name: digest(cells[name]) for name, _ in agb.CELL_FIELDS}
    out["count"] = cells.n
    out["next_id"] = int(nid)
    return out


def snapshot_record(data):
    """Snapshot file (contracts/snapshot_v1.h): its state hash, size and a digest
    of every byte, header included."""
    state_hash = int(np.frombuffer(data[248:256], np.uint64)[0])
    return {"state_hash": "%016x" % state_hash, "bytes": len(data),
            "digest": hashlib.sha256(data).hexdigest()[:24]}


def setup(world, sc):
    """Spawn, then the scenario's mutation and field overrides, identically on any backend."""
    world.spawn(sc["spawn"])
    if sc.get("mutate"):
        cells, nid = world.export_cells()
        sc["mutate"](cells, sc["desc"])
        world.import_cells(cells, nid)
    if sc.get("fields"):
        for f, arr in sc["fields"](sc["desc"]).items():
            world.import_field(f, arr)


def trace(world, sc, full_after=None):
    """Digest of every array after every stage; optionally full arrays after one tick."""
    rec = {"spawn": cells_digest(world), "steps": []}
    setup(world, sc)
    rec["initial"] = cells_digest(world)
    rec["snapshot_initial"] = snapshot_record(world.snapshot(b"golden"))
    full = None
    for t in range(sc["ticks"]):
        for stage, name in stages_for(sc["desc"]):
            world.stage(stage)
            e = {"tick": t, "stage": name, "cells": cells_digest(world),
                 "fields": [digest(world.export_field(f)) for f in range(4)]}
            if stage == agb.STAGE_HASH:
                dims, ks, vs, bs, be = world.export_hash()
                e["hash"] = [digest(dims), digest(ks), digest(vs), digest(bs), digest(be)]
            if stage == agb.STAGE_MOTION:
                e["forces"] = [digest(np.asarray(f, np.float64)) for f in world.export_forces()]
            rec["steps"].append(e)
        if full_after is not None and t == full_after:
            cells, nid = world.export_cells()
            full = {"cell_" + k: v for k, v in cells.as_dict().items()}
            for f in range(4):
                full["field_%d" % f] = world.export_field(f)
    rec["snapshot_final"] = snapshot_record(world.snapshot(b"golden"))
    st = world.stats()
    rec["stats"] = st if isinstance(st, dict) else st.as_dict()
    rec["accum"] = [int(v) for v in world.stats_accum()]
    rec["counters"] = [int(v) for v in world.counters()[:3]]
    return rec, full


# Brush strokes (world_apply_brush, src/sim/step.cu:80-89) on a slab world:
# (kind, x, y, radius, strength). A disc inside the chamber, one crossing the
# chamber's corner, one centred outside it, a chamber-global stroke (radius ten
# times the chamber, as the reference's scenario driver uses), a stroke smaller
# than a voxel, and an empty one (radius 0).
BRUSHES = [(agb.BRUSH_HEAT, 0.0, 0.0, 5.0e-4, 2.5),
           (agb.BRUSH_CHILL, 3.0e-4, -7.0e-4, 2.0e-4, 1.25),
           (agb.BRUSH_INJECT_CO2, 1.9e-3, 1.9e-3, 6.0e-4, 0.75),
           (agb.BRUSH_INJECT_CO2, -2.3e-3, 1.0e-3, 5.0e-4, 0.5),
           (agb.BRUSH_INJECT_N2, 0.0, 0.0, 8.0e-2, 0.3),
           (agb.BRUSH_HEAT, 1.0e-4, 1.0e-4, 1.0e-5, 7.0),
           (agb.BRUSH_CHILL, 0.0, 0.0, 0.0, 9.0)]


def brush_desc():
    return slab_desc(n_t=96, n_c=64, n_n=32, n_i=32, cap=16)


def brush_trace(world):
    """Digest of the temperature, CO2 and N2 fields after each stroke."""
    out = []
    for kind, x, y, r, s in BRUSHES:
        world.apply_brush(kind, x, y, r, s)
        out.append([digest(world.export_field(f)) for f in (agb.FIELD_T, agb.FIELD_CO2, agb.FIELD_N2)])
    return out
