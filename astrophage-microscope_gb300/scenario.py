"""Scenario spine: a scenario file (the JSON shape of contracts/scenario_v3.h)
parsed, a World built from it, driven tick by tick, its accept block evaluated.

This is the host-side mirror of the reference's src/sim/scenario.cpp
(scenario_parse, scenario_capacities, scenario_instantiate,
scenario_apply_drive), src/sim/accept.cpp (metric_needs, aggregates_sample,
metric_measure, accept_eval) and tools/headless.cpp:178-258 (`--scenario ID
--assert`), over the engine's C ABI. Names, argument meaning and error
behaviour follow the reference: an unknown accept metric or drive stimulus
kind is a parse error (ScenarioError); unknown enum strings fall back to the
documented defaults; scope, tools, param_overrides, density_model and
thermal_bc are parsed and not applied, as there.

The world is duck-typed: anything with the agb.World operations used below
(spawn with a seed, spawn_taumoeba, import_field, set_light, set_flash,
flash_audit, apply_brush, step, stats, count, export_cells,
export_taumoeba) can be driven, so the same scenario runs on the engine and,
in the tests, on the CPU oracle. Every stage a scenario file can name is
built; ScenarioUnsupported remains for callers that check a scenario against
a world lacking one (a world without an N2 grid cannot take N2 stimuli).
"""
import json
import math
import os
import sys
from dataclasses import dataclass, field
from typing import List

import numpy as np

if __package__ in (None, ""):
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import agb  # noqa: E402


class ScenarioError(Exception):
    """scenario_parse's InvalidArgument: not an object, unknown metric or stimulus."""


class ScenarioUnsupported(Exception):
    """The scenario needs something the world it is given cannot do."""


# contracts/scenario_v3.h enums (values as there).
PLACEMENT = {"uniform": agb.PLACE_UNIFORM, "gaussian": agb.PLACE_GAUSSIAN, "grid": agb.PLACE_GRID,
             "disc": agb.PLACE_DISC}
DISTRIBUTION = {"constant": agb.DIST_CONSTANT, "uniform": agb.DIST_UNIFORM, "normal": agb.DIST_NORMAL}
ASTROPHAGE, TAUMOEBA = 0, 1
CANON_MASS, WATER_DENSITY = 0, 1
REALTIME, MOTION, METABOLIC, GENERATIONAL, CUSTOM = range(5)
HEAT, CHILL, INJECT_CO2, INJECT_N2, SET_LIGHT, SET_N2, SEED_CELLS, FLASH = range(8)
STIMULUS = {"heat": HEAT, "chill": CHILL, "inject_co2": INJECT_CO2, "inject_n2": INJECT_N2,
            "set_light": SET_LIGHT, "set_n2": SET_N2, "seed_cells": SEED_CELLS, "flash": FLASH}
OPS = {"==": "eq", "!=": "ne", "<": "lt", "<=": "le", ">": "gt", ">=": "ge", "~=": "approx"}
# contracts/telemetry_v1.h Metric, in enum order.
METRICS = ["awake_fraction", "medium_temp_mean", "medium_temp_max", "boil_event_count", "population_live",
           "population_dead", "mean_charge", "total_energy_j", "mean_tau_tolerance", "max_tau_tolerance",
           "charge_depth_correlation", "charge_height_correlation", "rise_velocity_empty",
           "fall_velocity_full", "doubling_time_s", "impulse_per_cycle"]
MAX_LIGHT_SOURCES, MAX_POPULATIONS, MAX_ACCEPT_CHECKS, MAX_STIMULI, MAX_OVERRIDES = 8, 8, 16, 16, 32

TOOLS = {"heat": 1 << 0, "chill": 1 << 1, "illuminate": 1 << 2, "inject_co2": 1 << 3, "inject_n2": 1 << 4,
         "seed_cells": 1 << 5, "seed_taumoeba": 1 << 6, "kill": 1 << 7, "charge_beam": 1 << 8}


@dataclass
class Population:
    kind: int = ASTROPHAGE
    count: int = 0
    placement: int = agb.PLACE_UNIFORM
    place_x: float = 0.0
    place_y: float = 0.0
    place_radius: float = 0.0
    charge_dist: int = agb.DIST_CONSTANT
    charge_a: float = 0.0
    charge_b: float = 0.0
    awake: int = 0


@dataclass
class Stimulus:
    kind: int
    t0_s: float = 0.0
    t1_s: float = 0.0
    x: float = 0.0
    y: float = 0.0
    radius: float = 0.0
    v0: float = 0.0
    v1: float = 0.0


@dataclass
class Check:
    metric: str
    op: str = "eq"
    value: float = 0.0
    tol: float = 0.0
    after_s: float = 0.0
    tol_absolute: int = 0


@dataclass
class LightSpec:
    dir_x: float = 1.0
    dir_y: float = 0.0
    irradiance: float = 0.0
    wavelength: float = 0.0
    enabled: int = 0


@dataclass
class Scenario:
    schema: int = 1
    id: str = ""
    title: str = ""
    blurb: str = ""
    seed: int = 20260802
    chamber_w: float = agb.CHAMBER_W
    chamber_h: float = agb.CHAMBER_H
    chamber_d: float = agb.CHAMBER_D
    boundary_x: int = agb.WALL_REFLECTING
    boundary_y: int = agb.WALL_REFLECTING
    temp_init: float = agb.AMBIENT_TEMP_DEFAULT
    co2_init: float = 0.0
    n2_init: float = 0.0
    ambient_temp: float = agb.AMBIENT_TEMP_DEFAULT
    thermal_bc: int = agb.BC_ROBIN
    density_model: int = CANON_MASS
    store_disposition: int = agb.STORE_VOID
    gravity_axis: int = agb.GRAVITY_Y
    thermal_active: int = 1
    compaction: int = 0
    tau_compaction: int = 0
    lights: List[LightSpec] = field(default_factory=list)
    ambient_irradiance: float = 0.0
    populations: List[Population] = field(default_factory=list)
    clock: int = REALTIME
    physics_rate: float = 1.0
    biology_rate: float = 1.0
    tools: int = 0
    param_overrides: dict = field(default_factory=dict)
    drive: List[Stimulus] = field(default_factory=list)
    objective_text: str = ""
    accept: List[Check] = field(default_factory=list)
    run_duration_s: float = 0.0


# json.h accessors: a value of the wrong type reads as the default.
def _num(o, key, d):
    v = o.get(key) if isinstance(o, dict) else None
    return float(v) if isinstance(v, (int, float)) and not isinstance(v, bool) else d


def _flag(o, key, d):
    v = o.get(key) if isinstance(o, dict) else None
    return v if isinstance(v, bool) else d


def _text(o, key, d):
    v = o.get(key) if isinstance(o, dict) else None
    return v if isinstance(v, str) else d


def _obj(o, key):
    v = o.get(key) if isinstance(o, dict) else None
    return v if isinstance(v, dict) else None


def _arr(o, key):
    v = o.get(key) if isinstance(o, dict) else None
    return v if isinstance(v, list) else []


def _trunc(x):
    """static_cast<int> of a double: toward zero."""
    return int(math.trunc(x))


def _strip_comments(text):
    """The scenario files are JSON with `//` and `/* */` comments (the json.h
    reader skips them as whitespace); drop them outside strings."""
    out, i, n = [], 0, len(text)
    while i < n:
        c = text[i]
        if c == '"':
            j = i + 1
            while j < n and text[j] != '"':
                j += 2 if text[j] == "\\" else 1
            out.append(text[i:j + 1])
            i = j + 1
        elif text.startswith("//", i):
            j = text.find("\n", i)
            i = n if j < 0 else j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            i = n if j < 0 else j + 2
            out.append(" ")
        else:
            out.append(c)
            i += 1
    return "".join(out)


def _first_wins(pairs):
    """Object members as json.h keeps them: a lookup finds the first of a repeated key."""
    d = {}
    for k, v in pairs:
        d.setdefault(k, v)
    return d


def parse(text):
    """scenario_parse (src/sim/scenario.cpp:139-317) of a scenario's text."""
    try:
        root = json.loads(_strip_comments(text), object_pairs_hook=_first_wins)
    except ValueError:
        root = None
    if not isinstance(root, dict):
        raise ScenarioError("scenario: not a JSON object")
    s = Scenario()
    s.schema = _trunc(_num(root, "schema", 1))
    s.id, s.title, s.blurb = _text(root, "id", ""), _text(root, "title", ""), _text(root, "blurb", "")
    s.seed = _trunc(_num(root, "seed", 20260802.0)) & 0xFFFFFFFFFFFFFFFF
    ch = _obj(root, "chamber")
    if ch is not None:
        s.chamber_w = _num(ch, "w", agb.CHAMBER_W)
        s.chamber_h = _num(ch, "h", agb.CHAMBER_H)
        s.chamber_d = _num(ch, "d", agb.CHAMBER_D)
        walls = {"periodic": agb.WALL_PERIODIC, "absorbing": agb.WALL_ABSORBING}
        s.boundary_x = walls.get(_text(ch, "boundary_x", "reflecting"), agb.WALL_REFLECTING)
        s.boundary_y = walls.get(_text(ch, "boundary_y", "reflecting"), agb.WALL_REFLECTING)
    md = _obj(root, "medium")
    if md is not None:
        s.temp_init = _num(md, "temp_init", agb.AMBIENT_TEMP_DEFAULT)
        s.co2_init = _num(md, "co2_init", 0.0)
        s.n2_init = _num(md, "n2_init", 0.0)
        s.ambient_temp = _num(md, "ambient_temp", agb.AMBIENT_TEMP_DEFAULT)
        s.thermal_bc = {"dirichlet": agb.BC_DIRICHLET, "neumann": agb.BC_NEUMANN}.get(
            _text(md, "thermal_bc", "robin"), agb.BC_ROBIN)
        s.density_model = WATER_DENSITY if _text(md, "density_model", "canon-mass") == "water-density" else CANON_MASS
        s.store_disposition = {"flash": agb.STORE_FLASH, "retain": agb.STORE_RETAIN}.get(
            _text(md, "store_disposition", "void"), agb.STORE_VOID)
        s.gravity_axis = agb.GRAVITY_Z if _text(md, "gravity_axis", "y") == "z" else agb.GRAVITY_Y
        s.thermal_active = 1 if _flag(md, "thermal_active", True) else 0
    lt = _obj(root, "light")
    if lt is not None:
        s.ambient_irradiance = float(np.float32(_num(lt, "ambient", 0.0)))
        for src in _arr(lt, "sources")[:MAX_LIGHT_SOURCES]:
            s.lights.append(LightSpec(float(np.float32(_num(src, "dir_x", 1.0))),
                                      float(np.float32(_num(src, "dir_y", 0.0))),
                                      float(np.float32(_num(src, "irradiance", 0.0))),
                                      float(np.float32(_num(src, "wavelength", 0.0))), 1))
    for p in _arr(root, "populations")[:MAX_POPULATIONS]:
        ps = Population()
        ps.kind = TAUMOEBA if _text(p, "kind", "astrophage") == "taumoeba" else ASTROPHAGE
        ps.count = _trunc(_num(p, "count", 0))
        ps.placement = PLACEMENT.get(_text(p, "placement", "uniform"), agb.PLACE_UNIFORM)
        ps.place_x, ps.place_y = _num(p, "place_x", 0.0), _num(p, "place_y", 0.0)
        ps.place_radius = _num(p, "place_radius", 0.0)
        cg = p.get("charge") if isinstance(p, dict) and "charge" in p else None
        if cg is not None:
            ps.charge_dist = DISTRIBUTION.get(_text(cg, "dist", "constant"), agb.DIST_CONSTANT)
            ps.charge_a = _num(cg, "value", _num(cg, "a", 0.0))
            ps.charge_b = _num(cg, "b", 0.0)
        ps.awake = 1 if _flag(p, "awake", False) else 0
        s.populations.append(ps)
    s.compaction = 1 if _flag(root, "compaction", False) else 0
    s.tau_compaction = 1 if _flag(root, "tau_compaction", False) else 0
    ck = _obj(root, "clock")
    if ck is not None:
        s.clock = {"motion": MOTION, "metabolic": METABOLIC, "generational": GENERATIONAL,
                   "custom": CUSTOM}.get(_text(ck, "preset", "realtime"), REALTIME)
        s.physics_rate = _num(ck, "physics_rate", 1.0)
        s.biology_rate = _num(ck, "biology_rate", 1.0)
    for t in _arr(root, "tools"):
        if isinstance(t, str):
            s.tools |= TOOLS.get(t, 0)
    for e in _arr(root, "drive")[:MAX_STIMULI]:
        kind = STIMULUS.get(_text(e, "kind", ""))
        if kind is None:
            raise ScenarioError("scenario: unknown drive stimulus kind")
        v0 = _num(e, "v0", _num(e, "value", 0.0))
        s.drive.append(Stimulus(kind, _num(e, "t0_s", 0.0), _num(e, "t1_s", 0.0), _num(e, "x", 0.0),
                                _num(e, "y", 0.0), _num(e, "radius", 0.0), v0, _num(e, "v1", _num(e, "value", v0))))
    po = _obj(root, "param_overrides")
    if po is not None:
        for k, v in list(po.items())[:MAX_OVERRIDES]:
            s.param_overrides[k] = float(v) if isinstance(v, (int, float)) and not isinstance(v, bool) else 0.0
    ob = _obj(root, "objective")
    if ob is not None:
        s.objective_text = _text(ob, "text", "")
        s.run_duration_s = _num(ob, "duration_s", 0.0)
        for c in _arr(ob, "accept")[:MAX_ACCEPT_CHECKS]:
            m = _text(c, "metric", "")
            if m not in METRICS:
                raise ScenarioError("scenario: unknown accept metric")
            s.accept.append(Check(m, OPS.get(_text(c, "op", "=="), "eq"), _num(c, "value", 0.0), _num(c, "tol", 0.0),
                                  _num(c, "after_s", 0.0), 1 if _flag(c, "tol_absolute", False) else 0))
    return s


def load(path):
    """scenario_load: parse the file at `path`."""
    try:
        with open(path, "rb") as fh:
            text = fh.read().decode("utf-8", "replace")
    except OSError:
        raise ScenarioError("scenario: cannot open file")
    return parse(text)


def capacities(s):
    """scenario_capacities (src/sim/scenario.cpp:325-339): (cell, taumoeba) store sizes."""
    cells = sum(p.count for p in s.populations if p.kind != TAUMOEBA)
    tau = sum(p.count for p in s.populations if p.kind == TAUMOEBA)
    cap = min(max(cells * 2 + 4096, agb.DEFAULT_CELLS), agb.MAX_CELLS)
    return int(cap), int(min(tau * 4 + agb.DEFAULT_TAUMOEBA, agb.MAX_TAUMOEBA))


def clock_rates(preset, physics=1.0, biology=1.0):
    """world_set_clock's rates (src/sim/step.cu:190-215): the preset's, or the
    custom pair, clamped to the clock limits."""
    table = {MOTION: (agb.CLOCK_MOTION_PHYSICS, agb.CLOCK_MOTION_BIOLOGY),
             METABOLIC: (agb.CLOCK_METABOLIC_PHYSICS, agb.CLOCK_METABOLIC_BIOLOGY),
             GENERATIONAL: (agb.CLOCK_GENERATIONAL_PHYSICS, agb.CLOCK_GENERATIONAL_BIOLOGY)}
    if preset != CUSTOM:
        physics, biology = table.get(preset, (agb.CLOCK_REALTIME_PHYSICS, agb.CLOCK_REALTIME_BIOLOGY))
    physics = min(max(physics, agb.CLOCK_PHYSICS_MIN), agb.CLOCK_PHYSICS_MAX)
    biology = min(max(biology, agb.CLOCK_BIOLOGY_MIN), agb.CLOCK_BIOLOGY_MAX)
    return physics, biology


def unsupported(s, grids=None):
    """Why `s` cannot run on a world with these grids, or None."""
    if grids is not None and _n2_grid_missing(grids) and (
            s.n2_init != 0.0 or any(d.kind in (INJECT_N2, SET_N2) for d in s.drive)):
        return "the scenario drives N2 and the world has no N2 grid"
    return None


def _n2_grid_missing(grids):
    g = grids.get(agb.FIELD_N2)
    return g is not None and g.nx <= 0


def world_desc(s, grids=None):
    """scenario_instantiate's WorldDesc (src/sim/scenario.cpp:341-357) as an
    agb.WorldDesc. `grids` optionally replaces the default field grids
    (agb.GridDesc per field), e.g. to run a scenario at smaller resolution."""
    cap, tau_cap = capacities(s)   # the predator store is sized too (scenario.cpp:344)
    d = agb.default_desc(capacity=cap, seed=s.seed, co2_init=s.co2_init)
    d.chamber_w, d.chamber_h, d.chamber_d = s.chamber_w, s.chamber_h, s.chamber_d
    d.boundary_x, d.boundary_y = s.boundary_x, s.boundary_y
    d.gravity_axis = s.gravity_axis
    d.ambient_temp = s.ambient_temp
    d.store_disposition = s.store_disposition
    d.thermal_enabled = 1 if s.thermal_active else 0
    d.compaction_enabled = 1 if s.compaction else 0
    d.tau_capacity = tau_cap
    d.tau_compaction_enabled = 1 if s.tau_compaction else 0
    if grids is not None:
        for f, g in grids.items():
            d.grid[f] = g
    # The temperature grid is created at the ambient temperature (src/sim/step.cu:33-35).
    t = d.grid[agb.FIELD_T]
    t.init = s.ambient_temp
    for k in range(6):
        t.face_value[k] = s.ambient_temp
    # The primary light and the ambient irradiance (scenario.cpp:393-394): the
    # first source when the scenario names one, else the world's dark default.
    if s.lights and s.lights[0].enabled:
        L = s.lights[0]
        d.light = agb.Light(L.dir_x, L.dir_y, 0.0, L.irradiance, s.ambient_irradiance, 1)
    else:
        d.light = agb.Light(d.light.dir_x, d.light.dir_y, d.light.dir_z, d.light.irradiance,
                            s.ambient_irradiance, d.light.enabled)
    d.physics_rate, d.biology_rate = clock_rates(s.clock, s.physics_rate, s.biology_rate)
    return d


class Driven:
    """A World built from a scenario, with the host-side state the driver reads
    (World::sim_time_s, tick, seed, chamber, clock, the primary light)."""

    def __init__(self, world, s, desc):
        self.world, self.s, self.desc = world, s, desc
        self.tick = 0
        self.sim_time_s = 0.0
        self.physics_rate, self.biology_rate = desc.physics_rate, desc.biology_rate
        self.light = agb.Light(desc.light.dir_x, desc.light.dir_y, desc.light.dir_z, desc.light.irradiance,
                               desc.light.ambient, desc.light.enabled)
        self.flash = False                  # World::flash_active as last set

    @property
    def dt(self):
        return agb.DT_PHYSICS * self.physics_rate

    def step(self, graph=True):
        """world_step once; the clock advances as World::sim_time_s does."""
        self.world.step(1, graph=graph)
        self.tick += 1
        self.sim_time_s += self.dt


def instantiate(s, make_world=None, grids=None):
    """scenario_instantiate (src/sim/scenario.cpp:341-397): the World, the grid
    fills that differ from creation, one spawn per population with seeds
    seed, seed + 1, ... (populations of count <= 0 take no seed), the light
    and the clock. `make_world(desc)` builds the world (agb.World by default)."""
    why = unsupported(s, grids)
    if why:
        raise ScenarioUnsupported(why)
    d = world_desc(s, grids)
    w = (make_world or agb.World)(d)
    if s.temp_init != s.ambient_temp:
        w.import_field(agb.FIELD_T, np.full(agb.field_shape(d, agb.FIELD_T), s.temp_init, np.float32))
    if s.n2_init != 0.0 and d.grid[agb.FIELD_N2].nx > 0:
        w.import_field(agb.FIELD_N2, np.full(agb.field_shape(d, agb.FIELD_N2), s.n2_init, np.float32))
    seed = s.seed
    for p in s.populations:
        if p.count <= 0:
            continue
        if p.kind == TAUMOEBA:
            w.spawn_taumoeba(p.count, seed)
        else:
            w.spawn(_spawn_of(p, p.count), seed=seed)
        seed = (seed + 1) & 0xFFFFFFFFFFFFFFFF
    return Driven(w, s, d)


def _spawn_of(p, count):
    return agb.spawn(count, placement=p.placement, charge_dist=p.charge_dist, awake=bool(p.awake),
                     place_x=p.place_x, place_y=p.place_y, place_radius=p.place_radius,
                     charge_a=p.charge_a, charge_b=p.charge_b)


def apply_drive(dw):
    """scenario_apply_drive (src/sim/scenario.cpp:399-468) for the current tick:
    every stimulus whose window holds the world's time. Brush strengths are
    rates times this tick's dt; set_light and set_n2 are absolute levels; the
    flash is armed for exactly the ticks inside a flash window."""
    s, w = dw.s, dw.world
    t, dt = dw.sim_time_s, dw.dt
    flash = False
    for st in s.drive:
        open_ended = st.t1_s <= st.t0_s
        if t < st.t0_s:
            continue
        if not open_ended and t >= st.t1_s:
            continue
        frac = (t - st.t0_s) / (st.t1_s - st.t0_s) if not open_ended else 0.0
        strength = st.v0 + (st.v1 - st.v0) * frac
        radius = st.radius if st.radius > 0.0 else 10.0 * (s.chamber_w + s.chamber_h)
        if st.kind in (HEAT, CHILL, INJECT_CO2, INJECT_N2):
            kind = {HEAT: agb.BRUSH_HEAT, CHILL: agb.BRUSH_CHILL, INJECT_CO2: agb.BRUSH_INJECT_CO2,
                    INJECT_N2: agb.BRUSH_INJECT_N2}[st.kind]
            w.apply_brush(kind, st.x, st.y, radius, strength * dt)
        elif st.kind == SET_LIGHT:
            irr = float(np.float32(strength))
            enabled = 1 if strength > 0.0 else 0
            if irr != dw.light.irradiance or enabled != dw.light.enabled:
                dw.light.irradiance, dw.light.enabled = irr, enabled
                w.set_light(dw.light)
        elif st.kind == SET_N2:
            if dw.desc.grid[agb.FIELD_N2].nx > 0:
                w.import_field(agb.FIELD_N2, np.full(agb.field_shape(dw.desc, agb.FIELD_N2), strength, np.float32))
        elif st.kind == SEED_CELLS:
            count = w.count()
            deficit = _trunc(strength) - count
            for p in s.populations:
                if deficit <= 0:
                    break
                if p.kind != ASTROPHAGE:
                    continue
                # cell_store_spawn refuses (and the driver ignores) a spawn past capacity.
                if count + deficit <= dw.desc.capacity:
                    w.spawn(_spawn_of(p, deficit), seed=(s.seed + dw.tick) & 0xFFFFFFFFFFFFFFFF)
                break
        elif st.kind == FLASH:
            flash = True
    if flash != dw.flash:
        w.set_flash(flash)
        dw.flash = flash


# ---------------------------------------------------------------------------
# Acceptance (src/sim/accept.cpp)
# ---------------------------------------------------------------------------
def _seqsum(xs):
    """Left-to-right double sum (the reference's accumulation order)."""
    t = 0.0
    for x in xs:
        t += x
    return t


def _pearson(a, b):
    """Pearson correlation; 0 when undefined (fewer than 2 points, no spread)."""
    n = len(a)
    if n < 2 or len(b) != n:
        return 0.0
    ma, mb = _seqsum(a) / n, _seqsum(b) / n
    sab = saa = sbb = 0.0
    for x, y in zip(a, b):
        da, db = x - ma, y - mb
        sab += da * db
        saa += da * da
        sbb += db * db
    if saa <= 0.0 or sbb <= 0.0:
        return 0.0
    return sab / math.sqrt(saa * sbb)


@dataclass
class Aggregates:
    """RunAggregates (src/sim/accept.h:27-45)."""
    boil_events_total: int = 0
    max_medium_k: float = 0.0
    t_series: list = field(default_factory=list)
    n_series: list = field(default_factory=list)
    vel_stage: int = 0
    vel_ta: float = 0.0
    vel_y_a: list = field(default_factory=list)
    vel_charge_a: list = field(default_factory=list)
    rise_velocity_empty: float = 0.0
    fall_velocity_full: float = 0.0


def metric_needs(s):
    """(velocity, population): the full-state samples the accept block reads."""
    velocity = any(c.metric in ("rise_velocity_empty", "fall_velocity_full") for c in s.accept)
    population = any(c.metric == "doubling_time_s" for c in s.accept)
    return velocity, population


def _positions_energy(w):
    cells, _nid = w.export_cells()
    n = cells.n
    return (np.asarray(cells["x"][:n], np.float64), np.asarray(cells["y"][:n], np.float64),
            np.asarray(cells["energy"][:n], np.float64))


def aggregates_sample(agg, st, dw, needs, settle_s, interval_s):
    """aggregates_sample (src/sim/accept.cpp:127-184): one HUD-rate update."""
    velocity, population = needs
    agg.boil_events_total += st.boil_events
    if st.max_temp_medium_k > agg.max_medium_k:
        agg.max_medium_k = st.max_temp_medium_k
    if population:
        agg.t_series.append(st.sim_time_s)
        agg.n_series.append(float(st.n_live))
    if not velocity:
        return
    if agg.vel_stage == 0 and st.sim_time_s >= settle_s:
        x, y, e = _positions_energy(dw.world)
        if len(y) > 0:
            agg.vel_y_a = list(y)
            agg.vel_charge_a = list(e / agb.CELL_ENERGY_MAX)
            agg.vel_ta = st.sim_time_s
            agg.vel_stage = 1
    elif agg.vel_stage == 1 and st.sim_time_s >= agg.vel_ta + interval_s:
        x, y, _e = _positions_energy(dw.world)
        if len(y) == 0:
            return
        half_h = 0.5 * dw.s.chamber_h
        margin = 3.0 * agb.CELL_DIAMETER                  # drop wall-piled cells
        dt = st.sim_time_s - agg.vel_ta
        m = min(len(y), len(agg.vel_y_a))
        vset, chg = [], []
        for i in range(m):
            if abs(y[i]) > half_h - margin:
                continue
            vset.append(-(y[i] - agg.vel_y_a[i]) / dt)     # downward positive
            chg.append(agg.vel_charge_a[i])
        k = len(vset)
        if k >= 2 and dt > 0.0:
            mc, mv = _seqsum(chg) / k, _seqsum(vset) / k
            scv = scc = 0.0
            for c, v in zip(chg, vset):
                dc = c - mc
                scv += dc * (v - mv)
                scc += dc * dc
            b = scv / scc if scc > 0.0 else 0.0
            a = mv - b * mc
            agg.rise_velocity_empty = a                     # charge 0
            agg.fall_velocity_full = a + b                  # charge 1
        agg.vel_stage = 2


def _doubling_time(agg, biology_rate):
    """Slope of ln N against t below 60 % of the peak, as a culture-time doubling."""
    n = len(agg.n_series)
    if n < 2:
        return 0.0
    npeak = max(agg.n_series)
    if npeak <= 0.0:
        return 0.0
    cap = 0.6 * npeak
    pts = [(t, math.log(N)) for t, N in zip(agg.t_series, agg.n_series) if 0.0 < N <= cap]
    if len(pts) < 2:
        return 0.0
    mt = _seqsum(p[0] for p in pts) / len(pts)
    ml = _seqsum(p[1] for p in pts) / len(pts)
    stl = stt = 0.0
    for t, lg in pts:
        d = t - mt
        stl += d * (lg - ml)
        stt += d * d
    if stt <= 0.0:
        return 0.0
    slope = stl / stt
    if slope <= 0.0:
        return 0.0
    return (math.log(2.0) / slope) * biology_rate


def metric_measure(metric, fin, agg, dw):
    """metric_measure (src/sim/accept.cpp:186-214) at run end."""
    if metric == "awake_fraction":
        return fin.n_awake / fin.n_live if fin.n_live > 0 else 0.0
    if metric == "medium_temp_mean":
        return fin.mean_temp_medium_k
    if metric == "medium_temp_max":
        return agg.max_medium_k
    if metric == "boil_event_count":
        return float(agg.boil_events_total)
    if metric == "population_live":
        return float(fin.n_live)
    if metric == "population_dead":
        return float(fin.n_dead)
    if metric == "mean_charge":
        return fin.mean_charge
    if metric == "total_energy_j":
        return fin.total_energy_j
    if metric in ("charge_height_correlation", "charge_depth_correlation"):
        x, y, e = _positions_energy(dw.world)
        if len(x) < 2:
            return 0.0
        charge = list(e / agb.CELL_ENERGY_MAX)
        if metric == "charge_height_correlation":
            return _pearson(charge, list(y))
        L = dw.s.lights[0] if dw.s.lights else LightSpec()
        return _pearson(charge, [xi * L.dir_x + yi * L.dir_y for xi, yi in zip(x, y)])
    if metric == "rise_velocity_empty":
        return agg.rise_velocity_empty
    if metric == "fall_velocity_full":
        return agg.fall_velocity_full
    if metric == "doubling_time_s":
        return _doubling_time(agg, dw.biology_rate)
    if metric == "mean_tau_tolerance":
        return fin.mean_tau_tolerance
    if metric == "max_tau_tolerance":
        tau, _nid = dw.world.export_taumoeba()
        alive = (tau["flags"] & agb.FLAG_OCCUPIED).astype(bool) & (tau["flags"] & agb.FLAG_ALIVE).astype(bool)
        return float(np.max(tau["tolerance"][alive].astype(np.float64))) if alive.any() else 0.0
    if metric == "impulse_per_cycle":
        imp, dis = dw.world.flash_audit()
        return imp * agb.C_LIGHT / dis if dis > 0.0 else 0.0
    raise ScenarioUnsupported("metric %s needs a stage the engine does not build" % metric)


def accept_eval(c, measured):
    """accept_eval (src/sim/accept.cpp:216-231): exact compares; approx takes a
    relative tolerance unless tol_absolute."""
    if c.op == "eq":
        return measured == c.value
    if c.op == "ne":
        return measured != c.value
    if c.op == "lt":
        return measured < c.value
    if c.op == "le":
        return measured <= c.value
    if c.op == "gt":
        return measured > c.value
    if c.op == "ge":
        return measured >= c.value
    tol = c.tol if c.tol_absolute else c.tol * abs(c.value)
    return abs(measured - c.value) <= tol


# ---------------------------------------------------------------------------
# The headless runner (tools/headless.cpp:178-258)
# ---------------------------------------------------------------------------
SETTLE_S, INTERVAL_S = 2.0, 4.0      # velocity capture windows, physical seconds


def horizon_ticks(s, physics_rate):
    """The --assert horizon: the objective's duration, else the latest accept
    after_s or drive window end, else 60 s; in ticks of this clock."""
    horizon = s.run_duration_s
    if horizon <= 0.0:
        for c in s.accept:
            horizon = max(horizon, c.after_s)
        for d in s.drive:
            horizon = max(horizon, d.t1_s if d.t1_s > d.t0_s else d.t0_s)
    if horizon <= 0.0:
        horizon = 60.0
    return max(1, int(math.ceil(horizon / (agb.DT_PHYSICS * physics_rate))))


def _op_symbol(op):
    return {v: k for k, v in OPS.items()}[op]


def run_assert(s, dw, ticks=None, csv_path=None, graph=True, out=None):
    """run_scenario_assert: drive the world to the horizon, sampling Stats at
    most 2,000 times, then measure every accept check. Returns (accepted,
    [(metric, measured, passed), ...]). An empty accept block passes without
    running (sandbox). Lines of the reference's report go to `out`."""
    say = (lambda m: print(m, file=out)) if out is not None else (lambda m: None)
    if not s.accept:
        say("scenario %s: no objective (sandbox) -- ACCEPT" % s.id)
        return True, []
    n = ticks if ticks and ticks > 0 else horizon_ticks(s, dw.physics_rate)
    stride = n // 2000 if n > 2000 else 1
    needs = metric_needs(s)
    agg = Aggregates()
    csv = open(csv_path, "w") if csv_path else None
    if csv:
        csv.write("# scenario: %s\n# seed: %d\n" % (s.id, s.seed))
        csv.write("t_s,n_live,n_dead,n_tau,mean_charge,total_energy_J,mean_temp_cell_K,"
                  "mean_temp_medium_K,co2_total_kg,mean_tolerance,boil_events,divisions,deaths\n")

    def row(st):
        if csv:
            csv.write("%.6f,%d,%d,%d,%.6f,%.6e,%.4f,%.4f,%.6e,%.6f,%d,%d,%d\n" % (
                st.sim_time_s, st.n_live, st.n_dead, st.n_taumoeba, st.mean_charge, st.total_energy_j,
                st.mean_temp_cell_k, st.mean_temp_medium_k, st.co2_total_kg, st.mean_tau_tolerance,
                st.boil_events, st.divisions_this_window, st.deaths_this_window))

    for t in range(n):
        apply_drive(dw)
        dw.step(graph=graph)
        if t % stride == 0:
            st = dw.world.stats()
            aggregates_sample(agg, st, dw, needs, SETTLE_S, INTERVAL_S)
            row(st)
    st = dw.world.stats()
    aggregates_sample(agg, st, dw, needs, SETTLE_S, INTERVAL_S)
    row(st)
    if csv:
        csv.close()
    say("scenario %s: assert over %.1f s (%d ticks, %d checks)" % (s.id, st.sim_time_s, n, len(s.accept)))
    results, all_pass = [], True
    for c in s.accept:
        measured = metric_measure(c.metric, st, agg, dw)
        ok = accept_eval(c, measured)
        all_pass = all_pass and ok
        results.append((c.metric, measured, ok))
        line = "  [%s] %-26s %-12.6g %s %-.6g" % ("PASS" if ok else "FAIL", c.metric, measured,
                                                 _op_symbol(c.op), c.value)
        if c.op == "approx":
            line += " (tol %.4g%s)" % (c.tol, " abs" if c.tol_absolute else " rel")
        if c.after_s > 0.0:
            line += " [after %.0f s]" % c.after_s
        say(line)
    say("scenario %s: %s" % (s.id, "ACCEPT" if all_pass else "REJECT"))
    return all_pass, results


def main(argv=None):
    """`scenario.py --scenario ID|PATH [--scenarios-dir DIR] [--assert] [--ticks N]
    [--csv PATH]`: headless's scenario mode. Exit status 0 on ACCEPT (or a run
    without --assert), 1 on REJECT, 2 on a bad scenario, 3 when the world cannot run it."""
    import argparse
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--scenario", required=True)
    ap.add_argument("--scenarios-dir", default="scenarios")
    ap.add_argument("--assert", dest="do_assert", action="store_true")
    ap.add_argument("--ticks", type=int, default=0)
    ap.add_argument("--csv", default=None)
    a = ap.parse_args(argv)
    path = a.scenario if os.path.exists(a.scenario) else os.path.join(a.scenarios_dir, a.scenario + ".json")
    try:
        s = load(path)
        dw = instantiate(s)
    except ScenarioError as e:
        print(e)
        return 2
    except ScenarioUnsupported as e:
        print("scenario %s: unsupported: %s" % (s.id, e))
        return 3
    if a.do_assert:
        ok, _ = run_assert(s, dw, ticks=a.ticks, csv_path=a.csv, out=sys.stdout)
        return 0 if ok else 1
    for _ in range(a.ticks if a.ticks > 0 else horizon_ticks(s, dw.physics_rate)):
        apply_drive(dw)
        dw.step()
    st = dw.world.stats()
    print("scenario %s: %d ticks, %.3f s, live %d, dead %d, awake %d" % (
        s.id, dw.tick, st.sim_time_s, st.n_live, st.n_dead, st.n_awake))
    return 0


if __name__ == "__main__":
    sys.exit(main())
