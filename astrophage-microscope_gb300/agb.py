"""ctypes mirror of include/agb.h: the host-side interface of libagb.so.

The structures are field-for-field copies of the C ABI; World wraps the
engine's world handle with the reference's World operations
(src/sim/world.cuh:183-243): create, spawn, import/export of the contract
cell layout (contracts/cell_store_v1.h), step, per-stage calls and stats.
Loading the library needs no GPU; every compute call does, and fails loudly
(AgbError) when the CUDA engine cannot run.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libagb.so")

ABI_VERSION = 1
OK = 0
STATUS_NAMES = ["Ok", "OutOfMemory", "CudaError", "InvalidArgument", "NotFound", "ParseError",
                "ContractVersionMismatch", "CapacityExceeded", "FileIoError", "Unsupported",
                "DeviceTimeout"]
BC_DIRICHLET, BC_NEUMANN, BC_ROBIN = 0, 1, 2
FIELD_T, FIELD_CO2, FIELD_N2, FIELD_IRR = 0, 1, 2, 3
BRUSH_HEAT, BRUSH_CHILL, BRUSH_INJECT_CO2, BRUSH_INJECT_N2 = 0, 1, 2, 3       # src/sim/world.cuh:33
WALL_REFLECTING, WALL_PERIODIC, WALL_ABSORBING = 0, 1, 2
GRAVITY_Y, GRAVITY_Z = 0, 1
STORE_VOID, STORE_FLASH, STORE_RETAIN = 0, 1, 2
DIVIDE_CO2_QUOTA, DIVIDE_ENERGY = 0, 1
PLACE_UNIFORM, PLACE_GAUSSIAN, PLACE_GRID, PLACE_DISC, PLACE_SLAB_X, PLACE_CLUSTERS = range(6)
DIST_CONSTANT, DIST_UNIFORM, DIST_NORMAL, DIST_LOGNORMAL = range(4)
STAGE_HASH, STAGE_THERMAL, STAGE_EMISSION, STAGE_TAXIS, STAGE_MOTION = 0, 1, 2, 3, 4
STAGE_SLOW_FIELDS, STAGE_LIFECYCLE, STAGE_COMPACT, STAGE_CLOCK, STAGE_FLASH, STAGE_PREDATION = 5, 6, 7, 8, 9, 10
FLAG_OCCUPIED, FLAG_ALIVE, FLAG_AWAKE, FLAG_STUCK = 1, 2, 4, 8

# Canon values the Python side needs (include/agb_canon.h).
CELL_RADIUS = 5.0000000000000004e-06
CELL_DIAMETER = 1.0000000000000001e-05
CELL_ENERGY_MAX = 1500000.0
DT_PHYSICS = 0.001
AMBIENT_TEMP_DEFAULT = 293.14999999999998
WATER_THERMAL_DIFFUSIVITY = 1.4325163582348751e-07
CO2_DIFFUSIVITY_WATER = 1.92e-09
N2_DIFFUSIVITY = 2.0e-9
IRRADIANCE_NOMINAL_DIFFUSIVITY = 1.0e-9
DEPOSIT_SCALE = (1.0e9, 1.0e15, 1.0e15, 1.0e18)
CO2_MASS_PER_DIVISION = 2.0999999999999999e-14
HASH_CELL_FACTOR = 2.2000000000000002
PETROVA_MAX_POWER = 0.050000000000000003
AIR_CONVECTION_H = 10.0
WATER_CONDUCTIVITY = 0.59799999999999998
C_LIGHT = 299792458.0
PETROVA_FLASH_POWER = 3000000.0
CHAMBER_W, CHAMBER_H, CHAMBER_D = 0.0040000000000000001, 0.0040000000000000001, 6.0000000000000002e-05
DEFAULT_CELLS, MAX_CELLS = 25000, 2000000
DEFAULT_TAUMOEBA, MAX_TAUMOEBA = 256, 65536
CLOCK_PHYSICS_MIN, CLOCK_PHYSICS_MAX = 0.10000000000000001, 100.0
CLOCK_BIOLOGY_MIN, CLOCK_BIOLOGY_MAX = 1.0, 1000000.0
CLOCK_REALTIME_PHYSICS, CLOCK_REALTIME_BIOLOGY = 1.0, 1.0
CLOCK_MOTION_PHYSICS, CLOCK_MOTION_BIOLOGY = 10.0, 1.0
CLOCK_METABOLIC_PHYSICS, CLOCK_METABOLIC_BIOLOGY = 1.0, 10000.0
CLOCK_GENERATIONAL_PHYSICS, CLOCK_GENERATIONAL_BIOLOGY = 0.5, 1000000.0


class GridDesc(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("bc", C.c_int32 * 6), ("face_value", C.c_double * 6),
                ("diffusivity", C.c_double), ("init", C.c_double), ("deposit_scale", C.c_double)]


class Light(C.Structure):
    _fields_ = [("dir_x", C.c_float), ("dir_y", C.c_float), ("dir_z", C.c_float),
                ("irradiance", C.c_float), ("ambient", C.c_float), ("enabled", C.c_int32)]


class WorldDesc(C.Structure):
    _fields_ = [("abi_version", C.c_uint32),
                ("chamber_w", C.c_double), ("chamber_h", C.c_double), ("chamber_d", C.c_double),
                ("capacity", C.c_int32), ("seed", C.c_uint64),
                ("boundary_x", C.c_int32), ("boundary_y", C.c_int32), ("gravity_axis", C.c_int32),
                ("thermal_noise", C.c_uint8), ("contact_enabled", C.c_uint8),
                ("adhesion_enabled", C.c_uint8), ("thermal_enabled", C.c_uint8),
                ("emission_enabled", C.c_uint8), ("taxis_enabled", C.c_uint8),
                ("occlusion_exact", C.c_uint8), ("compaction_enabled", C.c_uint8),
                ("store_disposition", C.c_int32), ("ambient_temp", C.c_double),
                ("grid", GridDesc * 4), ("hash_cell_size", C.c_double), ("light", Light),
                ("physics_rate", C.c_double), ("biology_rate", C.c_double),
                ("co2_mass_per_division", C.c_double), ("max_emit_power", C.c_double),
                ("division_predicate", C.c_int32), ("division_energy", C.c_double),
                ("compaction_period", C.c_int32), ("trap_slot", C.c_int32),
                ("trap_x", C.c_double), ("trap_y", C.c_double), ("trap_stiffness", C.c_double),
                ("tau_capacity", C.c_int32), ("tau_compaction_enabled", C.c_int32)]


# The 25 arrays of contracts/cell_store_v1.h:42-75, in declaration order.
CELL_FIELDS = [("id", np.uint64), ("flags", np.uint32), ("death_cause", np.uint8),
               ("x", np.float64), ("y", np.float64), ("z", np.float64),
               ("vx", np.float64), ("vy", np.float64), ("vz", np.float64),
               ("energy", np.float64), ("temp_cell", np.float32), ("emit_power", np.float32),
               ("dir_x", np.float32), ("dir_y", np.float32), ("dir_z", np.float32),
               ("biomass", np.float64), ("co2_held", np.float64), ("age_s", np.float32),
               ("rng_state", np.uint64), ("taxis_memory", np.float32), ("run_timer", np.float32),
               ("t_local", np.float32), ("irradiance", np.float32), ("co2_local", np.float32),
               ("n2_local", np.float32)]
_CT = {np.uint64: C.c_uint64, np.uint32: C.c_uint32, np.uint8: C.c_uint8, np.int32: C.c_int32,
       np.float64: C.c_double, np.float32: C.c_float}


class Cells(C.Structure):
    _fields_ = [(n, C.POINTER(_CT[t])) for n, t in CELL_FIELDS] + [("count", C.c_int32), ("capacity", C.c_int32)]


class Taumoeba(C.Structure):
    """agb_taumoeba: one pointer per predator-store array."""
    _fields_ = [("id", C.POINTER(C.c_uint64)), ("flags", C.POINTER(C.c_uint32)),
                ("x", C.POINTER(C.c_double)), ("y", C.POINTER(C.c_double)), ("z", C.POINTER(C.c_double)),
                ("vx", C.POINTER(C.c_double)), ("vy", C.POINTER(C.c_double)), ("vz", C.POINTER(C.c_double)),
                ("dir_x", C.POINTER(C.c_float)), ("dir_y", C.POINTER(C.c_float)), ("dir_z", C.POINTER(C.c_float)),
                ("biomass", C.POINTER(C.c_double)), ("prey_biomass", C.POINTER(C.c_double)),
                ("digest_timer", C.POINTER(C.c_float)), ("tolerance", C.POINTER(C.c_float)),
                ("generation", C.POINTER(C.c_uint32)), ("rng_state", C.POINTER(C.c_uint64)),
                ("density_ema", C.POINTER(C.c_float)), ("run_timer", C.POINTER(C.c_float)),
                ("target", C.POINTER(C.c_int32))]


class Mirror(C.Structure):
    """agb_mirror: a world's host-visible state after a tick, read in one go."""
    _fields_ = [("cells", Cells), ("next_id", C.c_uint64), ("divisions_this_window", C.c_int64),
                ("deaths_total", C.c_int64), ("dead_slots_prev", C.c_int64), ("error", C.c_uint32),
                ("tau_count", C.c_int32), ("tau_next_id", C.c_uint64)]


class Spawn(C.Structure):
    _fields_ = [("count", C.c_int32), ("placement", C.c_int32), ("charge_dist", C.c_int32),
                ("awake", C.c_int32), ("place_x", C.c_double), ("place_y", C.c_double),
                ("place_radius", C.c_double), ("charge_a", C.c_double), ("charge_b", C.c_double),
                ("charge_max", C.c_double), ("clusters", C.c_int32), ("cluster_extent", C.c_double)]


class Stats(C.Structure):
    _fields_ = [("tick", C.c_uint64), ("sim_time_s", C.c_double),
                ("n_live", C.c_int32), ("n_dead", C.c_int32), ("n_dormant", C.c_int32),
                ("n_awake", C.c_int32), ("n_taumoeba", C.c_int32),
                ("mean_charge", C.c_double), ("total_energy_j", C.c_double),
                ("mean_temp_cell_k", C.c_double), ("mean_temp_medium_k", C.c_double),
                ("max_temp_medium_k", C.c_double), ("co2_total_kg", C.c_double),
                ("n2_total_kg", C.c_double), ("mean_tau_tolerance", C.c_double),
                ("divisions_this_window", C.c_int32), ("deaths_this_window", C.c_int32),
                ("boil_events", C.c_int32), ("ignitions_this_window", C.c_int32),
                ("physics_rate", C.c_double), ("biology_rate", C.c_double),
                ("non_canon_run", C.c_uint8)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class BatchOpts(C.Structure):
    _fields_ = [("abi_version", C.c_uint32), ("lanes", C.c_int32), ("autotune", C.c_int32),
                ("n_hash_candidates", C.c_int32), ("hash_candidates", C.c_double * 8),
                ("probe_ticks", C.c_int32), ("staged", C.c_int32)]


class Tuning(C.Structure):
    _fields_ = [("hash_cell_size", C.c_double), ("size_class", C.c_int32), ("lane", C.c_int32),
                ("ftcs_lx", C.c_int32 * 3), ("ftcs_rpt", C.c_int32 * 3), ("ftcs_zc", C.c_int32 * 3),
                ("probe_tick_ms", C.c_float), ("probe_pass_us", C.c_float)]

    def as_dict(self):
        return {"hash_cell_size": self.hash_cell_size, "size_class": self.size_class, "lane": self.lane,
                "ftcs": [[self.ftcs_lx[f], self.ftcs_rpt[f], self.ftcs_zc[f]] for f in range(3)],
                "probe_tick_ms": self.probe_tick_ms, "probe_pass_us": self.probe_pass_us}


def grid(n, nz, diffusivity, init, scale, bc, face_value=None):
    g = GridDesc()
    g.nx, g.ny, g.nz = n, n, nz
    for f in range(6):
        g.bc[f] = bc if isinstance(bc, int) else bc[f]
        fv = init if face_value is None else face_value
        g.face_value[f] = fv if not isinstance(fv, (list, tuple)) else fv[f]
    g.diffusivity, g.init, g.deposit_scale = diffusivity, init, scale
    return g


def default_desc(capacity=25000, seed=20260802, co2_init=0.0):
    """The reference world (src/sim/step.cu:9-78, src/sim/world.cuh:48-87):
    4 mm x 4 mm x 60 um slab, 512^2 temperature (Robin at ambient), 256^2 CO2,
    128^2 N2 and 512^2 irradiance grids, all depth-averaged (nz = 1).
    Mirrors agb_world_desc_default() in the engine."""
    d = WorldDesc()
    d.abi_version = ABI_VERSION
    d.chamber_w, d.chamber_h, d.chamber_d = 0.0040000000000000001, 0.0040000000000000001, 6.0000000000000002e-05
    d.capacity, d.seed = capacity, seed
    d.boundary_x = d.boundary_y = WALL_REFLECTING
    d.gravity_axis = GRAVITY_Y
    d.thermal_noise = d.contact_enabled = d.adhesion_enabled = 1
    d.thermal_enabled = d.emission_enabled = d.taxis_enabled = d.occlusion_exact = 1
    d.compaction_enabled = 0
    d.store_disposition = 0
    d.ambient_temp = AMBIENT_TEMP_DEFAULT
    d.grid[FIELD_T] = grid(512, 1, WATER_THERMAL_DIFFUSIVITY, AMBIENT_TEMP_DEFAULT, DEPOSIT_SCALE[0], BC_ROBIN)
    d.grid[FIELD_CO2] = grid(256, 1, CO2_DIFFUSIVITY_WATER, co2_init, DEPOSIT_SCALE[1], BC_NEUMANN)
    d.grid[FIELD_N2] = grid(128, 1, N2_DIFFUSIVITY, 0.0, DEPOSIT_SCALE[2], BC_NEUMANN)
    d.grid[FIELD_IRR] = grid(512, 1, IRRADIANCE_NOMINAL_DIFFUSIVITY, 0.0, DEPOSIT_SCALE[3], BC_NEUMANN)
    d.hash_cell_size = HASH_CELL_FACTOR * CELL_DIAMETER
    d.light = Light(1.0, 0.0, 0.0, 0.0, 0.0, 0)
    d.physics_rate, d.biology_rate = 1.0, 1.0
    d.co2_mass_per_division = CO2_MASS_PER_DIVISION
    d.max_emit_power = PETROVA_MAX_POWER
    d.division_predicate, d.division_energy = DIVIDE_CO2_QUOTA, 0.0
    d.compaction_period = 1
    d.trap_slot, d.trap_x, d.trap_y, d.trap_stiffness = -1, 0.0, 0.0, 0.0
    d.tau_capacity, d.tau_compaction_enabled = 0, 0
    return d


def spawn(count, placement=PLACE_UNIFORM, charge_dist=DIST_CONSTANT, awake=False,
          place_x=0.0, place_y=0.0, place_radius=0.0, charge_a=0.0, charge_b=0.0,
          charge_max=0.0, clusters=0, cluster_extent=0.0):
    return Spawn(count, placement, charge_dist, int(bool(awake)), place_x, place_y, place_radius,
                 charge_a, charge_b, charge_max, clusters, cluster_extent)


# TaumoebaStore (src/sim/predation.cuh:85-105), field for field.
TAU_FIELDS = [("id", np.uint64), ("flags", np.uint32), ("x", np.float64), ("y", np.float64), ("z", np.float64),
              ("vx", np.float64), ("vy", np.float64), ("vz", np.float64), ("dir_x", np.float32),
              ("dir_y", np.float32), ("dir_z", np.float32), ("biomass", np.float64), ("prey_biomass", np.float64),
              ("digest_timer", np.float32), ("tolerance", np.float32), ("generation", np.uint32),
              ("rng_state", np.uint64), ("density_ema", np.float32), ("run_timer", np.float32),
              ("target", np.int32)]


class TaumoebaArrays:
    """Host buffers of the predator store, one numpy array per field."""

    def __init__(self, n):
        self.n = n
        self.a = {name: np.zeros(max(n, 1), dtype=t) for name, t in TAU_FIELDS}

    def struct(self):
        t = Taumoeba()
        for name, ty in TAU_FIELDS:
            setattr(t, name, self.a[name].ctypes.data_as(C.POINTER(_CT[ty])))
        return t

    def __getitem__(self, k):
        return self.a[k][:self.n]


class CellArrays:
    """Host buffers in contract layout, one numpy array per SoA field."""

    def __init__(self, n):
        self.n = n
        self.a = {name: np.zeros(max(n, 1), dtype=t) for name, t in CELL_FIELDS}

    def struct(self):
        """The agb_cells view of the arrays. Building it costs tens of
        microseconds (25 ctypes pointer casts), so it is kept while the same
        array objects stay in `a`; the kept references also stop a replaced
        array's id from being reused by a new one."""
        arrs = [self.a[name] for name, _t in CELL_FIELDS]
        held = getattr(self, "_struct_arrays", None)
        if held is not None and all(x is y for x, y in zip(held, arrs)):
            return self._struct
        c = Cells()
        for (name, t), arr in zip(CELL_FIELDS, arrs):
            setattr(c, name, arr.ctypes.data_as(C.POINTER(_CT[t])))
        self._struct, self._struct_arrays = c, arrs
        return c

    def __getitem__(self, k):
        return self.a[k][:self.n]

    def copy(self):
        o = CellArrays(self.n)
        for k in self.a:
            o.a[k][:] = self.a[k]
        return o

    @classmethod
    def from_dict(cls, d):
        n = len(d["id"])
        o = cls(n)
        for name, t in CELL_FIELDS:
            o.a[name][:n] = np.asarray(d[name], dtype=t)
        return o

    def as_dict(self):
        return {k: self.a[k][:self.n].copy() for k in self.a}


class AgbError(RuntimeError):
    pass


NOALLOC_MAX_VOXELS = 4194304


def grid_diffuse_noalloc(value_ptr, nx, ny, nz, dx, diffusivity, dt, bc, face_value, stream=None, lib=None):
    """agb_grid_diffuse_noalloc on a caller-owned device buffer (an int pointer).
    Returns the status code; the library allocates nothing for it."""
    lib = lib or load()
    b = (C.c_int32 * 6)(*bc)
    f = (C.c_double * 6)(*face_value)
    return lib.agb_grid_diffuse_noalloc(C.c_void_p(int(value_ptr)), nx, ny, nz, dx, diffusivity, dt, b, f,
                                         None if stream is None else C.c_void_p(int(stream)))


def status_name(s):
    return STATUS_NAMES[s] if 0 <= s < len(STATUS_NAMES) else "Unknown(%d)" % s


_lib = None


def load(path=LIB_PATH):
    """Load libagb.so (built by __graft_entry__.build()); raises if missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise AgbError("libagb.so not built at %s; run __graft_entry__.build()" % path)
    lib = C.CDLL(path)
    P, I32, U64 = C.c_void_p, C.c_int32, C.c_uint64
    sigs = {
        "agb_world_desc_default": (None, [C.POINTER(WorldDesc)]),
        "agb_status_str": (C.c_char_p, [I32]),
        "agb_last_error": (C.c_char_p, [P]),
        "agb_device_info": (I32, [C.POINTER(I32), C.POINTER(I32), C.POINTER(I32)]),
        "agb_world_create": (I32, [C.POINTER(WorldDesc), C.POINTER(P)]),
        "agb_world_destroy": (None, [P]),
        "agb_world_spawn": (I32, [P, C.POINTER(Spawn), P]),
        "agb_world_spawn_seeded": (I32, [P, C.POINTER(Spawn), U64, P]),
        "agb_world_set_charge": (I32, [P, C.c_double, P]),
        "agb_world_set_boundary": (I32, [P, I32, C.POINTER(I32), C.POINTER(C.c_double)]),
        "agb_world_set_rates": (I32, [P, C.c_double, C.c_double]),
        "agb_world_set_overrides": (I32, [P, C.c_double, C.c_double]),
        "agb_world_mirror": (I32, [P, C.POINTER(Mirror), P]),
        "agb_world_import_cells": (I32, [P, C.POINTER(Cells), I32, U64, P]),
        "agb_world_export_cells": (I32, [P, C.POINTER(Cells), I32, C.POINTER(I32), C.POINTER(U64), P]),
        "agb_world_device_cells": (I32, [P, C.POINTER(Cells)]),
        "agb_world_step_host": (I32, [P, C.POINTER(Cells), I32, U64, I32, C.POINTER(Cells), I32, C.POINTER(I32),
                                      C.POINTER(U64), P]),
        "agb_world_count": (I32, [P, C.POINTER(I32), P]),
        "agb_world_import_field": (I32, [P, I32, P, P]),
        "agb_world_export_field": (I32, [P, I32, P, P]),
        "agb_world_export_deposit": (I32, [P, I32, P, P]),
        "agb_world_apply_brush": (I32, [P, I32, C.c_double, C.c_double, C.c_double, C.c_double, P]),
        "agb_world_set_flash": (I32, [P, I32, C.c_double]),
        "agb_world_spawn_taumoeba": (I32, [P, I32, U64, P]),
        "agb_world_import_taumoeba": (I32, [P, C.POINTER(Taumoeba), I32, U64, P]),
        "agb_world_export_taumoeba": (I32, [P, C.POINTER(Taumoeba), I32, C.POINTER(I32), C.POINTER(U64), P]),
        "agb_world_flash_audit": (I32, [P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "agb_world_step": (I32, [P, I32, P]),
        "agb_world_step_graph": (I32, [P, I32, P]),
        "agb_world_prepare_graphs": (I32, [P, I32, P]),
        "agb_world_set_timing": (I32, [P, I32]),
        "agb_world_section_times": (I32, [P, P]),
        "agb_world_stage": (I32, [P, I32, P]),
        "agb_world_graph_kernels": (I32, [P, C.POINTER(C.c_int64)]),
        "agb_world_set_walk": (I32, [P, I32, I32]),
        "agb_world_walk": (I32, [P, C.POINTER(I32), C.POINTER(I32)]),
        "agb_world_diffuse": (I32, [P, I32, C.c_double, P]),
        "agb_world_stats": (I32, [P, C.POINTER(Stats), P]),
        "agb_world_stats_accum": (I32, [P, P]),
        "agb_world_set_clock": (I32, [P, C.c_double, C.c_double]),
        "agb_world_set_light": (I32, [P, C.POINTER(Light)]),
        "agb_world_export_hash": (I32, [P, P, P, P, P, P, P]),
        "agb_world_export_forces": (I32, [P, P, P, P, P]),
        "agb_world_counters": (I32, [P, P, P]),
        "agb_grid_diffuse_noalloc": (I32, [P, I32, I32, I32, C.c_double, C.c_double, C.c_double,
                                           C.POINTER(I32), C.POINTER(C.c_double), P]),
        "agb_fnv1a64": (C.c_uint64, [P, C.c_uint64, C.c_uint64]),
        "agb_world_state_hash": (I32, [P, C.POINTER(C.c_uint64), P]),
        "agb_world_snapshot_save": (I32, [P, C.c_char_p, P, C.c_int64, C.POINTER(C.c_int64), P]),
        "agb_world_snapshot_load": (I32, [C.POINTER(WorldDesc), P, C.c_int64, C.POINTER(P)]),
        "agb_nn_conv3": (I32, [P, P, P, I32, I32, I32, I32, I32, I32, P, P, I32, P, P]),
        "agb_nn_wgrad_scratch_bytes": (C.c_int64, [I32, I32, I32, I32, I32]),
        "agb_nn_wgrad": (I32, [P, P, I32, I32, I32, I32, I32, P, P, P, C.c_int64, P, P]),
        "agb_nn_flip_weights": (I32, [P, P, I32, I32, P]),
        "agb_surrogate_desc_default": (None, [C.POINTER(SurrogateDesc)]),
        "agb_surrogate_create": (I32, [C.POINTER(SurrogateDesc), C.POINTER(P)]),
        "agb_surrogate_destroy": (None, [P]),
        "agb_surrogate_train": (I32, [P, I32, P, P]),
        "agb_surrogate_train_on": (I32, [P, P, P, P, P, P, P]),
        "agb_surrogate_advance": (I32, [P, P, P, P, P, I32, C.POINTER(SurrogateReport), P]),
        "agb_surrogate_reference": (I32, [P, P, P, P, P, P]),
        "agb_surrogate_window": (I32, [P, C.c_uint64, P, P, P, P, P]),
        "agb_surrogate_gradients": (I32, [P, P, P, P, P, P, P, P, C.c_int64, C.POINTER(C.c_float), P]),
        "agb_surrogate_params": (I32, [P, P, C.c_int64, C.POINTER(C.c_int64)]),
        "agb_surrogate_set_params": (I32, [P, P, C.c_int64]),
        "agb_surrogate_get_report": (I32, [P, C.POINTER(SurrogateReport)]),
        "agb_surrogate_error_word": (I32, [P, C.POINTER(C.c_uint32)]),
        "agb_world_attach_surrogate": (I32, [P, P, P]),
        "agb_batch_opts_default": (None, [C.POINTER(BatchOpts)]),
        "agb_batch_create": (I32, [P, P, I32, C.POINTER(BatchOpts), C.POINTER(P)]),
        "agb_batch_destroy": (None, [P]),
        "agb_batch_last_error": (C.c_char_p, [P]),
        "agb_batch_size": (I32, [P, C.POINTER(I32)]),
        "agb_batch_world": (I32, [P, I32, C.POINTER(P)]),
        "agb_batch_tuning": (I32, [P, I32, C.POINTER(Tuning)]),
        "agb_batch_step": (I32, [P, I32, P]),
        "agb_batch_graph_kernels": (I32, [P, C.POINTER(C.c_int64)]),
        "agb_batch_staged": (I32, [P, C.POINTER(I32)]),
        "agb_batch_stats": (I32, [P, P]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype, fn.argtypes = res, args
    _lib = lib
    return lib


def exported_symbols():
    """Names declared in include/agb.h, for the symbol-export test."""
    return ["agb_world_desc_default", "agb_status_str", "agb_last_error", "agb_device_info",
            "agb_world_create", "agb_world_destroy", "agb_world_spawn", "agb_world_spawn_seeded", "agb_world_set_charge",
            "agb_world_set_boundary", "agb_world_set_rates", "agb_world_set_overrides",
            "agb_world_mirror",
            "agb_world_import_cells",
            "agb_world_export_cells", "agb_world_device_cells", "agb_world_step_host", "agb_world_count",
            "agb_world_import_field", "agb_world_export_field", "agb_world_export_deposit",
            "agb_world_apply_brush", "agb_world_set_flash", "agb_world_flash_audit",
            "agb_world_spawn_taumoeba", "agb_world_import_taumoeba", "agb_world_export_taumoeba",
            "agb_world_step", "agb_world_step_graph", "agb_world_prepare_graphs", "agb_world_set_timing",
            "agb_world_section_times", "agb_world_graph_kernels", "agb_world_set_walk",
            "agb_world_walk", "agb_world_stage",
            "agb_world_diffuse",
            "agb_world_stats", "agb_world_stats_accum", "agb_world_set_clock",
            "agb_world_set_light", "agb_world_export_hash", "agb_world_export_forces",
            "agb_world_counters", "agb_grid_diffuse_noalloc",
            "agb_fnv1a64", "agb_world_state_hash", "agb_world_snapshot_save", "agb_world_snapshot_load",
            "agb_nn_conv3", "agb_nn_wgrad_scratch_bytes", "agb_nn_wgrad", "agb_nn_flip_weights",
            "agb_surrogate_desc_default", "agb_surrogate_create", "agb_surrogate_destroy", "agb_surrogate_train",
            "agb_surrogate_train_on",
            "agb_surrogate_advance", "agb_surrogate_reference", "agb_surrogate_window", "agb_surrogate_gradients",
            "agb_surrogate_params", "agb_surrogate_set_params", "agb_surrogate_get_report",
            "agb_surrogate_error_word", "agb_world_attach_surrogate",
            "agb_batch_opts_default", "agb_batch_create", "agb_batch_destroy", "agb_batch_last_error",
            "agb_batch_size", "agb_batch_world", "agb_batch_tuning", "agb_batch_step",
            "agb_batch_graph_kernels", "agb_batch_staged", "agb_batch_stats"]


def _st(stream):
    """A cudaStream_t given as an int handle (e.g. torch.cuda.Stream.cuda_stream) or None."""
    return None if stream is None else C.c_void_p(int(stream))


def field_shape(desc, f):
    g = desc.grid[f]
    return (g.nz, g.ny, g.nx)


class World:
    """One engine world (the reference's World) on the current CUDA device."""

    def __init__(self, desc, lib=None):
        self.lib = lib or load()
        self.desc = desc
        h = C.c_void_p()
        self._check(self.lib.agb_world_create(C.byref(desc), C.byref(h)), "agb_world_create")
        self.h = h

    def _check(self, rc, what):
        if rc != OK:
            detail = ""
            if getattr(self, "h", None):
                msg = self.lib.agb_last_error(self.h)
                detail = msg.decode() if msg else ""
            raise AgbError("%s failed: %s %s" % (what, status_name(rc), detail))

    def close(self):
        if getattr(self, "h", None):
            self.lib.agb_world_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def spawn(self, p, stream=None, seed=None):
        """cell_store_spawn: `seed` defaults to the world's seed."""
        if seed is None:
            self._check(self.lib.agb_world_spawn(self.h, C.byref(p), _st(stream)), "spawn")
        else:
            self._check(self.lib.agb_world_spawn_seeded(self.h, C.byref(p), seed, _st(stream)), "spawn")

    def set_charge(self, charge, stream=None):
        """cell_store_set_charge: every occupied slot's store to charge * CELL_ENERGY_MAX."""
        self._check(self.lib.agb_world_set_charge(self.h, float(charge), _st(stream)), "set_charge")

    def set_boundary(self, field, bc, face_value):
        """A field's six face kinds (BC_*) and face values, between ticks."""
        b = (C.c_int32 * 6)(*[int(v) for v in bc])
        f = (C.c_double * 6)(*[float(v) for v in face_value])
        self._check(self.lib.agb_world_set_boundary(self.h, field, b, f), "set_boundary")

    def mirror(self, stream=None):
        """agb_world_mirror as a dict: count, capacity, next id, counters,
        predator count and next id, and the cell store's device pointers."""
        m = Mirror()
        self._check(self.lib.agb_world_mirror(self.h, C.byref(m), _st(stream)), "mirror")
        out = {k: getattr(m, k) for k, _t in Mirror._fields_ if k != "cells"}
        out["count"], out["capacity"] = m.cells.count, m.cells.capacity
        out["pointers"] = [C.cast(getattr(m.cells, n), C.c_void_p).value for n, _t in CELL_FIELDS]
        return out

    def set_rates(self, physics_rate, biology_rate):
        """The clock rates as assigned to the World directly (unclamped)."""
        self._check(self.lib.agb_world_set_rates(self.h, float(physics_rate), float(biology_rate)), "set_rates")

    def set_overrides(self, co2_mass_per_division, max_emit_power):
        """World::co2_mass_per_division and World::petrova_max_power, between ticks."""
        self._check(self.lib.agb_world_set_overrides(self.h, float(co2_mass_per_division), float(max_emit_power)),
                    "set_overrides")

    def spawn_taumoeba(self, count, seed, stream=None):
        """taumoeba_spawn: `count` predators, streams from (splitmix64(seed), id)."""
        self._check(self.lib.agb_world_spawn_taumoeba(self.h, count, seed, _st(stream)), "spawn_taumoeba")

    def import_taumoeba(self, tau, next_id, stream=None):
        s = tau.struct()
        self._check(self.lib.agb_world_import_taumoeba(self.h, C.byref(s), tau.n, next_id, _st(stream)),
                    "import_taumoeba")

    def export_taumoeba(self, stream=None):
        """(TaumoebaArrays, next predator id)."""
        cnt, nid = C.c_int32(), C.c_uint64()
        empty = Taumoeba()
        self._check(self.lib.agb_world_export_taumoeba(self.h, C.byref(empty), 0, C.byref(cnt), C.byref(nid),
                                                       _st(stream)), "export_taumoeba")
        out = TaumoebaArrays(cnt.value)
        s = out.struct()
        self._check(self.lib.agb_world_export_taumoeba(self.h, C.byref(s), cnt.value, C.byref(cnt), C.byref(nid),
                                                       _st(stream)), "export_taumoeba")
        return out, nid.value

    def set_flash(self, active, power=0.0):
        """Arm (or disarm) the spin-drive flash; power <= 0 is the canon rate."""
        self._check(self.lib.agb_world_set_flash(self.h, int(bool(active)), power), "set_flash")

    def flash_audit(self):
        """(delivered impulse [N s], discharged store [J]) since creation."""
        i, e = C.c_double(), C.c_double()
        self._check(self.lib.agb_world_flash_audit(self.h, C.byref(i), C.byref(e)), "flash_audit")
        return i.value, e.value

    def set_light(self, light):
        """Replace the primary light source (dir, irradiance, ambient, enabled)."""
        self._check(self.lib.agb_world_set_light(self.h, C.byref(light)), "set_light")

    def import_cells(self, cells, next_id, stream=None):
        s = cells.struct()
        self._check(self.lib.agb_world_import_cells(self.h, C.byref(s), cells.n, next_id, _st(stream)),
                    "import_cells")

    def export_cells(self, stream=None, into=None):
        """Copy the population out; `into` reuses caller-owned (e.g. pinned)
        buffers in one call (their length bounds the copy; larger populations
        get fresh arrays)."""
        cnt, nid = C.c_int32(), C.c_uint64()
        if into is not None:
            cap = len(into.a["id"])
            s = into.struct()
            self._check(self.lib.agb_world_export_cells(self.h, C.byref(s), cap, C.byref(cnt), C.byref(nid),
                                                        _st(stream)), "export_cells")
            if cnt.value <= cap:
                into.n = cnt.value
                return into, nid.value
        n = self.count(stream)
        cells = CellArrays(n)
        s = cells.struct()
        self._check(self.lib.agb_world_export_cells(self.h, C.byref(s), n, C.byref(cnt), C.byref(nid),
                                                    _st(stream)), "export_cells")
        return cells, nid.value

    def step_host(self, cells_in, next_id, ticks=1, into=None, stream=None):
        """Import host cells, run `ticks` ticks, export into `into` (default:
        the input buffers): one engine call and one synchronisation."""
        out = into if into is not None else cells_in
        si, so = cells_in.struct(), out.struct()
        cnt, nid = C.c_int32(), C.c_uint64()
        self._check(self.lib.agb_world_step_host(self.h, C.byref(si), cells_in.n, next_id, ticks, C.byref(so),
                                                 len(out.a["id"]), C.byref(cnt), C.byref(nid), _st(stream)),
                    "step_host")
        if cnt.value > len(out.a["id"]):
            raise AgbError("step_host: population %d exceeds the output buffers" % cnt.value)
        out.n = cnt.value
        return out, nid.value

    def count(self, stream=None):
        c = C.c_int32()
        self._check(self.lib.agb_world_count(self.h, C.byref(c), _st(stream)), "count")
        return c.value

    def import_field(self, f, arr):
        a = np.ascontiguousarray(arr, dtype=np.float32)
        self._check(self.lib.agb_world_import_field(self.h, f, a.ctypes.data, None), "import_field")

    def export_field(self, f):
        out = np.zeros(field_shape(self.desc, f), dtype=np.float32)
        self._check(self.lib.agb_world_export_field(self.h, f, out.ctypes.data, None), "export_field")
        return out

    def export_deposit(self, f):
        out = np.zeros(field_shape(self.desc, f), dtype=np.uint64)
        self._check(self.lib.agb_world_export_deposit(self.h, f, out.ctypes.data, None), "export_deposit")
        return out

    def apply_brush(self, kind, x, y, radius, strength, stream=None):
        """world_apply_brush (src/sim/step.cu:80-89): a smooth disc of `strength`
        added to (chill: taken from) the brush kind's field between ticks."""
        self._check(self.lib.agb_world_apply_brush(self.h, kind, x, y, radius, strength, _st(stream)),
                    "apply_brush")

    def step(self, ticks=1, graph=False, stream=None):
        fn = self.lib.agb_world_step_graph if graph else self.lib.agb_world_step
        self._check(fn(self.h, ticks, _st(stream)), "step")

    def prepare_graphs(self, ticks=1, stream=None):
        """Capture every graph step(ticks, graph=True) will replay, without running
        them (agb_world_prepare_graphs); the world's state is unchanged."""
        self._check(self.lib.agb_world_prepare_graphs(self.h, ticks, _st(stream)), "prepare_graphs")

    SECTIONS = ("tick", "thermal", "t_diffuse", "irradiance", "slow_fields", "hash", "cell_pass", "integrate",
                "lifecycle")

    def set_timing(self, enable):
        """Section timers around the tick's parts, inside captured graphs too."""
        self._check(self.lib.agb_world_set_timing(self.h, int(bool(enable))), "set_timing")

    def section_times(self):
        """{section: milliseconds} of the last tick (sections that have not run: absent)."""
        out = np.zeros(len(self.SECTIONS), np.float32)
        self._check(self.lib.agb_world_section_times(self.h, out.ctypes.data), "section_times")
        return {k: float(v) for k, v in zip(self.SECTIONS, out) if v >= 0.0}

    def stage(self, s):
        self._check(self.lib.agb_world_stage(self.h, s, None), "stage %d" % s)

    def graph_kernels(self):
        k = C.c_int64()
        self._check(self.lib.agb_world_graph_kernels(self.h, C.byref(k)), "graph_kernels")
        return k.value

    def walk(self, lanes=None, fused=None):
        """(lanes per cell, fused) of the feeding/contact walks; sets whichever
        is given, keeping the other."""
        k, f = C.c_int32(), C.c_int32()
        self._check(self.lib.agb_world_walk(self.h, C.byref(k), C.byref(f)), "walk")
        if lanes is not None or fused is not None:
            lanes = k.value if lanes is None else int(lanes)
            fused = f.value if fused is None else int(bool(fused))
            self._check(self.lib.agb_world_set_walk(self.h, lanes, fused), "set_walk")
            self._check(self.lib.agb_world_walk(self.h, C.byref(k), C.byref(f)), "walk")
        return k.value, bool(f.value)

    def diffuse(self, f, dt, stream=None):
        self._check(self.lib.agb_world_diffuse(self.h, f, dt, _st(stream)), "diffuse")

    def stats(self):
        s = Stats()
        self._check(self.lib.agb_world_stats(self.h, C.byref(s), None), "stats")
        return s

    def stats_accum(self):
        out = np.zeros(12, dtype=np.uint64)
        self._check(self.lib.agb_world_stats_accum(self.h, out.ctypes.data), "stats_accum")
        return out

    def set_clock(self, physics, biology):
        self._check(self.lib.agb_world_set_clock(self.h, physics, biology), "set_clock")

    def export_hash(self):
        dims = np.zeros(4, dtype=np.int32)
        self._check(self.lib.agb_world_export_hash(self.h, dims.ctypes.data, None, None, None, None, None),
                    "export_hash")
        n = self.count()
        ks = np.zeros(max(n, 1), np.uint32)
        vs = np.zeros(max(n, 1), np.uint32)
        bs = np.zeros(int(dims[3]), np.int32)
        be = np.zeros(int(dims[3]), np.int32)
        self._check(self.lib.agb_world_export_hash(self.h, dims.ctypes.data, ks.ctypes.data, vs.ctypes.data,
                                                   bs.ctypes.data, be.ctypes.data, None), "export_hash")
        return dims, ks[:n], vs[:n], bs, be

    def export_forces(self):
        n = self.count()
        f = [np.zeros(max(n, 1), np.float32) for _ in range(3)]
        self._check(self.lib.agb_world_export_forces(self.h, f[0].ctypes.data, f[1].ctypes.data,
                                                     f[2].ctypes.data, None), "export_forces")
        return [a[:n] for a in f]

    def attach_surrogate(self, sg, stream=None):
        """Drive the temperature and CO2 grids by a Surrogate (None detaches)."""
        self._check(self.lib.agb_world_attach_surrogate(self.h, sg.h if sg is not None else None, _st(stream)),
                    "attach_surrogate")
        self._sg = sg

    def state_hash(self, stream=None):
        h = C.c_uint64()
        self._check(self.lib.agb_world_state_hash(self.h, C.byref(h), _st(stream)), "state_hash")
        return h.value

    def snapshot(self, scenario_id=b"test", stream=None):
        n = C.c_int64()
        self._check(self.lib.agb_world_snapshot_save(self.h, scenario_id, None, 0, C.byref(n), _st(stream)),
                    "snapshot size")
        buf = np.zeros(n.value, np.uint8)
        self._check(self.lib.agb_world_snapshot_save(self.h, scenario_id, buf.ctypes.data, n.value, C.byref(n),
                                                     _st(stream)), "snapshot")
        return buf.tobytes()

    def counters(self):
        out = np.zeros(4, dtype=np.int64)
        self._check(self.lib.agb_world_counters(self.h, out.ctypes.data, None), "counters")
        return out


SNAPSHOT_MAGIC = 0x48505341
FNV1A64_OFFSET = 1469598103934665603


def fnv1a64(data, h=FNV1A64_OFFSET, lib=None):
    """contracts/snapshot_v1.h fnv1a64 over a bytes-like object (engine implementation)."""
    lib = lib or load()
    buf = np.frombuffer(bytes(data), np.uint8)
    return int(lib.agb_fnv1a64(buf.ctypes.data if buf.size else None, buf.size, h))


def snapshot_load(base_desc, data, lib=None):
    """agb_world_snapshot_load: a World restored from snapshot bytes."""
    lib = lib or load()
    buf = np.frombuffer(bytes(data), np.uint8)
    h = C.c_void_p()
    rc = lib.agb_world_snapshot_load(C.byref(base_desc), buf.ctypes.data, buf.size, C.byref(h))
    if rc != OK:
        raise AgbError("agb_world_snapshot_load failed: %s" % status_name(rc))
    w = World.__new__(World)
    w.lib, w.desc, w.h = lib, base_desc, h
    return w


def snapshot_status(base_desc, data, lib=None):
    """Status code of agb_world_snapshot_load (the world, if any, is destroyed)."""
    lib = lib or load()
    buf = np.frombuffer(bytes(data), np.uint8)
    h = C.c_void_p()
    rc = lib.agb_world_snapshot_load(C.byref(base_desc), buf.ctypes.data, buf.size, C.byref(h))
    if rc == OK:
        lib.agb_world_destroy(h)
    return rc


class SurrogateDesc(C.Structure):
    _fields_ = [("abi_version", C.c_uint32), ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("extent", C.c_double), ("dt", C.c_double), ("steps", C.c_int32), ("judge_every", C.c_int32),
                ("tol_temperature", C.c_double), ("tol_energy", C.c_double), ("diffusivity", C.c_double * 2),
                ("init", C.c_double * 2), ("bc", (C.c_int32 * 6) * 2), ("face", (C.c_double * 6) * 2),
                ("seed", C.c_uint64), ("learning_rate", C.c_float),
                ("train_temperature_amplitude", C.c_double), ("train_source_density", C.c_double),
                ("train_heat_per_step", C.c_double), ("train_uptake_per_step", C.c_double)]

    def as_dict(self):
        return {"init": [self.init[0], self.init[1]], "steps": self.steps, "nx": self.nx, "extent": self.extent,
                "dt": self.dt, "diffusivity": [self.diffusivity[0], self.diffusivity[1]],
                "bc": [list(self.bc[0]), list(self.bc[1])], "face": [list(self.face[0]), list(self.face[1])],
                "train_temperature_amplitude": self.train_temperature_amplitude,
                "train_heat_per_step": self.train_heat_per_step,
                "train_uptake_per_step": self.train_uptake_per_step}


class SurrogateReport(C.Structure):
    _fields_ = [("calls", C.c_int64), ("judged", C.c_int64), ("fallbacks", C.c_int64),
                ("last_err_temperature", C.c_double), ("last_err_co2", C.c_double),
                ("last_energy_drift", C.c_double), ("last_used_surrogate", C.c_int32), ("last_loss", C.c_float)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def surrogate_desc(lib=None, **kw):
    lib = lib or load()
    d = SurrogateDesc()
    lib.agb_surrogate_desc_default(C.byref(d))
    for k, v in kw.items():
        setattr(d, k, v)
    return d


class Surrogate:
    """The learned field surrogate; field arguments are device pointers (ints)."""

    def __init__(self, desc=None, lib=None):
        self.lib = lib or load()
        self.desc = desc if desc is not None else surrogate_desc(self.lib)
        h = C.c_void_p()
        rc = self.lib.agb_surrogate_create(C.byref(self.desc), C.byref(h))
        if rc != OK:
            raise AgbError("agb_surrogate_create failed: %s" % status_name(rc))
        self.h = h

    def _ck(self, rc, what):
        if rc != OK:
            raise AgbError("%s failed: %s" % (what, status_name(rc)))

    def close(self):
        if getattr(self, "h", None):
            self.lib.agb_surrogate_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _p(x):
        return None if x is None else C.c_void_p(int(x))

    def train(self, windows, stream=None):
        losses = np.zeros(max(windows, 1), np.float32)
        self._ck(self.lib.agb_surrogate_train(self.h, windows, losses.ctypes.data, _st(stream)), "train")
        return losses[:windows]

    def train_on(self, T, Cf, qT, qC, stream=None):
        """One training step on a caller-supplied window (device pointers); returns its loss."""
        loss = C.c_float()
        self._ck(self.lib.agb_surrogate_train_on(self.h, self._p(T), self._p(Cf), self._p(qT), self._p(qC),
                                                 C.byref(loss), _st(stream)), "train_on")
        return loss.value

    def advance(self, T, Cf, qT, qC, judge=0, stream=None):
        rep = SurrogateReport()
        self._ck(self.lib.agb_surrogate_advance(self.h, self._p(T), self._p(Cf), self._p(qT), self._p(qC), judge,
                                                C.byref(rep), _st(stream)), "advance")
        return rep

    def reference(self, T, Cf, qT, qC, stream=None):
        self._ck(self.lib.agb_surrogate_reference(self.h, self._p(T), self._p(Cf), self._p(qT), self._p(qC),
                                                  _st(stream)), "reference")

    def window(self, index, T, Cf, qT, qC, stream=None):
        self._ck(self.lib.agb_surrogate_window(self.h, index, self._p(T), self._p(Cf), self._p(qT), self._p(qC),
                                               _st(stream)), "window")

    def params(self):
        n = C.c_int64()
        self._ck(self.lib.agb_surrogate_params(self.h, None, 0, C.byref(n)), "params")
        out = np.zeros(n.value, np.float32)
        self._ck(self.lib.agb_surrogate_params(self.h, out.ctypes.data, n.value, C.byref(n)), "params")
        return out

    def set_params(self, flat):
        a = np.ascontiguousarray(flat, np.float32)
        self._ck(self.lib.agb_surrogate_set_params(self.h, a.ctypes.data, a.size), "set_params")

    def gradients(self, T0, C0, qT, qC, T1, C1, stream=None):
        n = self.params().size
        g = np.zeros(n, np.float32)
        loss = C.c_float()
        self._ck(self.lib.agb_surrogate_gradients(self.h, self._p(T0), self._p(C0), self._p(qT), self._p(qC),
                                                  self._p(T1), self._p(C1), g.ctypes.data, n, C.byref(loss),
                                                  _st(stream)), "gradients")
        return float(loss.value), g

    def report(self):
        rep = SurrogateReport()
        self._ck(self.lib.agb_surrogate_get_report(self.h, C.byref(rep)), "report")
        return rep

    def error_word(self):
        w = C.c_uint32()
        self._ck(self.lib.agb_surrogate_error_word(self.h, C.byref(w)), "error_word")
        return w.value


class _ChamberView(World):
    """A chamber of a Batch: the World interface over a handle the batch owns."""

    def __init__(self, handle, desc, lib, owner):
        self.lib, self.desc, self.h, self._owner = lib, desc, handle, owner

    def close(self):
        self.h = None


def batch_opts(autotune=False, lanes=0, hash_candidates=(), probe_ticks=4, staged=True, lib=None):
    lib = lib or load()
    o = BatchOpts()
    lib.agb_batch_opts_default(C.byref(o))
    o.autotune = 1 if autotune else 0
    o.lanes = lanes
    o.staged = 1 if staged else 0
    o.n_hash_candidates = len(hash_candidates)
    for k, h in enumerate(hash_candidates[:8]):
        o.hash_candidates[k] = h
    o.probe_ticks = probe_ticks
    return o


class Batch:
    """Independent chambers advanced together, one graph launch per step()."""

    def __init__(self, descs, spawns, opts=None, lib=None):
        self.lib = lib or load()
        n = len(descs)
        self.descs = (WorldDesc * n)(*descs)
        self.spawns = (Spawn * n)(*spawns) if spawns is not None else None
        o = opts if opts is not None else batch_opts(lib=self.lib)
        h = C.c_void_p()
        rc = self.lib.agb_batch_create(C.cast(self.descs, C.c_void_p),
                                       C.cast(self.spawns, C.c_void_p) if self.spawns is not None else None,
                                       n, C.byref(o), C.byref(h))
        if rc != OK:
            raise AgbError("agb_batch_create failed: %s" % status_name(rc))
        self.h = h
        self.n = n
        self.chambers = []
        for i in range(n):
            wh = C.c_void_p()
            self._check(self.lib.agb_batch_world(self.h, i, C.byref(wh)), "agb_batch_world")
            self.chambers.append(_ChamberView(wh, self.descs[i], self.lib, self))

    def _check(self, rc, what):
        if rc != OK:
            msg = self.lib.agb_batch_last_error(self.h) if getattr(self, "h", None) else b""
            raise AgbError("%s failed: %s %s" % (what, status_name(rc), (msg or b"").decode()))

    def close(self):
        if getattr(self, "h", None):
            for c in self.chambers:
                c.h = None
            self.lib.agb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, ticks=1, stream=None):
        self._check(self.lib.agb_batch_step(self.h, ticks, _st(stream)), "agb_batch_step")

    def tuning(self, i):
        t = Tuning()
        self._check(self.lib.agb_batch_tuning(self.h, i, C.byref(t)), "agb_batch_tuning")
        return t

    def graph_kernels(self):
        k = C.c_int64()
        self._check(self.lib.agb_batch_graph_kernels(self.h, C.byref(k)), "agb_batch_graph_kernels")
        return k.value

    def staged(self):
        """True when steps run one launch per stage over every chamber."""
        k = C.c_int32()
        self._check(self.lib.agb_batch_staged(self.h, C.byref(k)), "agb_batch_staged")
        return bool(k.value)

    def stats(self):
        out = (Stats * self.n)()
        self._check(self.lib.agb_batch_stats(self.h, C.cast(out, C.c_void_p)), "agb_batch_stats")
        return list(out)
