"""Test-side bindings: the engine's Python mirror (agb.py), the C oracle
(oracle/liborc.so) and, where the reference sources are present, the
reference itself run on the CPU (oracle/_ref/libastro_ref.so).

Only tests, smoke() and bench.py's CPU baseline leg load the oracle."""
import ctypes as C
import importlib.util
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "astrophage-microscope_gb300")
ORACLE_SO = os.path.join(ROOT, "oracle", "liborc.so")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libastro_ref.so")
GOLDEN = os.path.join(ROOT, "tests", "golden")


def _load(name):
    """A module of the package, registered so that its own imports (scenario.py
    imports agb) resolve to the same module objects."""
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, os.path.join(PKG, name + ".py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def load_agb():
    return _load("agb")


agb = load_agb()


def load_scenario():
    return _load("scenario")


def load_workloads():
    return _load("workloads")


def load_surrogate_data():
    load_workloads()
    return _load("surrogate_data")


def build_oracle():
    src = os.path.join(ROOT, "oracle", "oracle.c")
    if (not os.path.exists(ORACLE_SO)) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                               "-fopenmp", "-o", ORACLE_SO, src, "-lm"])
    return ORACLE_SO


_orc = None


def oracle_lib():
    global _orc
    if _orc is None:
        lib = C.CDLL(build_oracle())
        P, I32, U64 = C.c_void_p, C.c_int32, C.c_uint64
        sigs = {
            "orc_world_create": (I32, [C.POINTER(agb.WorldDesc), C.POINTER(P)]),
            "orc_world_destroy": (None, [P]),
            "orc_set_threads": (None, [C.c_int]),
            "orc_world_spawn": (I32, [P, C.POINTER(agb.Spawn)]),
            "orc_world_spawn_seeded": (I32, [P, C.POINTER(agb.Spawn), U64]),
            "orc_world_set_light": (I32, [P, C.POINTER(agb.Light)]),
            "orc_world_set_flash": (I32, [P, I32, C.c_double]),
            "orc_world_spawn_taumoeba": (I32, [P, I32, U64]),
            "orc_world_import_taumoeba": (I32, [P, C.POINTER(agb.Taumoeba), I32, U64]),
            "orc_world_export_taumoeba": (I32, [P, C.POINTER(agb.Taumoeba), I32, C.POINTER(I32), C.POINTER(U64)]),
            "orc_world_flash_audit": (I32, [P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
            "orc_world_import_cells": (I32, [P, C.POINTER(agb.Cells), I32, U64]),
            "orc_world_export_cells": (I32, [P, C.POINTER(agb.Cells), I32, C.POINTER(I32), C.POINTER(U64)]),
            "orc_world_import_field": (I32, [P, I32, P]),
            "orc_world_export_field": (I32, [P, I32, P]),
            "orc_world_export_deposit": (I32, [P, I32, P]),
            "orc_world_apply_brush": (I32, [P, I32, C.c_double, C.c_double, C.c_double, C.c_double]),
            "orc_world_step": (I32, [P, I32]),
            "orc_world_stage": (I32, [P, I32]),
            "orc_world_diffuse": (I32, [P, I32, C.c_double]),
            "orc_world_stats": (I32, [P, C.POINTER(agb.Stats)]),
            "orc_world_stats_accum": (I32, [P, P]),
            "orc_world_set_clock": (I32, [P, C.c_double, C.c_double]),
            "orc_world_export_hash": (I32, [P, P, P, P, P, P]),
            "orc_world_export_forces": (I32, [P, P, P, P]),
            "orc_world_export_term_scales": (I32, [P, P, P, P]),
            "orc_world_counters": (I32, [P, P]),
            "orc_pcg32_seed_draws": (None, [U64, U64, I32, P]),
            "orc_cell_rng_init": (U64, [U64, U64]),
            "orc_pcg_split": (U64, [U64, U64]),
            "orc_fnv1a64": (U64, [P, U64, U64]),
            "orc_world_snapshot": (C.c_int64, [P, C.c_char_p, P, C.c_int64]),
        }
        for name, (res, args) in sigs.items():
            fn = getattr(lib, name)
            fn.restype, fn.argtypes = res, args
        _orc = lib
    return _orc


class OracleWorld:
    """The C oracle behind the same method names as agb.World."""

    def __init__(self, desc, threads=1):
        self.lib = oracle_lib()
        self.lib.orc_set_threads(threads)
        self.desc = desc
        h = C.c_void_p()
        rc = self.lib.orc_world_create(C.byref(desc), C.byref(h))
        if rc:
            raise agb.AgbError("orc_world_create: %s" % agb.status_name(rc))
        self.h = h
        self._n = 0

    def _ck(self, rc, what):
        if rc:
            raise agb.AgbError("%s: %s" % (what, agb.status_name(rc)))

    def close(self):
        if self.h:
            self.lib.orc_world_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def spawn(self, p, seed=None):
        if seed is None:
            self._ck(self.lib.orc_world_spawn(self.h, C.byref(p)), "spawn")
        else:
            self._ck(self.lib.orc_world_spawn_seeded(self.h, C.byref(p), seed), "spawn")

    def set_light(self, light):
        self._ck(self.lib.orc_world_set_light(self.h, C.byref(light)), "set_light")

    def set_flash(self, active, power=0.0):
        self._ck(self.lib.orc_world_set_flash(self.h, int(bool(active)), power), "set_flash")

    def spawn_taumoeba(self, count, seed):
        self._ck(self.lib.orc_world_spawn_taumoeba(self.h, count, seed), "spawn_taumoeba")

    def import_taumoeba(self, tau, next_id):
        s = tau.struct()
        self._ck(self.lib.orc_world_import_taumoeba(self.h, C.byref(s), tau.n, next_id), "import_taumoeba")

    def export_taumoeba(self):
        cnt, nid = C.c_int32(), C.c_uint64()
        empty = agb.Taumoeba()
        self.lib.orc_world_export_taumoeba(self.h, C.byref(empty), 0, C.byref(cnt), C.byref(nid))
        out = agb.TaumoebaArrays(cnt.value)
        s = out.struct()
        self.lib.orc_world_export_taumoeba(self.h, C.byref(s), cnt.value, C.byref(cnt), C.byref(nid))
        return out, nid.value

    def flash_audit(self):
        i, e = C.c_double(), C.c_double()
        self._ck(self.lib.orc_world_flash_audit(self.h, C.byref(i), C.byref(e)), "flash_audit")
        return i.value, e.value

    def import_cells(self, cells, next_id):
        s = cells.struct()
        self._ck(self.lib.orc_world_import_cells(self.h, C.byref(s), cells.n, next_id), "import")

    def count(self):
        cnt, nid = C.c_int32(), C.c_uint64()
        empty = agb.Cells()
        self.lib.orc_world_export_cells(self.h, C.byref(empty), 0, C.byref(cnt), C.byref(nid))
        return cnt.value

    def export_cells(self):
        n = self.count()
        cells = agb.CellArrays(n)
        s = cells.struct()
        cnt, nid = C.c_int32(), C.c_uint64()
        self._ck(self.lib.orc_world_export_cells(self.h, C.byref(s), n, C.byref(cnt), C.byref(nid)), "export")
        return cells, nid.value

    def import_field(self, f, arr):
        a = np.ascontiguousarray(arr, dtype=np.float32)
        self._ck(self.lib.orc_world_import_field(self.h, f, a.ctypes.data), "import_field")

    def export_field(self, f):
        out = np.zeros(agb.field_shape(self.desc, f), dtype=np.float32)
        self._ck(self.lib.orc_world_export_field(self.h, f, out.ctypes.data), "export_field")
        return out

    def export_deposit(self, f):
        out = np.zeros(agb.field_shape(self.desc, f), dtype=np.uint64)
        self._ck(self.lib.orc_world_export_deposit(self.h, f, out.ctypes.data), "export_deposit")
        return out

    def apply_brush(self, kind, x, y, radius, strength):
        self._ck(self.lib.orc_world_apply_brush(self.h, kind, x, y, radius, strength), "apply_brush")

    def step(self, ticks=1, graph=False):
        self._ck(self.lib.orc_world_step(self.h, ticks), "step")

    def stage(self, s):
        self._ck(self.lib.orc_world_stage(self.h, s), "stage")

    def diffuse(self, f, dt):
        self._ck(self.lib.orc_world_diffuse(self.h, f, dt), "diffuse")

    def stats(self):
        s = agb.Stats()
        self._ck(self.lib.orc_world_stats(self.h, C.byref(s)), "stats")
        return s

    def stats_accum(self):
        out = np.zeros(12, dtype=np.uint64)
        self.lib.orc_world_stats_accum(self.h, out.ctypes.data)
        return out

    def set_clock(self, p, b):
        self.lib.orc_world_set_clock(self.h, p, b)

    def export_hash(self):
        dims = np.zeros(4, dtype=np.int32)
        self.lib.orc_world_export_hash(self.h, dims.ctypes.data, None, None, None, None)
        n = self.count()
        ks, vs = np.zeros(max(n, 1), np.uint32), np.zeros(max(n, 1), np.uint32)
        bs, be = np.zeros(int(dims[3]), np.int32), np.zeros(int(dims[3]), np.int32)
        self.lib.orc_world_export_hash(self.h, dims.ctypes.data, ks.ctypes.data, vs.ctypes.data,
                                       bs.ctypes.data, be.ctypes.data)
        return dims, ks[:n], vs[:n], bs, be

    def export_forces(self):
        n = self.count()
        f = [np.zeros(max(n, 1), np.float64) for _ in range(3)]
        self.lib.orc_world_export_forces(self.h, f[0].ctypes.data, f[1].ctypes.data, f[2].ctypes.data)
        return [a[:n] for a in f]

    def export_term_scales(self):
        """Per cell, from the last motion stage: (force, velocity, displacement)
        summed term magnitudes, the floors of the parity bounds (parity.py)."""
        n = self.count()
        s = [np.zeros(max(n, 1), np.float64) for _ in range(3)]
        self.lib.orc_world_export_term_scales(self.h, s[0].ctypes.data, s[1].ctypes.data, s[2].ctypes.data)
        return [a[:n] for a in s]

    def counters(self):
        out = np.zeros(4, dtype=np.int64)
        self.lib.orc_world_counters(self.h, out.ctypes.data)
        return out

    def snapshot(self, scenario_id=b"test"):
        n = self.lib.orc_world_snapshot(self.h, scenario_id, None, 0)
        buf = np.zeros(n, np.uint8)
        self.lib.orc_world_snapshot(self.h, scenario_id, buf.ctypes.data, n)
        return buf.tobytes()


# ---------------------------------------------------------------------------
# The reference itself on the CPU (only where oracle/_ref was built from the
# reference's sources; absent on machines without them).
# ---------------------------------------------------------------------------
class RefParams(C.Structure):
    _fields_ = [("chamber_w", C.c_double), ("chamber_h", C.c_double), ("chamber_d", C.c_double),
                ("capacity", C.c_int32), ("seed", C.c_uint64),
                ("boundary_x", C.c_uint8), ("boundary_y", C.c_uint8), ("gravity_axis", C.c_uint8),
                ("thermal_noise", C.c_uint8), ("contact_enabled", C.c_uint8),
                ("adhesion_enabled", C.c_uint8), ("thermal_enabled", C.c_uint8),
                ("emission_enabled", C.c_uint8), ("taxis_enabled", C.c_uint8),
                ("occlusion_exact", C.c_uint8), ("store_disposition", C.c_uint8),
                ("compaction_enabled", C.c_uint8), ("ambient_temp", C.c_double), ("co2_init", C.c_double),
                ("n_temp", C.c_int32), ("n_co2", C.c_int32), ("n_n2", C.c_int32), ("n_irr", C.c_int32),
                ("bc_temp", C.c_int32), ("bc_co2", C.c_int32),
                ("light_dir_x", C.c_float), ("light_dir_y", C.c_float), ("light_irradiance", C.c_float),
                ("ambient_irradiance", C.c_float), ("light_enabled", C.c_uint8),
                ("physics_rate", C.c_double), ("biology_rate", C.c_double),
                ("co2_mass_per_division", C.c_double), ("tau_capacity", C.c_int32), ("tau_compaction", C.c_uint8)]


class RefSpawn(C.Structure):
    _fields_ = [("count", C.c_int32), ("placement", C.c_int32), ("charge_dist", C.c_int32),
                ("awake", C.c_int32), ("place_x", C.c_double), ("place_y", C.c_double),
                ("place_radius", C.c_double), ("charge_a", C.c_double), ("charge_b", C.c_double)]


def ref_available():
    return os.path.exists(REF_SO)


_ref = None


def ref_lib():
    """The reference built for the CPU (oracle/_ref/libastro_ref.so), loaded once."""
    global _ref
    if _ref is None:
        lib = C.CDLL(REF_SO)
        lib.ref_world_create.restype = C.c_void_p
        lib.ref_world_create.argtypes = [C.POINTER(RefParams)]
        for name in ("ref_world_destroy", "ref_spawn", "ref_count", "ref_next_id", "ref_cells_io",
                     "ref_field_n", "ref_field_io", "ref_field_deposit", "ref_step", "ref_stage",
                     "ref_hash_io", "ref_forces", "ref_stats", "ref_stats_accum", "ref_counters",
                     "ref_grid_diffuse", "ref_grid_substep", "ref_grid_substeps"):
            getattr(lib, name).argtypes = None
        lib.ref_next_id.restype = C.c_uint64
        lib.ref_grid_diffuse.argtypes = [C.c_void_p, C.c_int, C.c_double]
        lib.ref_apply_brush.argtypes = [C.c_void_p, C.c_int] + [C.c_double] * 4
        lib.ref_grid_substeps.argtypes = [C.c_void_p, C.c_int, C.c_double]
        lib.ref_cells_io.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_void_p), C.c_int32, C.c_uint64]
        lib.ref_snapshot.restype = C.c_int64
        lib.ref_snapshot.argtypes = [C.c_void_p, C.c_char_p, C.c_void_p, C.c_int64]
        lib.ref_state_hash.restype = C.c_uint64
        lib.ref_state_hash.argtypes = [C.c_void_p]
        lib.ref_set_flash.argtypes = [C.c_void_p, C.c_int, C.c_double]
        lib.ref_tau_spawn.argtypes = [C.c_void_p, C.c_int32, C.c_uint64]
        lib.ref_tau_count.argtypes = [C.c_void_p]
        lib.ref_tau_next_id.argtypes = [C.c_void_p]
        lib.ref_tau_next_id.restype = C.c_uint64
        lib.ref_tau_io.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_void_p), C.c_int32, C.c_uint64]
        lib.ref_flash_audit.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        lib.ref_scenario_run.restype = C.c_void_p
        lib.ref_scenario_run.argtypes = [C.c_char_p, C.c_int64, C.c_void_p, C.POINTER(C.c_int32)]
        _ref = lib
    return _ref


class RefWorld:
    """The reference's own World (src/sim/world.cuh) run on the CPU, driven from
    an agb.WorldDesc restricted to what the reference can express (nz = 1, one
    BC per field, in-plane light)."""

    def __init__(self, desc):
        lib = ref_lib()
        self.lib = lib
        self.desc = desc
        g = desc.grid
        for f in range(4):
            if g[f].nz != 1 or g[f].nx != g[f].ny:
                raise ValueError("reference grids are square and depth-averaged")
        L = desc.light
        p = RefParams(desc.chamber_w, desc.chamber_h, desc.chamber_d, desc.capacity, desc.seed,
                      desc.boundary_x, desc.boundary_y, desc.gravity_axis, desc.thermal_noise,
                      desc.contact_enabled, desc.adhesion_enabled, desc.thermal_enabled,
                      desc.emission_enabled, desc.taxis_enabled, desc.occlusion_exact,
                      desc.store_disposition, desc.compaction_enabled, desc.ambient_temp,
                      g[1].init, g[0].nx, g[1].nx, g[2].nx, g[3].nx, g[0].bc[0], g[1].bc[0],
                      L.dir_x, L.dir_y, L.irradiance, L.ambient, L.enabled,
                      desc.physics_rate, desc.biology_rate, desc.co2_mass_per_division, desc.tau_capacity,
                      desc.tau_compaction_enabled)
        self.h = C.c_void_p(lib.ref_world_create(C.byref(p)))
        if not self.h:
            raise RuntimeError("ref_world_create failed")

    def spawn_taumoeba(self, count, seed):
        assert self.lib.ref_tau_spawn(self.h, count, seed) == 0

    def export_taumoeba(self):
        n = self.lib.ref_tau_count(self.h)
        out = agb.TaumoebaArrays(n)
        ptrs = (C.c_void_p * 20)(*[out.a[name].ctypes.data for name, _t in agb.TAU_FIELDS])
        assert self.lib.ref_tau_io(self.h, 0, ptrs, n, 0) == 0
        return out, int(self.lib.ref_tau_next_id(self.h))

    def import_taumoeba(self, tau, next_id):
        ptrs = (C.c_void_p * 20)(*[tau.a[name].ctypes.data for name, _t in agb.TAU_FIELDS])
        assert self.lib.ref_tau_io(self.h, 1, ptrs, tau.n, next_id) == 0

    @classmethod
    def from_scenario(cls, text, ticks, desc):
        """ref_scenario_run: the reference's scenario loader, driver and accept
        evaluation over `ticks` ticks. Returns (world, measured values); `desc` is
        the agb.WorldDesc the scenario builds (for field shapes)."""
        lib = ref_lib()
        out = np.zeros(16, np.float64)
        n = C.c_int32(0)
        h = lib.ref_scenario_run(text.encode() if isinstance(text, str) else text, ticks,
                                 out.ctypes.data, C.byref(n))
        if not h:
            raise RuntimeError("ref_scenario_run failed")
        w = cls.__new__(cls)
        w.lib, w.desc, w.h = lib, desc, C.c_void_p(h)
        return w, list(out[:n.value])

    def close(self):
        if self.h:
            self.lib.ref_world_destroy(self.h)
            self.h = None

    def spawn(self, p):
        s = RefSpawn(p.count, p.placement, p.charge_dist, p.awake, p.place_x, p.place_y,
                     p.place_radius, p.charge_a, p.charge_b)
        assert self.lib.ref_spawn(self.h, C.byref(s)) == 0

    def count(self):
        return self.lib.ref_count(self.h)

    def _io(self, cells, direction, next_id=0):
        ptrs = (C.c_void_p * 25)(*[cells.a[name].ctypes.data for name, _ in agb.CELL_FIELDS])
        assert self.lib.ref_cells_io(self.h, direction, ptrs, cells.n, next_id) == 0

    def export_cells(self):
        cells = agb.CellArrays(self.count())
        self._io(cells, 0)
        return cells, self.lib.ref_next_id(self.h)

    def import_cells(self, cells, next_id):
        self._io(cells, 1, next_id)

    def export_field(self, f):
        n = self.lib.ref_field_n(self.h, f)
        out = np.zeros((1, n, n), np.float32)
        self.lib.ref_field_io(self.h, f, 0, out.ctypes.data_as(C.c_void_p))
        return out

    def import_field(self, f, arr):
        a = np.ascontiguousarray(arr, dtype=np.float32)
        self.lib.ref_field_io(self.h, f, 1, a.ctypes.data_as(C.c_void_p))

    def apply_brush(self, kind, x, y, radius, strength):
        assert self.lib.ref_apply_brush(self.h, kind, x, y, radius, strength) == 0

    def export_deposit(self, f):
        n = self.lib.ref_field_n(self.h, f)
        out = np.zeros((1, n, n), np.uint64)
        self.lib.ref_field_deposit(self.h, f, out.ctypes.data_as(C.c_void_p))
        return out

    def step(self, ticks=1, graph=False):
        self.lib.ref_step(self.h, ticks)

    def stage(self, s):
        assert self.lib.ref_stage(self.h, s) == 0

    def diffuse(self, f, dt):
        assert self.lib.ref_grid_diffuse(self.h, f, dt) == 0

    def export_hash(self):
        dims = np.zeros(4, np.int32)
        self.lib.ref_hash_io(self.h, dims.ctypes.data_as(C.c_void_p), None, None, None, None)
        n = self.count()
        ks, vs = np.zeros(max(n, 1), np.uint32), np.zeros(max(n, 1), np.uint32)
        bs, be = np.zeros(int(dims[3]), np.int32), np.zeros(int(dims[3]), np.int32)
        self.lib.ref_hash_io(self.h, dims.ctypes.data_as(C.c_void_p), ks.ctypes.data_as(C.c_void_p),
                             vs.ctypes.data_as(C.c_void_p), bs.ctypes.data_as(C.c_void_p),
                             be.ctypes.data_as(C.c_void_p))
        return dims, ks[:n], vs[:n], bs, be

    def export_forces(self):
        n = self.count()
        f = [np.zeros(max(n, 1), np.float64) for _ in range(3)]
        self.lib.ref_forces(self.h, *[a.ctypes.data_as(C.c_void_p) for a in f])
        return [a[:n] for a in f]

    def stats(self):
        out = np.zeros(24, np.float64)
        self.lib.ref_stats(self.h, out.ctypes.data_as(C.c_void_p))
        names = ["tick", "sim_time_s", "n_live", "n_dead", "n_dormant", "n_awake", "n_taumoeba",
                 "mean_charge", "total_energy_j", "mean_temp_cell_k", "mean_temp_medium_k",
                 "max_temp_medium_k", "co2_total_kg", "n2_total_kg", "mean_tau_tolerance",
                 "divisions_this_window", "deaths_this_window", "boil_events",
                 "ignitions_this_window", "physics_rate", "biology_rate", "non_canon_run"]
        return dict(zip(names, out.tolist()))

    def stats_accum(self):
        out = np.zeros(12, np.uint64)
        self.lib.ref_stats_accum(self.h, out.ctypes.data_as(C.c_void_p))
        return out

    def counters(self):
        out = np.zeros(3, np.int64)
        self.lib.ref_counters(self.h, out.ctypes.data_as(C.c_void_p))
        return out

    def snapshot(self, scenario_id=b"test"):
        n = self.lib.ref_snapshot(self.h, scenario_id, None, 0)
        buf = np.zeros(n, np.uint8)
        assert self.lib.ref_snapshot(self.h, scenario_id, buf.ctypes.data, n) == n
        return buf.tobytes()

    def state_hash(self):
        return int(self.lib.ref_state_hash(self.h))
