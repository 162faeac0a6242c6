"""Comparison helpers for engine-vs-oracle parity.

Integer state (ids, flags, death causes, PCG32 states, hash keys, sorted
order, bucket ranges, slot assignment, compaction survivors, the exact-zero
irradiance set) must match exactly.

Floating-point state is held to RTOL = 1e-5 relative, the bound the engine
is specified to (FP32 arithmetic committed into the contract's FP64 state).
A relative bound needs a scale where a value can sit at or near zero, and
each floor below is the scale that the value's own arithmetic works at:

  x, y, z        1e-5 of the coordinate, floored at one cell radius (a
                 coordinate has no natural zero; 1e-5 of 5 um is 50 pm).
                 With the oracle's term scales: also 1e-5 of the largest
                 summed term of that step's displacement (drift, velocity
                 relaxation and the Brownian kick), i.e. the displacement
                 itself must agree to 1e-5 of its own size.
  vx, vy, vz     1e-5 of the value, floored at 1e-5 of the summed magnitude
                 of the terms of that step's velocity update (decayed
                 velocity, force/drag, the two noise terms). A velocity is
                 the sum of these; near zero they cancel.
  forces         1e-5 of the value, floored at 1e-5 of the cell's force
                 scale: (cell mass + displaced water mass) g + |recoil| +
                 k * 2a per contact (a contact's force at full overlap).
                 The buoyant weight is a difference of the first two, and
                 contact sums cancel.
  irradiance     1e-5 of the value, floored at 1e-5 of the light source's
                 irradiance (a shading product is formed relative to the
                 unshaded value, at most the source).
  fields         1e-5 of the value (irradiance field: floored as above).
  everything else (energy, CO2 held, biomass, temperatures, samples, age,
  run-and-tumble state) 1e-5 of the value, no floor.

The term scales come from the oracle (orc_world_export_term_scales): per cell,
from the motion stage of the tick being compared.
"""
import numpy as np

from helpers import agb

RTOL = 1e-5
INT_FIELDS = ("id", "flags", "death_cause", "rng_state")
POS_FIELDS = ("x", "y", "z")
VEL_FIELDS = ("vx", "vy", "vz")
# Displacements agree to far better than a position's 1e-5; the absolute floor
# covers the FP64 rounding of the committed coordinate (|x| <= a few mm).
POS_ABS_FLOOR = 1e-18


def copy_state(src, dst, fields=True):
    cells, nid = src.export_cells()
    dst.import_cells(cells, nid)
    if fields:
        for f in range(4):
            if src.desc.grid[f].nx > 0:
                dst.import_field(f, src.export_field(f))
    return cells


def _excess(a, b, tol):
    """(number of elements beyond tol, worst |a - b| / tol) for float arrays."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.abs(a - b)
    bad = d > tol
    if not a.size:
        return 0, 0.0
    return int(np.count_nonzero(bad)), float(np.max(d / np.maximum(tol, 1e-300)))


def source_irradiance(desc):
    L = desc.light
    return float(L.irradiance) if L.enabled else 0.0


def compare_cells(got, want, before=None, rtol=RTOL, where="", scales=None, source=None, velocities=True):
    """Return a list of human-readable mismatches (empty when in parity).

    `scales` is the oracle's (force, velocity, displacement) term scales per
    slot of `want` (OracleWorld.export_term_scales) when the compared span
    contains a motion stage; without them velocities must agree to 1e-5 of
    themselves. `source` is the light source irradiance that floors the
    irradiance bound (default: 0, a purely relative bound). `velocities=False`
    leaves velocities out (free-running trajectories, where contact dynamics
    amplify FP32 rounding chaotically; positions stay compared). `before` is
    accepted for call compatibility and not used: both sides start from the
    same state, so |got - want| is the error of the step itself."""
    errs = []
    if got.n != want.n:
        return ["%s: count %d != %d" % (where, got.n, want.n)]
    src = 0.0 if source is None else float(source)
    for name, t in agb.CELL_FIELDS:
        a, b = got[name], want[name]
        if name in INT_FIELDS:
            nd = int(np.count_nonzero(a != b))
            if nd:
                idx = np.nonzero(a != b)[0][:5]
                errs.append("%s: %s differs in %d slots, e.g. %s" % (where, name, nd, idx.tolist()))
            continue
        bb = np.abs(np.asarray(b, np.float64))
        if name in POS_FIELDS:
            nb, worst = _excess(a, b, rtol * np.maximum(bb, agb.CELL_RADIUS))
            if nb:
                errs.append("%s: %s beyond 1e-5 of the coordinate (floor one radius) in %d slots (worst %.3g x)"
                            % (where, name, nb, worst))
            if scales is not None:
                nb, worst = _excess(a, b, rtol * scales[2] + POS_ABS_FLOOR)
                if nb:
                    errs.append("%s: %s displacement beyond 1e-5 of its term scale in %d slots (worst %.3g x)"
                                % (where, name, nb, worst))
            continue
        if name in VEL_FIELDS:
            if not velocities:
                continue
            floor = rtol * scales[1] if scales is not None else 0.0
            nb, worst = _excess(a, b, rtol * bb + floor + 1e-300)
        elif name == "irradiance":
            nb, worst = _excess(a, b, rtol * bb + rtol * src + 1e-300)
        else:
            nb, worst = _excess(a, b, rtol * bb + 1e-300)
        if nb:
            errs.append("%s: %s out of tolerance in %d slots (worst %.3g x the bound)" % (where, name, nb, worst))
    zero_a, zero_b = got["irradiance"] == 0.0, want["irradiance"] == 0.0
    nz = int(np.count_nonzero(zero_a != zero_b))
    if nz:
        errs.append("%s: exact-zero irradiance set differs in %d cells" % (where, nz))
    return errs


def compare_forces(fg, fo, where="", rtol=RTOL, scale=None):
    """Per axis |got - want| <= rtol * |want| + rtol * force scale (the oracle's
    per-cell summed magnitudes of the force's terms)."""
    errs = []
    for ax in range(3):
        b = np.asarray(fo[ax], np.float64)
        floor = rtol * np.asarray(scale, np.float64) if scale is not None else 0.0
        nb, worst = _excess(fg[ax], b, rtol * np.abs(b) + floor + 1e-300)
        if nb:
            errs.append("%s: force axis %d out of tolerance in %d cells (worst %.3g x the bound)"
                        % (where, ax, nb, worst))
    return errs


def compare_fields(got_world, want_world, rtol=RTOL, exact=False, where=""):
    errs = []
    src = source_irradiance(want_world.desc)
    for f in range(4):
        if want_world.desc.grid[f].nx <= 0:
            continue
        a, b = got_world.export_field(f), want_world.export_field(f)
        if exact:
            nd = int(np.count_nonzero(a != b))
            if nd:
                errs.append("%s: field %d differs in %d voxels (max %.3g)" % (where, f, nd, float(np.abs(a - b).max())))
        else:
            floor = rtol * src if f == agb.FIELD_IRR else 0.0
            nb, worst = _excess(a, b, rtol * np.abs(b.astype(np.float64)) + floor + 1e-300)
            if nb:
                errs.append("%s: field %d out of tolerance in %d voxels (worst %.3g x the bound)"
                            % (where, f, nb, worst))
    return errs
