"""Comparison helpers for engine-vs-oracle parity.

Integer state (ids, flags, death causes, PCG32 states, hash keys, sorted
order, bucket ranges, slot assignment) must match exactly. Floating-point
state is compared with the tolerance the engine is built to: the engine
computes per-cell physics in FP32 and commits it into FP64 state, so one
step's increments (displacement, velocity, energy and CO2 changes) agree to
~1e-6 relative; the test bound is RTOL = 1e-5. Positions are compared
through their per-step displacement, because 1e-5 of a millimetre position
is larger than a whole Brownian step.
"""
import numpy as np

from helpers import agb

RTOL = 1e-5
INT_FIELDS = ("id", "flags", "death_cause", "rng_state")
DELTA_FIELDS = ("x", "y", "z", "energy", "co2_held")


def copy_state(src, dst, fields=True):
    cells, nid = src.export_cells()
    dst.import_cells(cells, nid)
    if fields:
        for f in range(4):
            if src.desc.grid[f].nx > 0:
                dst.import_field(f, src.export_field(f))
    return cells


def _close(a, b, rtol, atol):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    bad = np.abs(a - b) > rtol * np.abs(b) + atol
    return int(np.count_nonzero(bad)), (float(np.max(np.abs(a - b))) if a.size else 0.0)


def _rms(a):
    a = np.asarray(a, np.float64)
    return float(np.sqrt(np.mean(a * a))) if a.size else 0.0


def compare_cells(got, want, before=None, rtol=RTOL, where=""):
    """Return a list of human-readable mismatches (empty when in parity).

    Per element: |got - want| <= rtol * |want| + atol, with atol = 1e-4 of the
    population's RMS of that quantity (for positions, energy and CO2: of the
    step's increment). The absolute floor covers components that happen to sit
    near zero, where FP32 contact sums (error ~1e-7 of the summed magnitudes)
    make a purely relative bound meaningless. Positions must also meet the
    stated 1e-5 relative bound on the position itself."""
    errs = []
    if got.n != want.n:
        return ["%s: count %d != %d" % (where, got.n, want.n)]
    for name, t in agb.CELL_FIELDS:
        a, b = got[name], want[name]
        if name in INT_FIELDS:
            nd = int(np.count_nonzero(a != b))
            if nd:
                idx = np.nonzero(a != b)[0][:5]
                errs.append("%s: %s differs in %d slots, e.g. %s" % (where, name, nd, idx.tolist()))
            continue
        if name in ("x", "y", "z"):
            # The stated bound, relative to the position (floored at one cell
            # radius so that cells near the chamber centre are not held to
            # sub-picometre agreement).
            bb = np.maximum(np.abs(b.astype(np.float64)), agb.CELL_RADIUS)
            nb = int(np.count_nonzero(np.abs(a.astype(np.float64) - b) > rtol * bb))
            if nb:
                errs.append("%s: %s beyond 1e-5 relative in %d slots" % (where, name, nb))
        if before is not None and name in DELTA_FIELDS and before.n == want.n:
            p = before[name].astype(np.float64)
            da, db = a.astype(np.float64) - p, b.astype(np.float64) - p
            atol = 1e-4 * _rms(db) + 1e-300
            if name in ("x", "y", "z"):
                atol = max(atol, 1e-15)
            if name == "energy":
                atol = max(atol, 1e-15 * float(np.max(np.abs(p))))
            nb, mx = _close(da, db, rtol, atol)
        else:
            nb, mx = _close(a, b, rtol, 1e-4 * _rms(b) + 1e-30)
        if nb:
            errs.append("%s: %s out of tolerance in %d slots (max abs diff %.3g)" % (where, name, nb, mx))
    zero_a, zero_b = got["irradiance"] == 0.0, want["irradiance"] == 0.0
    nz = int(np.count_nonzero(zero_a != zero_b))
    if nz:
        errs.append("%s: exact-zero irradiance set differs in %d cells" % (where, nz))
    return errs


def compare_forces(fg, fo, where="", rtol=RTOL):
    errs = []
    for ax in range(3):
        b = np.asarray(fo[ax], np.float64)
        nb, mx = _close(fg[ax], b, rtol, 1e-4 * _rms(b) + 1e-30)
        if nb:
            errs.append("%s: force axis %d out of tolerance in %d cells (max %.3g)" % (where, ax, nb, mx))
    return errs


def compare_fields(got_world, want_world, rtol=1e-6, exact=False, where=""):
    errs = []
    for f in range(4):
        if want_world.desc.grid[f].nx <= 0:
            continue
        a, b = got_world.export_field(f), want_world.export_field(f)
        if exact:
            nd = int(np.count_nonzero(a != b))
            if nd:
                errs.append("%s: field %d differs in %d voxels (max %.3g)" % (where, f, nd, float(np.abs(a - b).max())))
        else:
            scale = float(np.max(np.abs(b))) if b.size else 0.0
            nb, mx = _close(a, b, rtol, 1e-3 * rtol * scale + 1e-30)
            if nb:
                errs.append("%s: field %d out of tolerance in %d voxels (max %.3g)" % (where, f, nb, mx))
    return errs
