"""Independent pins of the 3-D generalisation of the reference's physics.

The reference's fields are depth-averaged 2-D grids; its own tests pin them
with analytic oracles (tests/physics/test_fields.cu:76-156: a Gaussian
spreading as sigma^2 = sigma0^2 + 2 D t, conservation under an insulated
boundary to 0.1 %; tests/physics/test_emission.cu:73-133: exact darkness
behind a collinear cell). The oracle's 3-D generalisation (7-point stencil
with a condition per face, trilinear sampling, the nearest voxel in z, a
voxel's heat capacity rho c_p dx^3, light along z and the voxel face dx^2 of
a 3-D sweep) is pinned here by the same kind of checks, restated in 3-D, plus
closed forms computed independently in numpy:

  * a Gaussian spreads as sigma^2 = sigma0^2 + 2 D t along each axis (2 %);
  * an insulated grid conserves its total (0.1 %), without overshoot;
  * a field uniform across y and z evolves as the 1-D three-point FTCS with
    the same coefficient and the x faces' conditions (Dirichlet, Robin);
  * trilinear sampling reproduces a linear field, and equals a float64
    restatement of clamped trilinear interpolation on a random field;
  * one awake cell exchanges heat with its voxel as the lumped closed form
    with C = rho c_p dx^3, and the energy it loses is the voxel's C dT;
  * a single cell shades its column along +x, -y, +z and -z by exactly
    (1 - area / dx^2) beyond its voxel, a dead cell by its albedo-reduced
    area, and a cell behind another on the light axis gets exactly zero.

Each check takes a world factory, so the same checks run on the engine
(test_gpu_parity3d.py) with the GPU world.
"""
import os
import re

import numpy as np
import pytest

import helpers as H

agb = H.agb


def canon(name):
    """A canon constant from include/agb_canon.h (the engine's own table)."""
    with open(os.path.join(H.ROOT, "include", "agb_canon.h")) as fh:
        m = re.search(r"#define AGB_%s ([-0-9.eE+]+)" % name, fh.read())
    return float(m.group(1))


def oracle(desc):
    return H.OracleWorld(desc, threads=os.cpu_count() or 1)


def grid_world(n, span, D, bc, face=None, nz=None, cap=16):
    """A world holding only a temperature grid of n x n x nz voxels over a
    cubic chamber of edge `span` (nz = n by default)."""
    nz = n if nz is None else nz
    d = agb.default_desc(capacity=cap, seed=5)
    d.taxis_enabled = 0
    d.chamber_w = d.chamber_h = span
    d.chamber_d = span * nz / n
    d.grid[agb.FIELD_T] = agb.grid(n, nz, D, agb.AMBIENT_TEMP_DEFAULT, 1e9, bc, face_value=face)
    for f in (agb.FIELD_CO2, agb.FIELD_N2, agb.FIELD_IRR):
        d.grid[f] = agb.GridDesc()
    return d


# ---------------------------------------------------------------------------
# The stencil and its boundary conditions
# ---------------------------------------------------------------------------
def check_gaussian_3d(make):
    n, span = 96, 1.2e-3
    D = agb.WATER_THERMAL_DIFFUSIVITY
    w = make(grid_world(n, span, D, agb.BC_NEUMANN))
    dx = span / n
    c = (np.arange(n) + 0.5) * dx - 0.5 * span
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    s0 = 5.0e-5
    f0 = (100.0 * np.exp(-(x * x + y * y + z * z) / (2 * s0 * s0))).astype(np.float32)
    w.import_field(agb.FIELD_T, f0)
    ticks = 20
    for _ in range(ticks):
        w.diffuse(agb.FIELD_T, agb.DT_PHYSICS)
    f = w.export_field(agb.FIELD_T).astype(np.float64)
    want = s0 * s0 + 2.0 * D * ticks * agb.DT_PHYSICS
    tot = f.sum()
    for axis, coord in (("x", x), ("y", y), ("z", z)):
        var = float((f * coord * coord).sum() / tot - ((f * coord).sum() / tot) ** 2)
        assert abs(var - want) <= 2e-2 * want, "%s variance %.4g, analytic %.4g" % (axis, var, want)


def check_conservation_3d(make):
    n = 48
    w = make(grid_world(n, 1.0e-3, agb.WATER_THERMAL_DIFFUSIVITY, agb.BC_NEUMANN))
    f0 = np.zeros((n, n, n), np.float32)
    f0[n // 2 - 5:n // 2 + 5, n // 2 - 5:n // 2 + 5, n // 2 - 5:n // 2 + 5] = 100.0
    w.import_field(agb.FIELD_T, f0)
    for _ in range(100):
        w.diffuse(agb.FIELD_T, agb.DT_PHYSICS)
    f = w.export_field(agb.FIELD_T)
    t0, t1 = float(f0.astype(np.float64).sum()), float(f.astype(np.float64).sum())
    assert np.isfinite(f).all()
    assert abs(t1 - t0) <= 1e-3 * t0, (t0, t1)
    assert f.min() >= -1e-4 and f.max() <= 100.0 + 1e-3


def ftcs_1d(u, coeff, lo, hi, bc, face, robin, passes):
    """The three-point FTCS with ghost cells, in float64: Dirichlet holds the
    face value, Robin relaxes toward it by `robin`, Neumann mirrors."""
    u = u.astype(np.float64).copy()

    def ghost(k, c):
        if bc[k] == agb.BC_DIRICHLET:
            return face[k]
        if bc[k] == agb.BC_ROBIN:
            return c - robin * (c - face[k])
        return c
    for _ in range(passes):
        left = np.concatenate(([ghost(lo, u[0])], u[:-1]))
        right = np.concatenate((u[1:], [ghost(hi, u[-1])]))
        u = u + coeff * (left + right - 2.0 * u)
    return u


def check_stencil_reduces_to_1d(make, bcx=(agb.BC_DIRICHLET, agb.BC_ROBIN)):
    n, span = 40, 4.0e-4
    D = agb.WATER_THERMAL_DIFFUSIVITY
    bc = [bcx[0], bcx[1], agb.BC_NEUMANN, agb.BC_NEUMANN, agb.BC_NEUMANN, agb.BC_NEUMANN]
    face = [373.15, 280.0, 0.0, 0.0, 0.0, 0.0]
    w = make(grid_world(n, span, D, bc, face=face, nz=24))
    rng = np.random.default_rng(3)
    prof = (290.0 + 40.0 * rng.random(n)).astype(np.float32)
    w.import_field(agb.FIELD_T, np.broadcast_to(prof, (24, n, n)).copy())
    dx = span / n
    dt = 3.0e-3
    steps = int(dt / (dx * dx / (6.0 * D))) + 1
    coeff = float(np.float32(D * (dt / steps) / (dx * dx)))
    robin = float(np.float32(dx * agb.AIR_CONVECTION_H / agb.WATER_CONDUCTIVITY))
    w.diffuse(agb.FIELD_T, dt)
    f = w.export_field(agb.FIELD_T).astype(np.float64)
    want = ftcs_1d(prof, coeff, 0, 1, bc, [float(np.float32(v)) for v in face], robin, steps)
    # Uniform across y and z: every column equals the 1-D solution (FP32 sums).
    assert np.abs(f - f[:1, :1, :]).max() <= 1e-4
    assert np.abs(f[0, 0] - want).max() <= 1e-5 * np.abs(want).max()


# ---------------------------------------------------------------------------
# Sampling and the nearest voxel
# ---------------------------------------------------------------------------
def trilinear(field, dx, x, y, z):
    """Clamped trilinear interpolation at voxel centres, in float64."""
    nz, ny, nx = field.shape

    def axis(p, n):
        g = (p + 0.5 * n * dx) / dx - 0.5
        i0 = np.floor(g).astype(np.int64)
        t = g - i0
        return np.clip(i0, 0, n - 1), np.clip(i0 + 1, 0, n - 1), t
    x0, x1, tx = axis(x, nx)
    y0, y1, ty = axis(y, ny)
    z0, z1, tz = axis(z, nz)
    f = field.astype(np.float64)

    def bil(zz):
        return ((1 - tx) * (1 - ty) * f[zz, y0, x0] + tx * (1 - ty) * f[zz, y0, x1] +
                (1 - tx) * ty * f[zz, y1, x0] + tx * ty * f[zz, y1, x1])
    return (1 - tz) * bil(z0) + tz * bil(z1)


def sampled_world(make, field, n, span, count, rng, margin):
    d = grid_world(n, span, agb.WATER_THERMAL_DIFFUSIVITY, agb.BC_NEUMANN, cap=count)
    d.thermal_enabled = 0
    d.contact_enabled = 0
    w = make(d)
    w.spawn(agb.spawn(count))
    cells, nid = w.export_cells()
    h = 0.5 * span - margin
    for k in ("x", "y", "z"):
        cells.a[k][:] = rng.uniform(-h, h, count)
    w.import_cells(cells, nid)
    w.import_field(agb.FIELD_T, field)
    w.stage(agb.STAGE_HASH)
    w.stage(agb.STAGE_MOTION)                 # samples t_local at the positions it starts from
    after, _ = w.export_cells()
    return cells, after


def check_trilinear_sampling(make):
    n, span = 32, 6.4e-4
    dx = span / n
    rng = np.random.default_rng(11)
    c = (np.arange(n) + 0.5) * dx - 0.5 * span
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    lin = (300.0 + 2.0e4 * x - 1.5e4 * y + 3.0e4 * z).astype(np.float32)
    cells, after = sampled_world(make, lin, n, span, 500, rng, 0.5 * dx + 1e-9)
    want = 300.0 + 2.0e4 * cells["x"] - 1.5e4 * cells["y"] + 3.0e4 * cells["z"]
    assert np.abs(after["t_local"] - want).max() <= 1e-5 * 300.0
    rnd = (290.0 + 60.0 * rng.random((n, n, n))).astype(np.float32)
    cells, after = sampled_world(make, rnd, n, span, 800, rng, 0.0)       # walls included: clamped
    want = trilinear(rnd, dx, cells["x"], cells["y"], cells["z"])
    assert np.abs(after["t_local"] - want).max() <= 1e-5 * np.abs(want).max()


def check_heat_capacity_3d(make):
    """One awake cell at the setpoint in a 293.15 K voxel of a grid that does
    not diffuse: the voxel warms by (T_set - T0)(1 - exp(-G dt / C)) with
    C = rho c_p dx^3, and the cell's store falls by C times that."""
    n, span = 16, 3.2e-4
    d = grid_world(n, span, 0.0, agb.BC_NEUMANN, cap=4)
    d.emission_enabled = 0
    w = make(d)
    w.spawn(agb.spawn(1, awake=True))
    cells, nid = w.export_cells()
    dx = span / n
    cells.a["x"][0], cells.a["y"][0], cells.a["z"][0] = 2.5 * dx - 0.5 * span, 7.5 * dx - 0.5 * span, \
        11.5 * dx - 0.5 * span
    cells.a["energy"][0] = 0.5 * agb.CELL_ENERGY_MAX
    w.import_cells(cells, nid)
    e0 = float(cells["energy"][0])
    w.stage(agb.STAGE_THERMAL)
    f = w.export_field(agb.FIELD_T).astype(np.float64)
    after, _ = w.export_cells()
    cap = canon("WATER_DENSITY") * canon("WATER_SPECIFIC_HEAT") * dx ** 3
    relax = -np.expm1(-canon("CONDUCTION_COEFF") * agb.DT_PHYSICS / cap)
    t0 = float(np.float32(agb.AMBIENT_TEMP_DEFAULT))
    dT = (canon("CELL_TEMP_SETPOINT") - t0) * relax
    got = f[11, 7, 2] - t0
    assert abs(got - dT) <= 2 * np.spacing(np.float32(t0 + dT)), (got, dT)
    others = f.copy()
    others[11, 7, 2] = t0
    assert np.all(others == t0)
    assert abs((e0 - after["energy"][0]) - cap * dT) <= 1e-5 * cap * dT


# ---------------------------------------------------------------------------
# Light along each axis: stamps, the 3-D sweep and exact shadows
# ---------------------------------------------------------------------------
def lit_world(make, direction, count, irr=1.0e4, amb=3.0):
    n, span = 24, 4.8e-4
    d = agb.default_desc(capacity=max(count, 1), seed=9)
    d.taxis_enabled = 0
    d.thermal_enabled = 0
    d.chamber_w = d.chamber_h = d.chamber_d = span
    for f in (agb.FIELD_T, agb.FIELD_CO2, agb.FIELD_N2):
        d.grid[f] = agb.GridDesc()
    d.grid[agb.FIELD_IRR] = agb.grid(n, n, agb.IRRADIANCE_NOMINAL_DIFFUSIVITY, 0.0, 1e18, agb.BC_NEUMANN)
    d.light = agb.Light(direction[0], direction[1], direction[2], irr, amb, 1)
    w = make(d)
    w.spawn(agb.spawn(count, awake=True))
    return w, n, span / n


def place(w, pts, alive=None):
    cells, nid = w.export_cells()
    for i, p in enumerate(pts):
        cells.a["x"][i], cells.a["y"][i], cells.a["z"][i] = p
        if alive is not None and not alive[i]:
            cells.a["flags"][i] &= np.uint32(0xFFFFFFFF ^ agb.FLAG_ALIVE)
    w.import_cells(cells, nid)


def check_column_shading(make, direction=(0.0, 0.0, 1.0)):
    irr, amb = np.float32(1.0e4), np.float32(3.0)
    w, n, dx = lit_world(make, direction, 3, irr, amb)
    vox = [(5, 7, 9), (5, 7, 9), (14, 3, 20)]               # two cells in one voxel, one dead elsewhere
    pts = [((i + 0.5) * dx - 12 * dx, (j + 0.5) * dx - 12 * dx, (k + 0.5) * dx - 12 * dx) for i, j, k in vox]
    pts[1] = (pts[1][0] + 0.3 * dx, pts[1][1] - 0.2 * dx, pts[1][2] + 0.1 * dx)
    place(w, pts, alive=[True, True, False])
    w.stage(agb.STAGE_HASH)
    w.stage(agb.STAGE_EMISSION)
    f = w.export_field(agb.FIELD_IRR)
    area = canon("CELL_CROSS_SECTION")
    q = lambda a: float(round(a * 1e18)) / 1e18           # the 1e18 fixed-point deposit
    want = np.full((n, n, n), irr + amb, np.float32)
    axis = int(np.argmax(np.abs(direction)))
    sign = 1 if direction[axis] > 0 else -1
    for (i, j, k), a in (((5, 7, 9), q(2 * area)), ((14, 3, 20), q(area * (1 - canon("CELL_ALBEDO_DEAD"))))):
        t = max(0.0, 1.0 - a / (dx * dx))
        val = np.float32(np.float64(irr) * t) + amb
        idx = [k, j, i]
        pos = idx[2 - axis]
        sl = [k, j, i]
        rng_ = range(pos + 1, n) if sign > 0 else range(0, pos)
        for p in rng_:
            sl[2 - axis] = p
            want[tuple(sl)] = val
    assert np.array_equal(f, want), "%d voxels differ" % int(np.count_nonzero(f != want))


def check_exact_zero_behind_3d(make):
    """T13 along z: the rear cell of a collinear pair on the light axis gets
    exactly zero directional irradiance; with no ambient it gains nothing."""
    w, n, dx = lit_world(make, (0.0, 0.0, 1.0), 2, 1.0e4, 0.0)
    place(w, [(1.0e-6, -2.0e-6, -7.5e-6), (1.0e-6, -2.0e-6, 7.5e-6)])
    cells, nid = w.export_cells()
    cells.a["energy"][:2] = 0.0
    w.import_cells(cells, nid)
    w.stage(agb.STAGE_HASH)
    w.stage(agb.STAGE_EMISSION)
    a, _ = w.export_cells()
    assert a["irradiance"][0] > 0.0 and a["energy"][0] > 0.0
    assert a["irradiance"][1] == 0.0 and a["energy"][1] == 0.0


CHECKS = [check_gaussian_3d, check_conservation_3d, check_stencil_reduces_to_1d, check_trilinear_sampling,
          check_heat_capacity_3d, check_exact_zero_behind_3d]
DIRECTIONS = [(1.0, 0.0, 0.0), (0.0, -1.0, 0.0), (0.0, 0.0, 1.0), (0.0, 0.0, -1.0)]


@pytest.mark.parametrize("check", CHECKS, ids=[c.__name__ for c in CHECKS])
def test_oracle_3d(check):
    check(oracle)


@pytest.mark.parametrize("bcx", [(agb.BC_DIRICHLET, agb.BC_ROBIN), (agb.BC_ROBIN, agb.BC_DIRICHLET)])
def test_oracle_stencil_faces(bcx):
    check_stencil_reduces_to_1d(oracle, bcx)


@pytest.mark.parametrize("direction", DIRECTIONS)
def test_oracle_column_shading(direction):
    check_column_shading(oracle, direction)
