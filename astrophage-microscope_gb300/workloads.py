"""The seeded synthetic workloads the engine is measured and parity-checked on.

Every workload is a (WorldDesc, Spawn, description) triple built from the
engine's own descriptor defaults; the population comes from the engine's
seeded PCG32 spawn, so the same seed gives the same cells on the GPU and in
the CPU oracle. Used by bench.py (timing) and the 3-D parity tests.

  cube2k      2,000 cells uniform in a 400 um cube, 64^3 grids, x- face held
              at 100 C, light along +z, 10 um hash cells, division off.
  slab25k     25,000 cells in a 550 um-wide slab of a 4 mm cube, lognormal
              charge (median 3 %, sigma_ln 0.5, clipped at 0.2), 128^3 grids,
              light along +x, division at 0.16 of the maximum store,
              compaction every 10 ticks.
  clusters1m  1,000,000 dormant cells from 64 Gaussian clusters (sigma 40 um)
              in a 4 mm cube, 256^3 grids, light along +z, CO2-quota division
              and compaction.
  clusters20k the 1M-cell workload scaled to 20,000 cells and 64^3 grids for
              the oracle: 8 clusters of sigma 20 um, which keeps the cluster
              cores as dense as the 1M-cell workload's.
  ref200k     the reference's own throughput test (tests/physics/test_perf.cu
              T28): its default world (4 mm x 4 mm x 60 um, depth-averaged
              512^2 temperature / 256^2 CO2 / 128^2 N2 / 512^2 irradiance
              grids), 200,000 dormant cells uniform at charge 0.02, seed
              20260802; the configuration the reference's published hash
              rebuild (0.110 ms) and tick rate (281 ticks/s) are quoted at.
  batch       n 4 mm chambers, cells log-uniform in [1e3, 2e5], grid edges
              from {64, 96, 128, 192}, charge swept to 20 %.
"""
import numpy as np

import agb

EMAX = agb.CELL_ENERGY_MAX
PLAIN = ("slab25k", "cube2k", "clusters1m", "clusters20k", "ref200k")


def grid3(n, D, init, scale, bc, face=None):
    return agb.grid(n, n, D, init, scale, bc, face_value=face)


def _clusters(cells, edge, clusters, sigma, seed, capacity):
    d = agb.default_desc(capacity=capacity, seed=seed, co2_init=1.5)
    d.chamber_w = d.chamber_h = d.chamber_d = 4.0e-3
    d.grid[agb.FIELD_T] = grid3(edge, agb.WATER_THERMAL_DIFFUSIVITY, agb.AMBIENT_TEMP_DEFAULT, 1e9, agb.BC_ROBIN)
    d.grid[agb.FIELD_CO2] = grid3(edge, agb.CO2_DIFFUSIVITY_WATER, 1.5, 1e15, agb.BC_NEUMANN)
    d.grid[agb.FIELD_N2] = agb.GridDesc()
    d.grid[agb.FIELD_IRR] = grid3(edge, agb.IRRADIANCE_NOMINAL_DIFFUSIVITY, 0.0, 1e18, agb.BC_NEUMANN)
    d.taxis_enabled = 0
    d.light = agb.Light(0.0, 0.0, 1.0, 1.0e4, 0.0, 1)
    d.compaction_enabled = 1
    d.biology_rate = 1.38e5
    d.hash_cell_size = 10e-6
    # Dormant: awake cells packed ~60 to a 15.6 um voxel overdrive the lumped
    # thermostat exchange past the lethal temperature within a few ticks.
    sp = agb.spawn(cells, placement=agb.PLACE_CLUSTERS, place_radius=sigma, clusters=clusters,
                   cluster_extent=3e-3, charge_dist=agb.DIST_UNIFORM, charge_a=0.0, charge_b=0.2, awake=False)
    info = dict(cells=cells, grid=edge, chamber_mm=4.0, light="+z", clusters=clusters,
                cluster_sigma_um=round(sigma * 1e6, 3), hash_cell_um=10.0, awake=False)
    return d, sp, info


def workload(name, seed=1):
    """(desc, spawn, description) for a plain-step configuration."""
    if name == "slab25k":
        d = agb.default_desc(capacity=50000, seed=seed, co2_init=1.0)
        d.chamber_w = d.chamber_h = d.chamber_d = 4.0e-3
        d.grid[agb.FIELD_T] = grid3(128, agb.WATER_THERMAL_DIFFUSIVITY, agb.AMBIENT_TEMP_DEFAULT, 1e9, agb.BC_ROBIN)
        d.grid[agb.FIELD_CO2] = grid3(128, agb.CO2_DIFFUSIVITY_WATER, 1.0, 1e15, agb.BC_NEUMANN)
        d.grid[agb.FIELD_N2] = agb.GridDesc()
        d.grid[agb.FIELD_IRR] = grid3(128, agb.IRRADIANCE_NOMINAL_DIFFUSIVITY, 0.0, 1e18, agb.BC_NEUMANN)
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
        d.grid[agb.FIELD_T] = grid3(64, agb.WATER_THERMAL_DIFFUSIVITY, agb.AMBIENT_TEMP_DEFAULT, 1e9, bc, face)
        d.grid[agb.FIELD_CO2] = grid3(64, agb.CO2_DIFFUSIVITY_WATER, 1.0, 1e15, agb.BC_NEUMANN)
        d.grid[agb.FIELD_N2] = agb.GridDesc()
        d.grid[agb.FIELD_IRR] = grid3(64, agb.IRRADIANCE_NOMINAL_DIFFUSIVITY, 0.0, 1e18, agb.BC_NEUMANN)
        d.taxis_enabled = 0
        d.hash_cell_size = 10e-6
        d.light = agb.Light(0.0, 0.0, 1.0, 1.0e4, 0.0, 1)
        sp = agb.spawn(2000, charge_dist=agb.DIST_UNIFORM, charge_a=0.0, charge_b=0.2, awake=True)
        return d, sp, dict(cells=2000, grid=64, chamber_mm=0.4, light="+z", hash_cell_um=10.0)
    if name == "clusters1m":
        return _clusters(1000000, 256, 64, 40e-6, seed, 2000000)
    if name == "clusters20k":
        return _clusters(20000, 64, 8, 20e-6, seed, 40000)
    if name == "ref200k":
        d = agb.default_desc(capacity=200000, seed=20260802 + seed - 1)
        sp = agb.spawn(200000, charge_dist=agb.DIST_CONSTANT, charge_a=0.02, awake=False)
        return d, sp, dict(cells=200000, grid="512^2 T, 256^2 CO2, 128^2 N2, 512^2 irradiance (depth-averaged)",
                           chamber_mm="4 x 4 x 0.06", light="off", hash_cell_um=22.0)
    raise ValueError("unknown workload " + name)


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
        d.grid[agb.FIELD_T] = grid3(e, agb.WATER_THERMAL_DIFFUSIVITY, agb.AMBIENT_TEMP_DEFAULT, 1e9, agb.BC_ROBIN)
        d.grid[agb.FIELD_CO2] = grid3(e, agb.CO2_DIFFUSIVITY_WATER, 1.0, 1e15, agb.BC_NEUMANN)
        d.grid[agb.FIELD_N2] = agb.GridDesc()
        d.grid[agb.FIELD_IRR] = grid3(e, agb.IRRADIANCE_NOMINAL_DIFFUSIVITY, 0.0, 1e18, agb.BC_NEUMANN)
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
