"""The allocation-free diffusion entry point, agb_grid_diffuse_noalloc.

It serves callers that may not allocate device memory themselves (a fixed
device-memory budget reserved at start-up, a plugin inside a host that owns
the allocation policy, a real-time loop that cannot take cudaMalloc's implicit
synchronisation): they pass their own field buffer and the library supplies
the ping-pong partner from a fixed scratch array of AGB_NOALLOC_MAX_VOXELS
floats.

Checked through the C ABI against the existing entry point, agb_world_diffuse,
on the same field: two calls in a row, each compared after it returns, with
the tolerance the other diffusion tests use (bit for bit). Runs the same alone
in a fresh process (the first call resolves the scratch address) or after the
other tests (the scratch then holds an earlier call's data, which must not
matter). Also checked: grids beyond the scratch or beyond the stencil's launch
grid are refused without touching the caller's buffer, and calls after the
first leave the device's free memory unchanged.
"""
import numpy as np
import pytest

import helpers as H

agb = H.agb
pytestmark = pytest.mark.gpu

CASES = [
    # nx, ny, nz, dx [m], dt [s], bcs, face values
    (40, 36, 24, 1.0e-5, 2.0e-4,
     [agb.BC_DIRICHLET, agb.BC_ROBIN, agb.BC_NEUMANN, agb.BC_DIRICHLET, agb.BC_ROBIN, agb.BC_NEUMANN],
     [373.15, 280.0, 300.0, 310.0, 285.0, 295.0]),
    (128, 128, 1, 4.0e-3 / 128, 1.0e-3, [agb.BC_ROBIN] * 6, [293.15] * 6),
    (64, 48, 32, 6.25e-6, 1.0e-3, [agb.BC_NEUMANN] * 6, [0.0] * 6),
]


def world_for(nx, ny, nz, dx, bcs, faces):
    d = agb.default_desc(capacity=16, seed=3)
    d.taxis_enabled = 0
    d.chamber_w, d.chamber_h = nx * dx, ny * dx
    d.chamber_d = nz * dx if nz > 1 else 6.0e-5
    g = agb.GridDesc()
    g.nx, g.ny, g.nz = nx, ny, nz
    for k in range(6):
        g.bc[k] = bcs[k]
        g.face_value[k] = faces[k]
    g.diffusivity, g.init, g.deposit_scale = agb.WATER_THERMAL_DIFFUSIVITY, 300.0, 1e9
    d.grid[agb.FIELD_T] = g
    for f in (agb.FIELD_CO2, agb.FIELD_N2, agb.FIELD_IRR):
        d.grid[f] = agb.GridDesc()
    return agb.World(d)


@pytest.mark.parametrize("nx,ny,nz,dx,dt,bcs,faces", CASES)
def test_noalloc_matches_world_diffuse_twice(nx, ny, nz, dx, dt, bcs, faces):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(nx * ny + nz)
    f0 = (280.0 + 90.0 * rng.random((nz, ny, nx))).astype(np.float32)
    w = world_for(nx, ny, nz, dx, bcs, faces)
    w.import_field(agb.FIELD_T, f0)
    buf = torch.from_numpy(f0.copy()).cuda()
    for call in range(2):
        w.diffuse(agb.FIELD_T, dt)
        want = w.export_field(agb.FIELD_T)
        rc = agb.grid_diffuse_noalloc(buf.data_ptr(), nx, ny, nz, dx, agb.WATER_THERMAL_DIFFUSIVITY, dt,
                                      bcs, faces)
        assert rc == agb.OK, agb.status_name(rc)
        torch.cuda.synchronize()
        got = buf.cpu().numpy()
        assert np.array_equal(got, want), "call %d differs from agb_world_diffuse" % (call + 1)
    w.close()


def test_noalloc_rejects_grids_beyond_the_scratch():
    torch = pytest.importorskip("torch")
    buf = torch.zeros(16, dtype=torch.float32, device="cuda")
    n = 256
    assert n * n * 65 > agb.NOALLOC_MAX_VOXELS
    rc = agb.grid_diffuse_noalloc(buf.data_ptr(), n, n, 65, 1e-5, 1e-9, 1e-3, [agb.BC_NEUMANN] * 6, [0.0] * 6)
    assert agb.status_name(rc) == "CapacityExceeded"
    torch.cuda.synchronize()
    assert float(buf.abs().sum().item()) == 0.0, "nothing may be written when the call is rejected"


@pytest.mark.parametrize("nx,ny,nz", [(4, 1048576, 1), (2, 2, 1048576)])
def test_noalloc_rejects_unlaunchable_shapes(nx, ny, nz):
    """Grids within the voxel limit whose stencil launch would need more than
    65,535 blocks along y or z are refused up front; the buffer is untouched."""
    torch = pytest.importorskip("torch")
    assert nx * ny * nz <= agb.NOALLOC_MAX_VOXELS
    gen = torch.Generator(device="cuda").manual_seed(5)
    buf = 280.0 + 40.0 * torch.rand(nx * ny * nz, dtype=torch.float32, device="cuda", generator=gen)
    before = buf.clone()
    rc = agb.grid_diffuse_noalloc(buf.data_ptr(), nx, ny, nz, 1e-5, 1e-9, 1e-3, [agb.BC_NEUMANN] * 6, [0.0] * 6)
    assert agb.status_name(rc) == "Unsupported"
    torch.cuda.synchronize()
    assert torch.equal(buf, before), "a refused call must leave the caller's field as it was"


def test_noalloc_allocates_nothing():
    """The property the entry point exists for: once the first call on the
    device has resolved the scratch array, further calls leave the device's
    free memory exactly where it was."""
    torch = pytest.importorskip("torch")
    n = 96
    bufs = [torch.full((n, n, n), 300.0, dtype=torch.float32, device="cuda") for _ in range(3)]
    bufs[0][n // 2, n // 2, n // 2] = 400.0
    args = (n, n, n, 1e-5, agb.WATER_THERMAL_DIFFUSIVITY, 1e-3, [agb.BC_NEUMANN] * 6, [0.0] * 6)
    assert agb.grid_diffuse_noalloc(bufs[0].data_ptr(), *args) == agb.OK
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for b in bufs:
        for _ in range(3):
            assert agb.grid_diffuse_noalloc(b.data_ptr(), *args) == agb.OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
