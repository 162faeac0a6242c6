"""The host <-> device cell transfer kernels (agb_world_import_cells /
agb_world_export_cells when the GPU addresses the host arrays directly): one
thread per cell moves its 25 contract elements. Host arrays need only be
aligned to their element size; populations of any size, including empty and
one cell, and arrays one element past a 16-byte boundary move the same bytes
as aligned ones."""
import numpy as np
import pytest

import helpers as H

agb = H.agb
pytestmark = pytest.mark.gpu


def world(n, seed=5, spawn=True):
    d = agb.default_desc(capacity=max(n, 1) + 64, seed=seed)
    w = agb.World(d)
    if n and spawn:
        w.spawn(agb.spawn(n, charge_dist=agb.DIST_UNIFORM, charge_a=0.1, charge_b=0.9, awake=True))
        w.step(1)                     # every array non-trivial (velocities, temperatures, timers)
    return w


def misaligned(n, hold):
    """CellArrays whose arrays start one element past a 16-byte boundary (an
    element-aligned, not 16-byte-aligned address; byte arrays one byte past)."""
    c = agb.CellArrays(n)
    for name, t in agb.CELL_FIELDS:
        e = np.dtype(t).itemsize
        buf = np.zeros(max(n, 1) * e + 64, np.uint8)
        base = (-buf.ctypes.data) % 16
        arr = buf[base + e: base + e + max(n, 1) * e].view(t)
        assert arr.ctypes.data % 16 == e % 16
        hold.append(buf)
        c.a[name] = arr
    return c


def same(x, y):
    assert x.n == y.n
    for name, _t in agb.CELL_FIELDS:
        assert np.array_equal(x[name].view(np.uint8), y[name].view(np.uint8)), name


@pytest.mark.parametrize("n", [0, 1, 3, 17, 1001, 25000])
def test_export_import_aligned_and_misaligned_move_the_same_bytes(n):
    w = world(n)
    ref, nid = w.export_cells()
    hold = []
    mis = misaligned(n, hold)
    got, nid2 = w.export_cells(into=mis)
    assert nid2 == nid
    same(got, ref)
    # Import from the misaligned arrays into a fresh world; export aligned.
    w2 = world(n, spawn=False)
    w2.import_cells(got, nid)
    back, nid3 = w2.export_cells()
    assert nid3 == nid and w2.count() == n
    same(back, ref)
    w.close()
    w2.close()


def test_export_into_bounded_buffers_stops_at_their_length():
    w = world(500)
    ref, _ = w.export_cells()
    small = agb.CellArrays(123)
    got, _ = w.export_cells(into=small)     # 500 cells do not fit: fresh arrays come back
    same(got, ref)
    w.close()
