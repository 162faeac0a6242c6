"""Snapshots (contracts/snapshot_v1.h, src/sim/snapshot.cu): the engine writes
the reference's bytes for the same state, restores them bit for bit, and its
state hash is deterministic across a save/restore (INV-8)."""
import json
import os

import numpy as np
import pytest

import helpers as H
import parity as P
import scenarios as S

agb = H.agb
pytestmark = pytest.mark.gpu


def golden(name):
    with open(os.path.join(H.GOLDEN, name + ".json")) as fh:
        return json.load(fh)


def engine_from_oracle(sc):
    """Oracle world set up as the scenario says, and an engine world holding the same state."""
    orc = H.OracleWorld(sc["desc"])
    S.setup(orc, sc)
    gpu = agb.World(sc["desc"])
    P.copy_state(orc, gpu)
    return orc, gpu


@pytest.mark.parametrize("name", ["slab_uniform", "lifecycle_compaction", "hot_field", "dense_cluster"])
def test_engine_snapshot_is_reference_bytes(name):
    """Same state in, same file out: the engine's snapshot of the scenario's
    initial state carries the digest and state hash the reference produced."""
    sc = S.scenarios()[name]
    orc, gpu = engine_from_oracle(sc)
    data = gpu.snapshot(b"golden")
    assert data == orc.snapshot(b"golden")
    assert S.snapshot_record(data) == golden(name)["snapshot_initial"]
    assert gpu.state_hash() == int(golden(name)["snapshot_initial"]["state_hash"], 16)


def test_restore_round_trip_and_determinism():
    sc = S.scenarios()["lifecycle_compaction"]
    gpu = agb.World(sc["desc"])
    S.setup(gpu, sc)
    gpu.step(3)
    data = gpu.snapshot(b"rt")
    back = agb.snapshot_load(sc["desc"], data)
    assert back.snapshot(b"rt") == data
    assert back.state_hash() == gpu.state_hash()
    hdr = np.frombuffer(data[:256], np.uint8)
    assert int(hdr[8:16].view(np.uint64)[0]) == sc["desc"].seed
    assert int(hdr[16:24].view(np.uint64)[0]) == 3              # tick
    # Same state + same ticks -> same state hash (INV-8), and the same cells.
    gpu.step(2)
    back.step(2)
    assert back.state_hash() == gpu.state_hash()
    a, _ = gpu.export_cells()
    b, _ = back.export_cells()
    for n, _t in agb.CELL_FIELDS:
        assert np.array_equal(a[n], b[n]), n


def test_load_reference_snapshot():
    """A snapshot the reference algorithm wrote (oracle bytes == reference bytes
    on the CPU) restores into the engine with every array intact."""
    sc = S.scenarios()["hot_field"]
    orc = H.OracleWorld(sc["desc"])
    S.setup(orc, sc)
    orc.step(1)
    data = orc.snapshot(b"from-reference")
    gpu = agb.snapshot_load(sc["desc"], data)
    a, na = gpu.export_cells()
    b, nb = orc.export_cells()
    assert na == nb
    for n, _t in agb.CELL_FIELDS:
        assert np.array_equal(a[n], b[n]), n
    for f in (agb.FIELD_T, agb.FIELD_CO2, agb.FIELD_N2):
        assert np.array_equal(gpu.export_field(f), orc.export_field(f))
    assert gpu.snapshot(b"from-reference") == data


def test_rejects_bad_snapshots():
    sc = S.scenarios()["slab_uniform"]
    gpu = agb.World(sc["desc"])
    S.setup(gpu, sc)
    data = bytearray(gpu.snapshot(b"bad"))
    corrupt = bytearray(data)
    corrupt[300] ^= 1                                           # body byte: hash mismatch
    assert agb.snapshot_status(sc["desc"], bytes(corrupt)) == 3          # InvalidArgument
    magic = bytearray(data)
    magic[0] ^= 1
    assert agb.snapshot_status(sc["desc"], bytes(magic)) == 3
    ver = bytearray(data)
    ver[4] = 2
    assert agb.snapshot_status(sc["desc"], bytes(ver)) == 6              # ContractVersionMismatch
    assert agb.snapshot_status(sc["desc"], bytes(data[:100])) == 8       # FileIoError: too small
    other = S.slab_desc(n_t=32)                                           # resolution differs
    assert agb.snapshot_status(other, bytes(data)) == 3
    assert agb.snapshot_status(sc["desc"], bytes(data)) == 0
