"""CPU-side checks of the C ABI: the library loads without a GPU and exports
every entry point include/agb.h declares; the Python mirror agrees with the
C default descriptor."""
import ctypes
import os
import re

import helpers as H

agb = H.agb


def declared_symbols():
    with open(os.path.join(H.ROOT, "include", "agb.h")) as fh:
        text = fh.read()
    return sorted(set(re.findall(r"\b(agb_[a-z_0-9]+)\s*\(", text)))


def test_header_matches_python_list():
    assert declared_symbols() == sorted(agb.exported_symbols())


def test_library_exports_every_declared_symbol():
    lib = agb.load()
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_default_desc_matches_c():
    lib = agb.load()
    d = agb.WorldDesc()
    lib.agb_world_desc_default(ctypes.byref(d))
    assert bytes(d) == bytes(agb.default_desc(capacity=25000, seed=20260802, co2_init=0.0))


def test_status_strings():
    lib = agb.load()
    assert lib.agb_status_str(0) == b"Ok"
    assert lib.agb_status_str(7) == b"CapacityExceeded"
