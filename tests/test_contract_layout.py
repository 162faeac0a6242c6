"""The boundary's structs are the reference's contract structs, byte for byte.

agb_cells must be CellStoreView (contracts/cell_store_v1.h:42-78) and agb_stats
must be Stats (contracts/telemetry_v1.h:17-39): same members, offsets, sizes,
total size and alignment, so a caller of the reference can hand its own views
and receive its own Stats through the C ABI. The reference's layout is pinned
in tests/golden/contract_layout.json (written by tests/golden/make_layout.py
from the reference's headers); the checks here compile include/agb.h as C and
as C++ with one static assert per member, and compare the Python mirror. With
AGB_REFERENCE_DIR pointing at the reference's sources, a translation unit that
includes both headers asserts the equalities directly.
"""
import ctypes
import json
import os
import subprocess
import tempfile

import pytest

import helpers as H

agb = H.agb
GOLD = os.path.join(H.GOLDEN, "contract_layout.json")
PAIRS = (("agb_cells", "CellStoreView"), ("agb_stats", "Stats"))


def layout():
    with open(GOLD) as fh:
        return json.load(fh)


def asserts(c_lang):
    sa = "_Static_assert" if c_lang else "static_assert"
    out = []
    for mine, theirs in PAIRS:
        t = layout()[theirs]
        out.append('%s(sizeof(%s) == %d, "%s size");' % (sa, mine, t["__size__"], mine))
        out.append('%s(_Alignof(%s) == %d, "%s align");' % (sa, mine, t["__align__"], mine) if c_lang else
                   '%s(alignof(%s) == %d, "%s align");' % (sa, mine, t["__align__"], mine))
        for m, v in t.items():
            if m.startswith("__"):
                continue
            off, size = v
            out.append('%s(offsetof(%s, %s) == %d, "%s.%s offset");' % (sa, mine, m, off, mine, m))
            out.append('%s(sizeof(((%s*)0)->%s) == %d, "%s.%s size");' % (sa, mine, m, size, mine, m))
    return "\n".join(out)


def compile_tu(text, suffix, cmd):
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "layout" + suffix)
        with open(src, "w") as fh:
            fh.write(text)
        r = subprocess.run(cmd + [src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


INC = os.path.join(H.ROOT, "include")


def test_agb_structs_match_reference_layout_in_c():
    compile_tu('#include <stddef.h>\n#include "agb.h"\n' + asserts(True) + "\n", ".c",
               ["gcc", "-std=c11", "-fsyntax-only", "-I" + INC])


def test_agb_structs_match_reference_layout_in_cpp():
    compile_tu('#include <cstddef>\n#include "agb.h"\n' + asserts(False) + "\n", ".cpp",
               ["g++", "-std=c++17", "-fsyntax-only", "-I" + INC])


def test_python_mirror_matches_reference_layout():
    for cls, theirs in ((agb.Cells, "CellStoreView"), (agb.Stats, "Stats")):
        t = layout()[theirs]
        assert ctypes.sizeof(cls) == t["__size__"], theirs
        for m, v in t.items():
            if not m.startswith("__"):
                assert getattr(cls, m).offset == v[0] and getattr(cls, m).size == v[1], (theirs, m)


@pytest.mark.skipif(not os.path.isdir(os.path.join(os.environ.get("AGB_REFERENCE_DIR", "/nonexistent"), "contracts")),
                    reason="AGB_REFERENCE_DIR does not point at the reference's sources")
def test_agb_structs_equal_reference_structs_directly():
    ref = os.environ["AGB_REFERENCE_DIR"]
    lines = ['#include <cstddef>', '#include "agb.h"', '#include "contracts/cell_store_v1.h"',
             '#include "contracts/telemetry_v1.h"', 'using astro::contract::CellStoreView;',
             'using astro::contract::Stats;']
    for mine, theirs in PAIRS:
        lines.append('static_assert(sizeof(%s) == sizeof(%s), "size");' % (mine, theirs))
        for m in layout()[theirs]:
            if not m.startswith("__"):
                lines.append('static_assert(offsetof(%s, %s) == offsetof(%s, %s), "%s");' % (mine, m, theirs, m, m))
    compile_tu("\n".join(lines) + "\n", ".cpp", ["g++", "-std=c++20", "-fsyntax-only", "-I" + INC, "-I" + ref])
