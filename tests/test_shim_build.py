"""The C++ shim (astrophage-microscope_gb300/shim/astro_sim_gb.cu) compiles
against the reference's own headers, its static_asserts hold (agb_cells is
CellStoreView, agb_stats is Stats), and programs written against the
reference's World API link to it with none of the reference's physics
compiled in: thirteen of its tests/physics programs, and its test_scenario
and tools/headless with the reference's own (host-side) scenario loader and
acceptance code.

Needs a reference checkout named by AGB_REFERENCE_DIR (skipped otherwise) and
nvcc; runs nothing on a GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "astrophage-microscope_gb300")
SCRIPT = os.path.join(PKG, "shim", "build_shim.sh")
REF = os.environ.get("AGB_REFERENCE_DIR", "")
# Reference test programs that use only the World API the shim provides.
PROGRAMS = ["test_clock", "test_perf", "test_stats", "test_buoyancy", "test_emission", "test_taxis",
            "test_contact", "test_param_override", "test_thermal", "test_lifecycle", "test_predation",
            "test_snapshot", "test_evolution"]
# Programs that also compile the reference's scenario loader and acceptance code.
WITH_SCENARIOS = {"test_scenario": "tests/physics/test_scenario.cu", "headless": "tools/headless.cpp"}

pytestmark = pytest.mark.skipif(not (REF and os.path.isfile(os.path.join(REF, "src", "sim", "world.cuh"))),
                                reason="AGB_REFERENCE_DIR does not name a reference checkout")


@pytest.fixture(scope="module")
def engine():
    if shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("nvcc not found")
    lib = os.path.join(PKG, "libagb.so")
    if not os.path.exists(lib):
        import sys
        sys.path.insert(0, PKG)
        import build
        build.build()
    return lib


def test_shim_links_reference_programs(engine, tmp_path):
    progs = [os.path.join(REF, "tests", "physics", p + ".cu") for p in PROGRAMS]
    extra = [os.path.join(REF, "src", "sim", f) for f in ("scenario.cpp", "accept.cpp")]
    progs += [":".join([os.path.join(REF, src)] + extra) for src in WITH_SCENARIOS.values()]
    env = dict(os.environ)
    env.setdefault("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")
    r = subprocess.run(["sh", SCRIPT, REF, str(tmp_path)] + progs, capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    assert (tmp_path / "libastro_sim_gb.so").exists()
    for p in PROGRAMS + list(WITH_SCENARIOS):
        assert (tmp_path / p).exists(), p
    # The programs resolve the World API from the shim, not from reference code.
    nm = subprocess.run(["nm", "-D", "--defined-only", str(tmp_path / "libastro_sim_gb.so")],
                        capture_output=True, text=True).stdout
    for sym in ("world_create", "world_step", "world_stats", "cell_store_spawn", "grid_download"):
        assert sym in nm, sym
