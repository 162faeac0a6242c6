"""Record the reference's contract struct layouts (tests/golden/contract_layout.json).

Compiles a small program against the reference's own headers,
contracts/cell_store_v1.h (CellStoreView) and contracts/telemetry_v1.h
(Stats), that prints sizeof, alignof and every member's offsetof, and stores
the table. tests/test_contract_layout.py checks include/agb.h's agb_cells and
agb_stats against it with compile-time asserts. Run from the repo root:
python tests/golden/make_layout.py reference_root (or with the reference's
root in AGB_REFERENCE_DIR).
"""
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))

CELL_MEMBERS = ["id", "flags", "death_cause", "x", "y", "z", "vx", "vy", "vz", "energy", "temp_cell",
                "emit_power", "dir_x", "dir_y", "dir_z", "biomass", "co2_held", "age_s", "rng_state",
                "taxis_memory", "run_timer", "t_local", "irradiance", "co2_local", "n2_local", "count", "capacity"]
STATS_MEMBERS = ["tick", "sim_time_s", "n_live", "n_dead", "n_dormant", "n_awake", "n_taumoeba", "mean_charge",
                 "total_energy_j", "mean_temp_cell_k", "mean_temp_medium_k", "max_temp_medium_k", "co2_total_kg",
                 "n2_total_kg", "mean_tau_tolerance", "divisions_this_window", "deaths_this_window", "boil_events",
                 "ignitions_this_window", "physics_rate", "biology_rate", "non_canon_run"]


def program():
    lines = ['#include <cstddef>', '#include <cstdio>', '#include "contracts/cell_store_v1.h"',
             '#include "contracts/telemetry_v1.h"', 'using namespace astro::contract;', 'int main() {']
    for struct, members in (("CellStoreView", CELL_MEMBERS), ("Stats", STATS_MEMBERS)):
        lines.append('  std::printf("%s size %%zu align %%zu\\n", sizeof(%s), alignof(%s));' % (struct, struct, struct))
        for m in members:
            lines.append('  std::printf("%s %s %%zu %%zu\\n", offsetof(%s, %s), sizeof(((%s*)0)->%s));'
                         % (struct, m, struct, m, struct, m))
    lines += ['  return 0;', '}']
    return "\n".join(lines) + "\n"


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("AGB_REFERENCE_DIR", "")
    if not ref:
        sys.exit("usage: make_layout.py reference_root (or set AGB_REFERENCE_DIR)")
    with tempfile.TemporaryDirectory() as tmp:
        src, exe = os.path.join(tmp, "layout.cpp"), os.path.join(tmp, "layout")
        with open(src, "w") as fh:
            fh.write(program())
        subprocess.check_call(["g++", "-std=c++20", "-I" + ref, src, "-o", exe])
        out = subprocess.check_output([exe], text=True)
    table = {}
    for line in out.splitlines():
        parts = line.split()
        if parts[1] == "size":
            table.setdefault(parts[0], {})["__size__"] = int(parts[2])
            table[parts[0]]["__align__"] = int(parts[4])
        else:
            table.setdefault(parts[0], {})[parts[1]] = [int(parts[2]), int(parts[3])]
    table["__source__"] = "contracts/cell_store_v1.h:42-78, contracts/telemetry_v1.h:17-39 (g++ -std=c++20, " \
                          "this machine's ABI: %s)" % os.uname().machine
    with open(os.path.join(HERE, "contract_layout.json"), "w") as fh:
        json.dump(table, fh, indent=1, sort_keys=True)
    print("wrote contract_layout.json")


if __name__ == "__main__":
    main()
