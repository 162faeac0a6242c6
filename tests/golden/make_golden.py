"""Generate tests/golden/ from the REFERENCE itself.

Builds the reference's own src/sim + src/fields sources for the host
(oracle/build_ref.sh, serial CUDA emulation; sources read in place) and runs
every scenario in tests/scenarios.py through its World API, recording a
digest of every array after every stage of every tick, the final Stats, and
for three scenarios the full state after the first tick; and the fields after
each of a list of brush strokes. Run from the repo
root: python tests/golden/make_golden.py reference_root (or with the reference's
root in AGB_REFERENCE_DIR).
"""
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import helpers as H  # noqa: E402
import scenarios as S  # noqa: E402


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("AGB_REFERENCE_DIR", "")
    if not ref_root:
        sys.exit("usage: make_golden.py reference_root (or set AGB_REFERENCE_DIR)")
    subprocess.check_call(["sh", os.path.join(H.ROOT, "oracle", "build_ref.sh"), ref_root])
    full_for = {"slab_uniform", "lifecycle_compaction", "collinear_shadow"}
    for name, sc in S.scenarios().items():
        w = H.RefWorld(sc["desc"])
        rec, full = S.trace(w, sc, full_after=0 if name in full_for else None)
        w.close()
        rec["stats"] = {k: float(v) for k, v in rec["stats"].items()}
        with open(os.path.join(HERE, name + ".json"), "w") as fh:
            json.dump(rec, fh, indent=0, sort_keys=True)
        if full is not None:
            np.savez_compressed(os.path.join(HERE, name + "_tick0.npz"), **full)
        print("golden", name, "count", rec["initial"]["count"], "->", rec["steps"][-1]["cells"]["count"])
    w = H.RefWorld(S.brush_desc())
    with open(os.path.join(HERE, "brushes.json"), "w") as fh:
        json.dump({"brushes": S.brush_trace(w)}, fh, indent=0)
    w.close()
    print("golden brushes")


if __name__ == "__main__":
    main()
