"""The deposit flush's fixed-point -> float conversion (fixed_to_f,
astrophage-microscope_gb300/csrc/dev.cuh) equals the reference's
(float)((double)raw / scale) bit for bit: its C restatement
(tests/csrc/fixed_to_f_check.c) against the double division, on random
deposits and on deposits next to rounding midpoints, at the temperature,
CO2/N2 and irradiance scales. On the GPU the same conversion is checked
through the CO2 field (tests/test_gpu_rationing.py)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_fixed_to_f_equals_double_division(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = tmp_path / "fixed_to_f_check"
    subprocess.run([cc, "-O2", "-ffp-contract=off", "-o", str(exe), os.path.join(HERE, "csrc", "fixed_to_f_check.c"),
                    "-lm"], check=True)
    r = subprocess.run([str(exe), "1000000", "1000000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    words = r.stdout.split()
    checked, bad, fallbacks = int(words[1]), int(words[3]), int(words[5])
    assert bad == 0 and checked > 4000000
    assert fallbacks < checked // 4            # the FP64 path stays the exception
