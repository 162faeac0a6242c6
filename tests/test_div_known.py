"""Division by a divisor known ahead (div_known,
astrophage-microscope_gb300/csrc/dev.cuh), used for the CO2 rationing's
divisions by the voxel volume and the deposit scale: Markstein's correction
step on a reciprocal computed on the host, returned only where an exact
half-ulp residual test proves it is the correctly rounded quotient, else the
IEEE division. Its C restatement (tests/csrc/div_known_check.c) must equal
a / b bit for bit on random dividends and on dividends whose quotients sit
next to rounding midpoints, for the benchmark grids' voxel volumes, the
deposit scales and random divisors. On the GPU the same divisions are checked
through the CO2 state against the oracle (tests/test_gpu_rationing.py)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_div_known_equals_ieee_division(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = tmp_path / "div_known_check"
    subprocess.run([cc, "-O2", "-ffp-contract=off", "-o", str(exe), os.path.join(HERE, "csrc", "div_known_check.c"),
                    "-lm"], check=True)
    r = subprocess.run([str(exe), "200000", "200000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    words = r.stdout.split()
    checked, bad, fallbacks = int(words[1]), int(words[3]), int(words[5])
    assert bad == 0 and checked >= 16000000
    assert fallbacks < checked // 100          # the IEEE division stays the exception
