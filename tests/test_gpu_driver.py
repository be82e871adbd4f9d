"""GPU: the C++ driver (the reference's time loop over the C-ABI) reproduces
the reference's own captured stdout of the same runs, line by line."""
import json
import os
import re
import subprocess

import pytest

from f90_dns_gb300 import build

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
LINE = re.compile(r"Step\s+(\d+), t=\s*([0-9.]+), \|u\|max=\s*(\S+), \|v\|max=\s*(\S+), \|w\|max=\s*(\S+), "
                  r"E=\s*(\S+), dP/dx=\s*([0-9.Ee+-]+)")


@pytest.mark.parametrize("key", ["standard", "weak_form"])
def test_driver_prints_reference_trace(built_lib, key):
    inp = os.path.join(HERE, "golden", f"input_trace_32x32x17_{key}.dat")
    env = dict(os.environ, DNS3D_OUTPUT_DIR="none")  # stdout only; the files are tested elsewhere
    res = subprocess.run([build.RUNNER, inp], capture_output=True, text=True, timeout=300, env=env)
    assert res.returncode == 0, res.stderr
    got = [m.groups() for m in map(LINE.search, res.stdout.splitlines()) if m]
    with open(os.path.join(HERE, "golden", "reference_traces.json")) as f:
        want = json.load(f)[key]["steps"]
    assert len(got) == len(want) == 15
    for g, w in zip(got, want):
        assert int(g[0]) == w["step"] and abs(float(g[1]) - w["time"]) < 1e-9
        for val, k in zip(g[2:], ("umax", "vmax", "wmax", "energy", "dpdx")):
            assert abs(float(val) - w[k]) <= 0.51e-4 * abs(w[k]), (w["step"], k, val, w[k])
    assert "Step      0, Max divergence:" in res.stdout


def test_driver_rejects_bad_input(built_lib, tmp_path):
    bad = tmp_path / "bad.dat"
    bad.write_text("&grid\n nx_input = 100, ny_input = 32, nz_input = 17\n/\n")
    res = subprocess.run([build.RUNNER, str(bad)], capture_output=True, text=True, timeout=120,
                         env=dict(os.environ, DNS3D_OUTPUT_DIR="none"))
    assert res.returncode == 1
    assert "unsupported grid size" in res.stderr
