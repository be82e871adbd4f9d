"""GPU: flow statistics reduced on the device (dns3d_flow_statistics) and the
output files written from a handle and by the driver, against the oracle's
restatement of write_time_series_data / write_flow_statistics /
write_spanwise_averaged_profile / write_velocity_field_snapshot
(DNS_pressure_BC_3D.f90:2702-2952)."""
import os
import subprocess

import numpy as np
import pytest

from f90_dns_gb300 import ChannelDNS, build, capi, config_from
from f90_dns_gb300.workloads import WORKLOADS
from oracle import dns3d_ref as ref
from tests.helpers import oracle_config

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
C1 = WORKLOADS["channel_32x32x33_re180_dpdx"]
PI_SMALL = dict(C1, nx=32, ny=24, nz=17, flow_control_method=2, target_bulk_velocity=2.0 / 3.0,
                perturbation_amplitude=0.05, analytical_mode_x=2)
TOL = 1e-10


def _runs(wl, nsteps):
    d = ChannelDNS(config_from(wl))
    d.step(nsteps)
    cfg = oracle_config(wl)
    g, st, _ = ref.run(cfg, nsteps, record_every=nsteps)
    return d, cfg, g, st


@pytest.mark.parametrize("wl", [C1, PI_SMALL], ids=["dpdx", "pi"])
def test_flow_statistics_match_oracle(built_lib, wl):
    d, cfg, g, st = _runs(wl, 20)
    with d:
        got = d.flow_statistics(profiles=True)
    want = ref.flow_statistics(cfg, g, st)
    vs = want["umax"]
    shear = vs / cfg.re / float(g.zpts[1] - g.zpts[0])
    scale = dict(umax=vs, vmax=vs, wmax=vs, energy=want["energy"], bulk_velocity=vs, dpdx=abs(want["dpdx"]) + 1e-3,
                 dpdx_avg=abs(want["dpdx_avg"]) + 1e-3, wall_shear_lower=shear, wall_shear_upper=shear,
                 friction_velocity_avg=want["friction_velocity_avg"], re_tau=want["re_tau"], time=1.0)
    for k, s in scale.items():
        assert abs(got[k] - want[k]) <= TOL * s, (k, got[k], want[k])
    assert got["step"] == want["step"] == 20
    assert got["flow_control_method"] == cfg.flow_control_method
    for a, b in zip((got["u_avg"], got["v_avg"], got["w_avg"]), ref.spanwise_profile(g, st)):
        assert np.max(np.abs(a - b)) <= TOL * vs
    assert abs(got["wall_shear_lower"]) > 0 and got["re_tau"] > 0


def _same_text(path, want_text, rel=2e-6, floor=1e-13):
    """Token by token: words equal, numbers within the last printed digit
    (values at round-off level, below `floor`, only to within `floor`)."""
    got = open(path).read().splitlines()
    want = want_text.splitlines()
    assert len(got) == len(want)
    for gl, wl_ in zip(got, want):
        assert len(gl) == len(wl_), (gl, wl_)
        for a, b in zip(gl.split(), wl_.split()):
            try:
                fa, fb = float(a), float(b)
            except ValueError:
                assert a == b, (gl, wl_)
                continue
            assert abs(fa - fb) <= rel * abs(fb) + floor, (gl, wl_)


@pytest.mark.parametrize("wl", [C1, PI_SMALL], ids=["dpdx", "pi"])
def test_handle_writers_match_oracle_text(built_lib, tmp_path, wl):
    out = str(tmp_path)
    capi.output_init(out)
    cfg = oracle_config(wl)
    g = ref.setup_grid(cfg)
    st = ref.initial_state(cfg, g)
    rows = []
    with ChannelDNS(config_from(wl)) as d:
        for _ in range(3):
            d.step(5)
            for _ in range(5):
                ref.step(cfg, g, st)
            d.write_time_series_data(out)
            rows.append(ref.time_series_row(ref.flow_statistics(cfg, g, st)))
        d.write_flow_statistics(out)
        d.write_spanwise_averaged_profile(out)
        d.write_velocity_field_snapshot(out)
    s = ref.flow_statistics(cfg, g, st)
    head = "# DNS 3D Time Series Data\n# Columns: step, time, u_max, v_max, w_max, energy, pressure_gradient, " \
           "bulk_velocity\n"
    _same_text(tmp_path / "output_time_series.dat", head + "\n".join(rows) + "\n")
    _same_text(tmp_path / "flow_statistics.dat", ref.flow_statistics_text(s))
    _same_text(tmp_path / "spanwise_profile_00015.dat",
               ref.spanwise_profile_text(15, st.time, g.zpts, *ref.spanwise_profile(g, st)))
    _same_text(tmp_path / "velocity_field_00015.dat",
               ref.velocity_snapshot_text(15, st.time, g.xlen, g.ylen, g.zpts, st.u, st.v, st.w))


def test_driver_writes_reference_output_files(built_lib, tmp_path):
    inp = os.path.join(HERE, "golden", "input_trace_32x32x17_standard.dat")
    env = dict(os.environ, DNS3D_OUTPUT_DIR=str(tmp_path / "out"))
    res = subprocess.run([build.RUNNER, inp], capture_output=True, text=True, timeout=300, env=env)
    assert res.returncode == 0, res.stderr
    out = tmp_path / "out"
    names = sorted(os.listdir(out))
    assert names == ["flow_statistics.dat", "output_time_series.dat", "restart.dat", "simulation_summary.txt",
                     "spanwise_profile_00010.dat", "velocity_field_00010.dat"]
    rows = [ln.split() for ln in open(out / "output_time_series.dat").read().splitlines()[2:]]
    assert [int(r[0]) for r in rows] == list(range(1, 16))
    # the time series carries the same numbers as the printed diagnostics lines
    printed = [ln for ln in res.stdout.splitlines() if "|u|max=" in ln]
    assert len(printed) == 15
    for r, ln in zip(rows, printed):
        umax = float(ln.split("|u|max=")[1].split(",")[0])
        assert abs(float(r[2]) - umax) <= 1e-4 * umax
    rst = capi.restart_read(str(out / "restart.dat"), 32, 32, 17)
    assert rst["istep"] == 15 and abs(rst["time"] - 15 * 0.002) < 1e-12
    assert len(open(out / "velocity_field_00010.dat").read().splitlines()) == 4 + 32 * 32 * 17
