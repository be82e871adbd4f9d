"""CPU: the output-file writers (write_time_series_data, write_flow_statistics,
write_spanwise_averaged_profile, write_velocity_field_snapshot,
write_simulation_summary of DNS_pressure_BC_3D.f90:2594-2952) produce the
reference's text, character for character, against the oracle's restatement
of the Fortran edit descriptors.  No GPU: these are host functions."""
import math
import os

import numpy as np
import pytest

from f90_dns_gb300 import capi
from oracle import dns3d_ref as ref

EDGE = [0.0, 1.0, -1.0, 2.5e-8, -3.7e-3, 9.9999995, 0.99999995, 123456.75, 1e-120, -3.2e150, 5e-324,
        1.7976931348623157e308, float("nan"), float("inf"), -float("inf")]


def _stats(rng, method, values=None):
    names = [n for n, _ in capi.CFlowStats._fields_ if n not in ("step", "flow_control_method")]
    vals = values if values is not None else rng.standard_normal(len(names)) * 10.0 ** rng.integers(-9, 4, len(names))
    d = dict(zip(names, (float(v) for v in vals)))
    d["step"] = int(rng.integers(0, 10 ** 6))
    d["flow_control_method"] = method
    return d


def test_fortran_edit_descriptors_pinned():
    # gfortran renderings of ES15.6 / F12.6, written out from the standard's rules
    assert ref.fortran_es(1.0, 15, 6) == "   1.000000E+00"
    assert ref.fortran_es(-3.7e-3, 15, 6) == "  -3.700000E-03"
    assert ref.fortran_es(9.9999999e9, 15, 6) == "   1.000000E+10"
    assert ref.fortran_es(1e-120, 15, 6) == "   1.000000-120"
    assert ref.fortran_es(float("inf"), 15, 6) == "       Infinity"
    assert ref.fortran_f(0.002, 12, 6) == "    0.002000"
    assert ref.fortran_f(123456.75, 12, 6) == "*" * 12


@pytest.mark.parametrize("method", [1, 2])
def test_time_series_and_statistics_text(tmp_path, method):
    rng = np.random.default_rng(7 + method)
    d = str(tmp_path)
    capi.output_init(d)
    rows = []
    for i in range(40):
        st = _stats(rng, method)
        capi.output_time_series_row(d, st)
        rows.append(ref.time_series_row(st))
    for v in EDGE:
        st = _stats(rng, method, [v] * 12)
        capi.output_time_series_row(d, st)
        rows.append(ref.time_series_row(st))
    got = open(os.path.join(d, "output_time_series.dat")).read().splitlines()
    assert got[:2] == ["# DNS 3D Time Series Data",
                       "# Columns: step, time, u_max, v_max, w_max, energy, pressure_gradient, bulk_velocity"]
    assert got[2:] == rows
    assert all(len(r) == 8 + 15 * (7 if method == 2 else 6) for r in rows)
    st = _stats(rng, method)
    capi.output_flow_statistics(d, st)
    assert open(os.path.join(d, "flow_statistics.dat")).read() == ref.flow_statistics_text(st)


def test_time_series_needs_initialised_file(tmp_path):
    with pytest.raises(capi.Dns3DError) as e:
        capi.output_time_series_row(str(tmp_path), _stats(np.random.default_rng(0), 1))
    assert e.value.code == capi.DNS3D_E_IO


def test_profile_and_snapshot_text(tmp_path):
    rng = np.random.default_rng(3)
    nx, ny, nz = 6, 4, 5
    z, _ = capi.lgl_nodes_weights(nz)
    prof = [rng.standard_normal(nz) for _ in range(3)]
    capi.output_spanwise_profile(str(tmp_path), 120, 0.24, z, *prof)
    got = open(tmp_path / "spanwise_profile_00120.dat").read()
    assert got == ref.spanwise_profile_text(120, 0.24, z, *prof)
    u, v, w = (rng.standard_normal((nz, ny, nx)) for _ in range(3))
    u[0] = 0.0
    capi.output_velocity_snapshot(str(tmp_path), 7, 0.014, 4.0 * math.pi, 2.0 * math.pi, z, u, v, w)
    got = open(tmp_path / "velocity_field_00007.dat").read()
    assert got == ref.velocity_snapshot_text(7, 0.014, 4.0 * math.pi, 2.0 * math.pi, z, u, v, w)
    assert len(got.splitlines()) == 4 + nx * ny * nz


def test_lgl_nodes_match_oracle():
    for nz in (17, 33, 65, 129):
        z, w = capi.lgl_nodes_weights(nz)
        zr, wr = ref.lgl_nodes_weights(nz)
        np.testing.assert_array_equal(z, zr)
        np.testing.assert_array_equal(w, wr)


@pytest.mark.parametrize("method", [1, 2])
def test_simulation_summary(tmp_path, method):
    cfg = capi.default_config(nx=32, ny=32, nz=17, re=500.0, dt=0.002, nsteps=15, nwrt=1,
                              flow_control_method=method, target_bulk_velocity=0.6667)
    capi.output_simulation_summary(str(tmp_path), cfg, "input_3d.dat", restarted=(method == 2),
                                   restart_step=40, restart_time=0.08)
    lines = open(tmp_path / "simulation_summary.txt").read().splitlines()
    assert lines[0] == lines[2] == lines[-1] == "=" * 44
    assert " Input file: input_3d.dat" in lines
    assert "   Grid size: 32 × 32 × 17" in lines
    assert "   Domain Lz:   2.0000" in lines
    assert "   Reynolds number:   500.0000" in lines
    assert "   Time step:   0.002000" in lines
    assert "   Total time:     0.0300" in lines
    assert ("   Target bulk velocity:   0.666700" in lines) == (method == 2)
    if method == 2:
        assert "   Restart mode: ENABLED (restarting from checkpoint)" in lines
        assert "   Restart time:     0.080000" in lines
    else:
        assert "   Restart mode: DISABLED (new simulation)" in lines


def test_es_format_property():
    """Property check over random doubles of all magnitudes: the writer's
    ES15.6 text equals the oracle's, reads back within half a unit in the
    sixth decimal, and is always 15 characters."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies

    @hyp.settings(max_examples=300, deadline=None)
    @hyp.given(st.floats(allow_nan=False, allow_infinity=False, width=64))
    def check(v):
        s = _stats(np.random.default_rng(0), 1, [v] * 12)
        d = capi.CFlowStats()
        for n, _ in capi.CFlowStats._fields_:
            setattr(d, n, s[n])
        import tempfile
        with tempfile.TemporaryDirectory() as td:
            capi.output_init(td)
            capi.output_time_series_row(td, d)
            row = open(os.path.join(td, "output_time_series.dat")).read().splitlines()[2]
        assert row == ref.time_series_row(s)
        field = ref.fortran_es(v, 15, 6)
        assert len(field) == 15
        if "*" not in field and abs(v) >= 1e-99 and abs(v) < 1e99:
            back = float(field)
            assert abs(back - v) <= 0.5e-6 * abs(v) * 10 + 1e-300

    check()
