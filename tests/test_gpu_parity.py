"""GPU parity: the sm_103a library against the CPU oracle (FP64).

Bars: max |GPU - oracle| <= 1e-10 of each field's own max|.| (u, v, w floored
at 1e-4 of the velocity scale U = max(|u|,|v|,|w|), p_total on max|p_total|)
after the horizon; the diagnostics of output_diagnostics_3d and
check_divergence_3d (DNS_pressure_BC_3D.f90:2094-2146, 2171-2190) at EVERY
step: kinetic energy, max|u|, max|v|, max|w| within 1e-10 relative (the same
floor), dP/dx within 1e-12, max|div u| within 1e-10 of the velocity scale U
(a velocity gradient: the divergence differentiates the state, so its
round-off is the state's amplified by |D1| ~ nz^2/4 at the wall rows where
the maximum sits, and a bar relative to max|div u| itself, 1e-6..1e-4 U,
would ask for state errors below 1e-20).
"""
import json
import os

import numpy as np
import pytest

from f90_dns_gb300 import ChannelDNS, Dns3DError, config_from
from f90_dns_gb300.capi import DNS3D_E_SINGULAR
from f90_dns_gb300.workloads import WORKLOADS
from oracle import dns3d_ref as ref
from tests.helpers import oracle_config, scaled_velocity_errors, velocity_errors

pytestmark = pytest.mark.gpu

TOL = 1e-10
C1 = WORKLOADS["channel_32x32x33_re180_dpdx"]


def gpu_run(wl, nsteps, stage_api=False, history=False):
    hist = []
    with ChannelDNS(config_from(wl)) as d:
        for _ in range(nsteps if history else 1):
            n = 1 if history else nsteps
            if stage_api:
                for _ in range(n):
                    d.compute_source_terms_3d()
                    d.viscous_step_3d()
                    d.solve_pressure_3d()
                    d.pressure_correction_3d()
                    d.apply_boundary_conditions_3d()
            else:
                d.step(n)
            if history:
                hist.append(d.diagnostics())
        st = d.get_state()
        diag = d.diagnostics()
    return (st, diag, hist) if history else (st, diag)


def oracle_run(wl, nsteps):
    """The oracle's run with its diagnostics and max|div u| at every step."""
    cfg = oracle_config(wl)
    g = ref.setup_grid(cfg)
    st = ref.initial_state(cfg, g)
    hist = []
    for _ in range(nsteps):
        ref.step(cfg, g, st)
        d = ref.diagnostics(cfg, g, st)
        d["max_div"] = ref.max_divergence(g, st)
        hist.append(d)
    return cfg, g, st, hist


def check_history(ghist, hist, tol=TOL, floor=1e-4):
    assert len(ghist) == len(hist)
    for i, (gd, d) in enumerate(zip(ghist, hist)):
        for k in ("umax", "vmax", "wmax", "energy"):
            sc = max(abs(d[k]), floor * d["umax"])
            assert abs(getattr(gd, k) - d[k]) <= tol * sc, (i + 1, k, getattr(gd, k), d[k])
        assert abs(gd.dpdx - d["dpdx"]) <= 1e-12 * max(1.0, abs(d["dpdx"])), (i + 1, gd.dpdx, d["dpdx"])
        assert abs(gd.max_div - d["max_div"]) <= tol * d["umax"], (i + 1, gd.max_div, d["max_div"])


def check(wl, nsteps, tol=TOL):
    gst, gdiag, ghist = gpu_run(wl, nsteps, history=True)
    cfg, g, st, hist = oracle_run(wl, nsteps)
    err = velocity_errors(gst, st)
    assert max(err["u"], err["v"], err["w"]) <= tol, err
    assert err["p_total"] <= tol, err
    check_history(ghist, hist, tol)
    return gst, st, err


def test_c1_50_steps_matches_oracle(built_lib):
    check(C1, 50)


def test_stage_api_equals_fused_step(built_lib):
    a, _ = gpu_run(C1, 5, stage_api=True)
    b, _ = gpu_run(C1, 5, stage_api=False)
    for k in ("u", "v", "w", "p_total", "gpx_w1", "gpy_w2"):
        assert np.array_equal(a[k], b[k]), k


def test_deterministic(built_lib):
    a, _ = gpu_run(C1, 10)
    b, _ = gpu_run(C1, 10)
    for k in ("u", "v", "w", "p_total"):
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("key", ["standard", "weak_form"])
def test_reference_trace(built_lib, key):
    """The reference's own captured run (5 printed digits per step)."""
    with open(os.path.join(os.path.dirname(__file__), "golden", "reference_traces.json")) as f:
        tr = json.load(f)
    p = tr["params"]
    wl = dict(nx=32, ny=32, nz=17, re=500.0, dt=0.002, xlen=2 * ref.PI, ylen=ref.PI, u_centerline=1.5,
              use_crank_nicolson=True, flow_control_method=1, target_pressure_gradient=0.006,
              enable_perturbations=True, use_analytical_perturbations=True, perturbation_amplitude=0.01,
              analytical_mode_x=1, analytical_mode_y=1, use_weak_form_divergence=(key == "weak_form"))
    assert p["nz"] == wl["nz"]
    with ChannelDNS(config_from(wl)) as d:
        d0 = d.diagnostics()
        assert d0.max_div < 1e-13
        for row in tr[key]["steps"]:
            d.step(1)
            dg = d.diagnostics()
            assert dg.step == row["step"]
            for k in ("umax", "vmax", "wmax", "energy", "dpdx"):
                want = row[k]
                assert abs(getattr(dg, k) - want) <= 0.51e-4 * abs(want) + 1e-300, (row["step"], k, getattr(dg, k), want)


@pytest.mark.parametrize("variant", [
    dict(use_dealias_23_rule=False),
    dict(use_weak_form_divergence=True, perturbation_amplitude=0.001),
    dict(use_crank_nicolson=False),
    dict(flow_control_method=2, target_bulk_velocity=2.0 / 3.0, perturbation_amplitude=0.05,
         analytical_mode_x=2),
    dict(flow_control_method=2, target_bulk_velocity=0.7, istart=3),
    dict(analytical_mode_y=0),
])
def test_variants_match_oracle(built_lib, variant):
    wl = dict(C1)
    wl.update(variant)
    if variant.get("use_weak_form_divergence"):
        # the weak-form right-hand side is unstable on perturbed runs (the
        # reference's own weak_form_output.txt grows to |u|max 2.5 in 15
        # steps): round-off is amplified, and two FP64 restatements of the
        # step (numpy, C) already differ by 8.5e-9 of w's own scale after 20
        # steps, so this variant is held to 1e-10 of the velocity scale
        gst, gdiag, ghist = gpu_run(wl, 20, history=True)
        cfg, g, st, hist = oracle_run(wl, 20)
        err = scaled_velocity_errors(gst, st)
        assert max(err["u"], err["v"], err["w"]) <= TOL and err["p_total"] <= TOL, err
        check_history(ghist, hist, floor=1.0)
        return
    check(wl, 20)


@pytest.mark.parametrize("nx,ny,nz", [(48, 96, 17), (96, 48, 25), (64, 32, 33)])
def test_radix3_and_rectangular_grids(built_lib, nx, ny, nz):
    wl = dict(C1, nx=nx, ny=ny, nz=nz, analytical_mode_x=2, analytical_mode_y=1, perturbation_amplitude=0.05)
    check(wl, 10)


@pytest.mark.parametrize("nx,ny", [(16, 12), (32, 24), (96, 48)])
def test_nyquist_content_matches_oracle(built_lib, nx, ny):
    """Random state with energy at kx = nx/2 and ky = ny/2: exercises FFTW's
    c2r treatment of the non-Hermitian derivative spectra (16x12 runs the
    generic transform kernels, the other grids the compile-time ones)."""
    wl = dict(C1, nx=nx, ny=ny, nz=17)
    cfg = oracle_config(wl)
    g = ref.setup_grid(cfg)
    rng = np.random.default_rng(7)
    shp = (g.nz, g.ny, g.nx)
    u, v, w, p = (rng.standard_normal(shp) * s for s in (0.3, 0.2, 0.1, 1.0))
    for a in (u, v, w):
        a[0] = 0.0
        a[-1] = 0.0
    st = ref.initial_state(cfg, g)
    st.u, st.v, st.w, st.p_total = u.copy(), v.copy(), w.copy(), p.copy()
    st.gpx, st.gpy, st.gpz = ref.derivatives(g, p)
    with ChannelDNS(config_from(wl)) as d:
        d.set_state(u=u, v=v, w=w, p_total=p)
        d.step(2)
        gst = d.get_state()
    for _ in range(2):
        ref.step(cfg, g, st)
    err = velocity_errors(gst, st)
    assert max(err["u"], err["v"], err["w"]) <= TOL, err


def test_guarded_dmatrix_is_singular_at_nz65(built_lib):
    wl = dict(C1, nz=65, lgl_dmatrix_guard=True)
    with pytest.raises(Dns3DError) as ei:
        ChannelDNS(config_from(wl))
    assert ei.value.code == DNS3D_E_SINGULAR


def test_unguarded_nz65_matches_oracle(built_lib):
    wl = dict(C1, nx=16, ny=16, nz=65, lgl_dmatrix_guard=False, flow_control_method=2,
              target_bulk_velocity=2.0 / 3.0, perturbation_amplitude=0.05, analytical_mode_x=2)
    check(wl, 10)


def test_state_roundtrip(built_lib):
    wl = dict(C1, nx=32, ny=16, nz=17)
    rng = np.random.default_rng(3)
    shp = (17, 16, 32)
    u = rng.standard_normal(shp)
    with ChannelDNS(config_from(wl)) as d:
        d.set_state(u=u)
        st = d.get_state()
    assert np.max(np.abs(st["u"] - u)) < 1e-13


def test_restart_save_load_continue(built_lib, tmp_path):
    """Save after 6 steps, load into a fresh handle, continue 4 steps; the
    oracle does the same with the reference's restart semantics (grad_p_prev
    not restored, i.e. zero after the restart)."""
    wl = dict(C1, flow_control_method=2, target_bulk_velocity=2.0 / 3.0, nx=32, ny=16, nz=17)
    path = str(tmp_path / "restart.dat")
    with ChannelDNS(config_from(wl)) as d:
        d.step(6)
        d.save_restart(path, 6, 6 * wl["dt"])
    with ChannelDNS(config_from(wl)) as d:
        istep, t = d.load_restart(path)
        assert istep == 6 and abs(t - 6 * wl["dt"]) < 1e-15
        d.step(4)
        gst = d.get_state()
    cfg = oracle_config(wl)
    g = ref.setup_grid(cfg)
    st = ref.initial_state(cfg, g)
    for _ in range(6):
        ref.step(cfg, g, st)
    st.gpx[:] = 0.0
    st.gpy[:] = 0.0
    for _ in range(4):
        ref.step(cfg, g, st)
    err = velocity_errors(gst, st)
    assert max(err["u"], err["v"], err["w"]) <= TOL, err


def test_cached_physical_fields_stay_coherent(built_lib):
    """get_state and diagnostics share the physical fields they transform;
    every state change (graph steps, stage calls, set_state) must drop them."""
    wl = dict(C1, nx=32, ny=24, nz=17)
    with ChannelDNS(config_from(wl)) as d, ChannelDNS(config_from(wl)) as e:
        d.step(3)
        a = d.diagnostics()
        s1 = d.get_state()
        assert d.diagnostics() == a
        d.step(2)
        d.compute_source_terms_3d()
        d.viscous_step_3d()
        d.solve_pressure_3d()
        d.pressure_correction_3d()
        d.apply_boundary_conditions_3d()
        c = d.diagnostics()
        s2 = d.get_state()
        e.step(6)
        se = e.get_state()
        for k in ("u", "v", "w", "p_total"):
            np.testing.assert_array_equal(s2[k], se[k])
        ce = e.diagnostics()
        for k in ("umax", "vmax", "wmax", "energy", "max_div"):
            assert getattr(c, k) == getattr(ce, k), k
        d.set_state(u=s1["u"], v=s1["v"], w=s1["w"], p_total=s1["p_total"])
        b = d.diagnostics()
        for k in ("umax", "vmax", "wmax", "energy"):
            assert abs(getattr(b, k) - getattr(a, k)) <= 1e-13 * abs(getattr(a, k)), k


def test_taylor_green_divergence_on_device(built_lib):
    """test_taylor_green_divergence.f90:64-145 on the library: the divergence
    diagnostic of a w = 0 Taylor-Green field (spectral dx, dy, LGL dz) is
    below 1e-12."""
    wl = dict(C1, nx=32, ny=32, nz=17, xlen=2 * ref.PI, ylen=2 * ref.PI, enable_perturbations=False)
    cfg = oracle_config(wl)
    g = ref.setup_grid(cfg)
    x = np.arange(g.nx) * g.xlen / g.nx
    y = np.arange(g.ny) * g.ylen / g.ny
    cz = np.cos(np.pi * g.zpts / 2.0)
    u = 0.1 * np.sin(x)[None, None, :] * np.cos(y)[None, :, None] * cz[:, None, None]
    v = -0.1 * np.cos(x)[None, None, :] * np.sin(y)[None, :, None] * cz[:, None, None]
    with ChannelDNS(config_from(wl)) as d:
        d.set_state(u=u, v=v, w=np.zeros_like(u))
        assert d.diagnostics().max_div < 1e-12


def test_nonfinite_state_is_reported(built_lib):
    """A NaN in a host buffer handed to set_state makes the diagnostics return
    DNS3D_E_NONFINITE (a status, not a fault); the handle stays usable."""
    from f90_dns_gb300.capi import DNS3D_E_NONFINITE
    wl = dict(C1, nx=32, ny=16, nz=17)
    with ChannelDNS(config_from(wl)) as d:
        st = d.get_state()
        bad = st["u"].copy()
        bad[5, 3, 7] = np.nan
        d.set_state(u=bad)
        with pytest.raises(Dns3DError) as ei:
            d.diagnostics()
        assert ei.value.code == DNS3D_E_NONFINITE
        d.set_state(u=st["u"])
        d.step(2)
        assert np.isfinite(d.diagnostics().energy)


def test_nonfinite_state_survives_a_step_of_the_integer_kernels(built_lib, monkeypatch):
    """With the tensor-core and fixed-point forms forced, a NaN in the state is
    still non-finite after a step (the emulated products and the fixed-point
    Poisson solve do not turn it into finite values): the diagnostics report
    DNS3D_E_NONFINITE."""
    from f90_dns_gb300.capi import DNS3D_E_NONFINITE
    monkeypatch.setenv("DNS3D_TENSOR_CORES", "1")
    wl = dict(C1, nx=32, ny=16, nz=17)
    with ChannelDNS(config_from(wl)) as d:
        st = d.get_state()
        bad = st["w"].copy()
        bad[6, 3, 7] = np.nan
        d.set_state(w=bad)
        d.step(1)
        with pytest.raises(Dns3DError) as ei:
            d.diagnostics()
        assert ei.value.code == DNS3D_E_NONFINITE


def test_split_diagnostics_match_combined(built_lib):
    """dns3d_output_diagnostics and dns3d_check_divergence (the reference's
    output_diagnostics_3d and check_divergence_3d, called on their own
    schedules) give exactly what dns3d_diagnostics gives in one call."""
    wl = dict(C1, nx=32, ny=24, nz=17)
    with ChannelDNS(config_from(wl)) as d:
        d.step(3)
        full = d.diagnostics()
        out = d.output_diagnostics_3d()
        div = d.check_divergence_3d()
    assert out.max_div == 0.0 and div == full.max_div
    for k in ("umax", "vmax", "wmax", "energy", "u_bulk", "dpdx", "dpdx_avg", "time", "step"):
        assert getattr(out, k) == getattr(full, k), k
