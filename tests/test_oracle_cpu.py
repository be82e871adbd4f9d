"""CPU: the C/OpenMP restatement of the reference step (oracle/dns3d_cpu.c), the
CPU baseline of bench.py, pinned to the reference's captured runs and to the
numpy restatement.

  * its FFTs reproduce FFTW's r2c and non-Hermitian c2r conventions (numpy's
    pocketfft has the same ones) to round-off;
  * its 15-step runs reproduce the reference's printed trace (standard and
    weak-form pressure; 5 printed digits);
  * its steps agree with the numpy restatement to round-off (1e-12 of the
    velocity scale over 20 steps; the weak form, unstable in the reference
    too, to 1e-10), for dealiased / not, CN / implicit, constant forcing / PI.
"""
import json
import os

import numpy as np
import pytest

from oracle import cpu_ref
from oracle import dns3d_ref as ref
from tests.test_oracle_pins import GOLD, trace_config


@pytest.mark.parametrize("nx,ny", [(8, 6), (32, 32), (48, 96), (24, 12), (6, 4), (96, 48)])
def test_fft_conventions(nx, ny):
    rng = np.random.default_rng(nx * 1000 + ny)
    f = rng.standard_normal((ny, nx))
    F = cpu_ref.r2c_plane(f)
    R = np.fft.rfft2(f)
    assert np.max(np.abs(F - R)) <= 1e-14 * np.max(np.abs(R))
    # non-Hermitian input: the c2r ignores Im at kx = 0 and kx = nx/2
    G = rng.standard_normal((ny, nx // 2 + 1)) + 1j * rng.standard_normal((ny, nx // 2 + 1))
    g = cpu_ref.c2r_plane(G, nx)
    r = np.fft.irfft2(G, s=(ny, nx))
    assert np.max(np.abs(g - r)) <= 1e-14 * np.max(np.abs(r))


@pytest.mark.parametrize("key,weak", [("standard", False), ("weak_form", True)])
def test_reproduces_reference_trace(key, weak):
    with open(GOLD) as f:
        tr = json.load(f)[key]
    with cpu_ref.CpuChannel(trace_config(weak), threads=2) as c:
        for row in tr["steps"]:
            c.step(1)
            d = c.diagnostics()
            for k in ("umax", "vmax", "wmax", "energy", "dpdx"):
                assert abs(d[k] - row[k]) <= 0.51e-4 * abs(row[k]), (row["step"], k, d[k], row[k])


CASES = [
    ("dealias_dpdx", dict(nx=32, ny=32, nz=33, re=180.0, dt=0.002, xlen=4 * ref.PI, ylen=2 * ref.PI,
                          u_centerline=1.0, flow_control_method=1, target_pressure_gradient=2 / 180,
                          enable_perturbations=True, use_analytical_perturbations=True,
                          perturbation_amplitude=0.01, use_dealias_23_rule=True), 1e-12),
    ("pi_control", dict(nx=32, ny=24, nz=17, re=180.0, dt=0.002, xlen=4 * ref.PI, ylen=2 * ref.PI,
                        u_centerline=1.0, flow_control_method=2, target_bulk_velocity=2 / 3,
                        enable_perturbations=True, use_analytical_perturbations=True,
                        perturbation_amplitude=0.05, analytical_mode_x=2, use_dealias_23_rule=True), 1e-12),
    ("implicit_euler", dict(nx=24, ny=48, nz=17, re=300.0, dt=0.002, use_crank_nicolson=False,
                            enable_perturbations=True, use_analytical_perturbations=True,
                            perturbation_amplitude=0.02, analytical_mode_y=2), 1e-12),
    ("weak_form", dict(nx=32, ny=32, nz=17, re=500.0, dt=0.002, u_centerline=1.5, target_pressure_gradient=0.006,
                       enable_perturbations=True, use_analytical_perturbations=True,
                       perturbation_amplitude=0.01, use_weak_form_divergence=True), 1e-10),
]


@pytest.mark.parametrize("name,kw,tol", CASES, ids=[c[0] for c in CASES])
def test_matches_numpy_restatement(name, kw, tol):
    cfg = ref.Config(**kw)
    g = ref.setup_grid(cfg)
    st = ref.initial_state(cfg, g)
    with cpu_ref.CpuChannel(cfg, threads=4) as c:
        s0 = c.get_state()
        for k in ("u", "v", "w"):
            np.testing.assert_array_equal(s0[k], getattr(st, k))
        for _ in range(20):
            ref.step(cfg, g, st)
        c.step(20)
        s = c.get_state()
        d = c.diagnostics()
    scale = max(np.max(np.abs(st.u)), np.max(np.abs(st.v)), np.max(np.abs(st.w)))
    for k in ("u", "v", "w"):
        assert np.max(np.abs(s[k] - getattr(st, k))) <= tol * scale, k
    assert np.max(np.abs(s["p_total"] - st.p_total)) <= tol * 10 * np.max(np.abs(st.p_total))
    dr = ref.diagnostics(cfg, g, st)
    assert abs(d["dpdx"] - dr["dpdx"]) <= 1e-13
    assert abs(d["energy"] - dr["energy"]) <= tol * dr["energy"]
    assert abs(d["max_div"] - ref.max_divergence(g, st)) <= 1e-9 * max(1.0, d["max_div"])


def test_thread_count_does_not_change_results():
    cfg = ref.Config(**CASES[1][1])
    out = []
    for th in (1, 3):
        with cpu_ref.CpuChannel(cfg, threads=th) as c:
            c.step(5)
            out.append(c.get_state())
    for k in ("u", "v", "w", "p_total"):
        np.testing.assert_array_equal(out[0][k], out[1][k])
