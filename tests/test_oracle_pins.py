"""CPU: pin the oracle to the reference's own captured runs and known answers.

The oracle (oracle/dns3d_ref.py) restates DNS_pressure_BC_3D.f90; before it is
trusted as the parity checker it must reproduce
  * the reference's captured stdout of two real 3D runs (standard_output.txt,
    weak_form_output.txt: 32x32x17, Re 500, 15 steps; 5 printed digits), and
  * the analytic checks of the reference's test programs.
"""
import json
import math
import os

import numpy as np
import pytest

from oracle import dns3d_ref as ref

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_traces.json")


def trace_config(weak: bool, dealias: bool = False) -> ref.Config:
    return ref.Config(nx=32, ny=32, nz=17, dt=0.002, re=500.0, xlen=2 * ref.PI, ylen=ref.PI,
                      u_centerline=1.5, use_crank_nicolson=True, flow_control_method=1,
                      target_pressure_gradient=0.006, enable_perturbations=True,
                      use_analytical_perturbations=True, perturbation_amplitude=0.01,
                      analytical_mode_x=1, analytical_mode_y=1, use_weak_form_divergence=weak,
                      use_dealias_23_rule=dealias)


@pytest.mark.parametrize("key,weak", [("standard", False), ("weak_form", True)])
def test_oracle_reproduces_reference_trace(key, weak):
    with open(GOLD) as f:
        tr = json.load(f)[key]
    g, st, hist = ref.run(trace_config(weak), 15)
    assert len(hist) == len(tr["steps"]) == 15
    for h, row in zip(hist, tr["steps"]):
        assert h["step"] == row["step"]
        for k in ("umax", "vmax", "wmax", "energy", "dpdx"):
            assert abs(h[k] - row[k]) <= 0.51e-4 * abs(row[k]), (row["step"], k, h[k], row[k])
    # "Step 0, Max divergence: 0.3044E-14" (check_divergence_3d at 3D:206)
    g = ref.setup_grid(trace_config(weak))
    st0 = ref.initial_state(trace_config(weak), g)
    assert ref.max_divergence(g, st0) < 1e-13


def test_trace_insensitive_to_dealias_flag():
    """use_dealias_23_rule is not logged in the captured runs; both settings
    reproduce the trace (the (1,1) perturbation has no filtered content)."""
    with open(GOLD) as f:
        tr = json.load(f)["standard"]
    _, _, hist = ref.run(trace_config(False, dealias=True), 15)
    row, h = tr["steps"][-1], hist[-1]
    for k in ("umax", "vmax", "wmax", "energy"):
        assert abs(h[k] - row[k]) <= 0.51e-4 * abs(row[k])


def test_d2_poiseuille_known_answer():
    """debug_flow_analysis.f90:60-66: d2 . 1.5(1-z^2) = -3 at nz = 33."""
    cfg = ref.Config(nx=8, ny=8, nz=33)
    g = ref.setup_grid(cfg)
    assert np.max(np.abs(g.d2 @ (1.5 * (1 - g.zpts ** 2)) + 3.0)) < 1e-9


def test_lgl_nodes_weights():
    for n in (9, 17, 33, 49):
        x, w = ref.lgl_nodes_weights(n)
        assert x[0] == -1.0 and x[-1] == 1.0
        assert abs(w.sum() - 2.0) < 1e-13
        assert np.max(np.abs(x + x[::-1])) < 1e-14
        # exact for polynomials up to degree 2n-3
        assert abs(np.sum(w * x ** (2 * n - 4)) - 2.0 / (2 * n - 3)) < 1e-12


def test_spectral_integration_known_answer():
    """Known answer of test_spectral_integration.f90:32-66 (dw/dz = -sin(pi z),
    exact w = (cos(pi z) + 1)/pi).  The reference program replaces both end rows
    of D and calls a node routine lgl_module does not have, so it never ran; the
    well-posed form keeps one boundary row, w(-1) = 0, and converges spectrally."""
    for n, tol in ((9, 1e-3), (17, 1e-10), (33, 1e-13)):
        x, _ = ref.lgl_nodes_weights(n)
        A = ref.differentiation_matrix(x)
        A[0] = 0.0
        A[0, 0] = 1.0
        b = -np.sin(np.pi * x)
        b[0] = 0.0
        sol = np.linalg.solve(A, b)
        exact = (np.cos(np.pi * x) + 1.0) / np.pi
        assert np.max(np.abs(sol - exact)) < tol, n


def test_taylor_green_divergence_known_answer():
    """test_taylor_green_divergence.f90:64-145: spectral dx, dy + LGL dz of a
    w = 0 Taylor-Green field give max |div| < 1e-12."""
    cfg = ref.Config(nx=32, ny=32, nz=17, xlen=2 * ref.PI, ylen=2 * ref.PI)
    g = ref.setup_grid(cfg)
    x = np.arange(g.nx) * g.xlen / g.nx
    y = np.arange(g.ny) * g.ylen / g.ny
    cz = np.cos(np.pi * g.zpts / 2.0)
    u = 0.1 * np.sin(x)[None, None, :] * np.cos(y)[None, :, None] * cz[:, None, None]
    v = -0.1 * np.cos(x)[None, None, :] * np.sin(y)[None, :, None] * cz[:, None, None]
    w = np.zeros_like(u)
    assert np.max(np.abs(ref.divergence(g, u, v, w))) < 1e-12


def test_fft_roundtrip_known_answer():
    """test_fft_roundtrip (3D:2002-2069): r2c then c2r per plane, error < 1e-12."""
    cfg = ref.Config(nx=32, ny=24, nz=9, xlen=2 * ref.PI, ylen=2 * ref.PI)
    g = ref.setup_grid(cfg)
    x = np.arange(g.nx) * g.xlen / g.nx
    y = np.arange(g.ny) * g.ylen / g.ny
    f = (np.sin(2 * g.alpha * x)[None, None, :] * np.cos(3 * g.beta * y)[None, :, None]
         * (1 - g.zpts ** 2)[:, None, None])
    assert np.max(np.abs(ref.c2r(ref.r2c(f), g.nx, g.ny) - f)) < 1e-12


def test_c2r_nonhermitian_semantics():
    """c2r of non-Hermitian data: Im of the kx=0 and kx=nx/2 entries is ignored
    (the behaviour the derivative Nyquist rules rely on)."""
    rng = np.random.default_rng(1)
    nx, ny = 8, 6
    F = rng.standard_normal((ny, nx // 2 + 1)) + 1j * rng.standard_normal((ny, nx // 2 + 1))
    out = ref.c2r(F, nx, ny)
    # explicit definition: ifft along y, then 1D c2r with Re-only ends
    G = np.fft.ifft(F, axis=0)
    expect = np.empty((ny, nx))
    n = np.arange(nx)
    for j in range(ny):
        row = G[j].real[0] + ((-1.0) ** n) * G[j].real[nx // 2]
        for k in range(1, nx // 2):
            row = row + 2 * np.real(G[j, k] * np.exp(2j * np.pi * k * n / nx))
        expect[j] = row / nx
    assert np.max(np.abs(out - expect)) < 1e-14


def test_poiseuille_energy_and_fixed_point():
    """E = 0.6 for u = 1.5(1-z^2) (DNS_Enhancement notebook), and with forcing
    2 u_c/Re the laminar profile is a fixed point of the step."""
    cfg = ref.Config(nx=16, ny=8, nz=33, dt=0.01, re=180.0, u_centerline=1.5,
                     target_pressure_gradient=3.0 / 180.0)
    g = ref.setup_grid(cfg)
    st = ref.initial_state(cfg, g)
    d = ref.diagnostics(cfg, g, st)
    assert abs(d["energy"] - 0.6) < 1e-12
    u0 = st.u.copy()
    for _ in range(5):
        ref.step(cfg, g, st)
    assert np.max(np.abs(st.u - u0)) < 1e-11
    assert np.max(np.abs(st.v)) < 1e-13 and np.max(np.abs(st.w)) < 1e-13


def test_dealias_limits():
    """kx_max = ((nx/2)*2)/3, ky_max = ((ny/2)*2)/3 in integer arithmetic (3D:1169-1170)."""
    for n, kmax in ((32, 10), (48, 16), (64, 21), (96, 32), (128, 42), (256, 85), (384, 128), (512, 170)):
        g = ref.setup_grid(ref.Config(nx=n, ny=n, nz=5))
        keep = ref.dealias_mask(g)
        assert keep[0, kmax] and not keep[0, kmax + 1]
        assert keep[kmax, 0] and not keep[kmax + 1, 0]
        assert keep[n - kmax, 0] and not keep[n - kmax - 1, 0]


def test_dmatrix_guard_degenerates_at_nz58():
    """lgl_module.f90:247-251 zeroes D entries whose denominator is <= 1e-15;
    from nz = 58 on that removes off-diagonal entries and the reference's pinned
    Poisson mode becomes singular (zgesv info /= 0 -> stop)."""
    x, _ = ref.lgl_nodes_weights(57)
    assert np.count_nonzero(ref.differentiation_matrix(x) == 0.0) == 0
    x, _ = ref.lgl_nodes_weights(65)
    D = ref.differentiation_matrix(x)
    assert np.count_nonzero(D - np.diag(np.diag(D))) == 0
    cfg = ref.Config(nx=8, ny=8, nz=65, enable_perturbations=True, use_analytical_perturbations=True)
    with pytest.raises(np.linalg.LinAlgError):
        ref.run(cfg, 1)
    Dn = ref.differentiation_matrix(x, guard=False)
    assert np.max(np.abs(Dn @ x - 1.0)) < 1e-10


def test_pi_controller_quirks():
    """Method 2 is called with the namelist istart (3D:1118): istart = 0 updates
    every step with the Euler integral; istart not a multiple of the update
    frequency never updates."""
    base = dict(nx=8, ny=8, nz=9, dt=0.01, re=180.0, u_centerline=1.0, flow_control_method=2,
                target_bulk_velocity=0.7, controller_gain=0.15, controller_update_freq=7)
    cfg = ref.Config(**base)
    g = ref.setup_grid(cfg)
    st = ref.initial_state(cfg, g)
    ub = ref.calculate_bulk_velocity(g, st.u)
    assert abs(ub - 2.0 / 3.0) < 1e-14
    ref.step(cfg, g, st)
    err = 0.7 - ub
    assert abs(st.pi.bulk_velocity_error_integral - err * 0.01) < 1e-15
    assert abs(st.pi.current_pressure_gradient - (3 / 180 + 0.15 * err)) < 1e-15
    ref.step(cfg, g, st)
    assert st.pi.pressure_gradient_count == 2
    cfg3 = ref.Config(**dict(base, istart=3))
    g3 = ref.setup_grid(cfg3)
    st3 = ref.initial_state(cfg3, g3)
    ref.step(cfg3, g3, st3)
    assert st3.pi.pressure_gradient_count == 0
    assert st3.pi.current_pressure_gradient == cfg3.target_pressure_gradient


def test_zero_mode_y_gives_no_perturbation():
    """mode_y = 0 => ky = 0 => u' = v' = 0: 'Zero perturbation field' (scale skipped)."""
    cfg = ref.Config(nx=16, ny=8, nz=9, enable_perturbations=True, use_analytical_perturbations=True,
                     analytical_mode_y=0, perturbation_amplitude=0.05, u_centerline=1.0)
    g = ref.setup_grid(cfg)
    st = ref.initial_state(cfg, g)
    assert np.max(np.abs(st.v)) == 0.0
    assert np.max(np.abs(st.u - (1 - g.zpts ** 2)[:, None, None] * np.where(
        (np.arange(g.nz) == 0) | (np.arange(g.nz) == g.nz - 1), 0, 1)[:, None, None])) < 1e-15


def test_splitmix64_known_answer():
    """SplitMix64 with seed 0 (the reference implementation's first outputs)."""
    u = ref.splitmix64_uniform(0, 3)
    want = [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]
    assert [int(x * 2.0 ** 53) for x in u] == [w >> 11 for w in want]


@pytest.mark.parametrize("zero_w", [False, True])
def test_random_solenoidal_perturbation_properties(zero_w):
    """generate_channel_solenoidal_perturbations restated with a seeded
    stream: walls zero, mean energy = amplitude * 0.5 * 1.5^2, the seed
    decides the field, zero_w_perturbations gives w = 0, and the x-y
    projection makes each mode's (kx, ky) . (u^, v^) vanish before damping."""
    cfg = ref.Config(nx=16, ny=12, nz=17, xlen=4 * ref.PI, ylen=2 * ref.PI, enable_perturbations=True,
                     use_analytical_perturbations=False, perturbation_amplitude=0.02,
                     zero_w_perturbations=zero_w, perturbation_seed=11)
    g = ref.setup_grid(cfg)
    up, vp, wp = ref.random_solenoidal_perturbation(cfg, g)
    for a in (up, vp, wp):
        assert np.all(a[0] == 0.0) and np.all(a[-1] == 0.0)
    e = 0.5 * (np.sum(up ** 2) + np.sum(vp ** 2) + np.sum(wp ** 2)) / up.size
    assert abs(e - 0.02 * 0.5 * 1.5 ** 2) < 1e-14
    assert np.all(wp == 0.0) == zero_w
    up2, _, _ = ref.random_solenoidal_perturbation(cfg.with_(perturbation_seed=12), g)
    assert np.max(np.abs(up2 - up)) > 1e-3
    up3, _, _ = ref.random_solenoidal_perturbation(cfg, g)
    np.testing.assert_array_equal(up3, up)
    # u, v of each level: r2c gives spectra with kx u^ + ky v^ = 0 up to the
    # round-off of the transforms (the kx = 0, nx/2 columns are Hermitian-
    # projected by the c2r, which keeps the constraint)
    uh, vh = ref.r2c(up), ref.r2c(vp)
    kd = g.xw[None, None, :] * uh + g.yw[None, :, None] * vh
    keep = np.ones(g.ny, bool)
    keep[g.ny // 2] = False  # ky = ny/2 is not symmetric in the FFTW order
    assert np.max(np.abs(kd[:, keep, :-1])) < 1e-12 * np.max(np.abs(uh))


def test_philox_known_answers():
    """Philox4x32-10, the published known-answer vectors (Random123 kat_vectors)."""
    cases = [((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
             ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
             ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
              (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1))]
    for ctr, key, want in cases:
        out = ref.philox4x32_10(tuple(np.array([c], np.uint64) for c in ctr), key)
        assert tuple(int(o[0]) for o in out) == want


def test_philox_noise_range_and_seed():
    a = ref.philox_noise(3, (5, 6, 7), 0, 1e-3)
    assert a.shape == (5, 6, 7) and np.all(np.abs(a) <= 1e-3)
    assert abs(np.mean(a)) < 2e-4 and np.std(a) > 5e-4
    assert np.max(np.abs(ref.philox_noise(4, (5, 6, 7), 0, 1e-3) - a)) > 1e-4
    assert np.max(np.abs(ref.philox_noise(3, (5, 6, 7), 1, 1e-3) - a)) > 1e-4
