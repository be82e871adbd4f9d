"""CPU restatement of the 3D channel-flow time step (TEST INFRASTRUCTURE ONLY).

This module is the parity oracle for the GB300 implementation.  Only the test
suite, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl
reference`` legs of ``bench.py`` may import it, and only as the checker or as
the timed CPU baseline.  The product path (``f90_dns_gb300``) never calls it.

It restates, in FP64 numpy, the reference Fortran program
``DNS_pressure_BC_3D.f90`` (chandc/F90_DNS) exactly as written, quirks
included, working in PHYSICAL space the way the reference does (every
derivative is an r2c -> multiply -> c2r round trip per z-plane; z-derivatives
are ``d1`` column products).  The GPU path is spectral-resident, so this
restatement is an independent formulation of the same arithmetic.

Third-party arithmetic restated here:
  * FFTW3 ``fftw_plan_dft_r2c_2d(ny, nx, ...)`` / ``c2r`` (version unpinned;
    call sites ``fftw3_dns_module.f90:72,75,106,127``).  numpy's pocketfft
    ``rfft2`` / ``irfft2(s=(ny, nx))`` has the same conventions: unnormalised
    forward, c2r = inverse c2c along y then 1D c2r along x that ignores the
    imaginary parts of the kx=0 and kx=nx/2 entries; the wrapper divides by
    nx*ny (``fftw3_dns_module.f90:130``), which is numpy's default ``ifft``
    normalisation.
  * LAPACK ``zgesv`` (unpinned; 3D:1505, 1714, 1816) -> ``numpy.linalg.solve``
    (LAPACK ``gesv``: LU with partial pivoting) on the same matrices.

Layout: Fortran ``u(nx,ny,nz)`` (i fastest) is the C array ``u[nz][ny][nx]``;
spectral planes are ``[nz][ny][nx//2+1]`` complex128 in FFTW order.

Pins: ``tests/test_oracle_pins.py`` checks this module against the reference's
own captured run (``standard_output.txt``) and its analytic known answers.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, replace

import numpy as np

PI = 4.0 * math.atan(1.0)  # DNS_pressure_BC_3D.f90:43


# --------------------------------------------------------------------------
# Configuration: the namelist variables of read_input_3d (3D:554-708)
# --------------------------------------------------------------------------
@dataclass
class Config:
    """Namelist parameters with the reference defaults (3D:571-603)."""

    nx: int = 128
    ny: int = 32
    nz: int = 33
    istart: int = 0
    dt: float = 0.01
    nsteps: int = 1000
    nwrt: int = 100
    restart_write_freq: int = 1000
    re: float = 180.0
    xlen: float = 2.0 * PI
    ylen: float = 2.0 * PI
    use_crank_nicolson: bool = True
    u_centerline: float = 1.5
    flow_control_method: int = 1
    target_pressure_gradient: float = 0.03
    target_bulk_velocity: float = 1.0
    controller_gain: float = 0.15
    controller_update_freq: int = 7
    enable_perturbations: bool = False
    perturbation_amplitude: float = 0.01
    zero_w_perturbations: bool = False
    use_analytical_perturbations: bool = False
    analytical_mode_x: int = 1
    analytical_mode_y: int = 1
    use_weak_form_divergence: bool = False
    use_dealias_23_rule: bool = False
    # Not a namelist variable.  True reproduces lgl_module.f90:247-251, which
    # zeroes every D entry whose Lagrange denominator is <= 1e-15; for nz >= 58
    # that is every off-diagonal entry and the reference's pinned Poisson mode
    # becomes singular (zgesv info /= 0 -> stop, 3D:1715-1718).  False keeps
    # the same Lagrange formula without the cutoff.
    lgl_dmatrix_guard: bool = True
    # Not a namelist variable of the reference: seed of the stream that
    # replaces its clock-seeded random_number in the random solenoidal
    # perturbation (perturbation_module.f90:78-83).
    perturbation_seed: int = 0
    # Optional schemes (not in the reference's 3D solver; from its 2D solver):
    # convection_scheme 1 = jst4 (DNS_pressure_BC_2D.f90:931-1014 lifted to
    # 3D), linear_solver 1 = jacgs (DNS_pressure_BC_2D.f90:2361-2476) with a
    # relative stopping test at cgstol (3D default 1e-6, 3D:575).
    convection_scheme: int = 0
    linear_solver: int = 0
    cgstol: float = 1.0e-6
    # Not a reference feature: seeded white noise on the initial u, v, w
    # (the large-grid workload), Philox4x32-10 keyed by perturbation_seed.
    noise_amplitude: float = 0.0

    def with_(self, **kw) -> "Config":
        return replace(self, **kw)


# --------------------------------------------------------------------------
# LGL nodes, weights and differentiation matrix (lgl_module.f90)
# --------------------------------------------------------------------------
def _legendre(n: int, x: float) -> float:
    """legendre_poly, lgl_module.f90:86-110 (three-term recurrence)."""
    if n == 0:
        return 1.0
    if n == 1:
        return x
    p0, p1 = 1.0, x
    for k in range(2, n + 1):
        p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k
        p0, p1 = p1, p2
    return p1


def _legendre_d(n: int, x: float):
    """legendre_poly_and_deriv, lgl_module.f90:115-155: P_n, P_n', P_n''."""
    if n == 0:
        return 1.0, 0.0, 0.0
    if n == 1:
        return x, 1.0, 0.0
    p0, dp0, d2p0 = 1.0, 0.0, 0.0
    p1, dp1, d2p1 = x, 1.0, 0.0
    for k in range(2, n + 1):
        p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k
        dp2 = ((2 * k - 1) * (x * dp1 + p1) - (k - 1) * dp0) / k
        d2p2 = ((2 * k - 1) * (x * d2p1 + 2.0 * dp1) - (k - 1) * d2p0) / k
        p0, p1 = p1, p2
        dp0, dp1 = dp1, dp2
        d2p0, d2p1 = d2p1, d2p2
    return p1, dp1, d2p1


def lgl_nodes_weights(n: int):
    """lgl_nodes_weights, lgl_module.f90:30-80.

    Newton on P'_{n-1} from Chebyshev guesses -cos(pi*(i-1)/(n-1)), tolerance
    1e-15, at most 100 iterations; weights 2/(n(n-1) P_{n-1}(x)^2), endpoint
    weights 2/(n(n-1)).  Node 1 is z=-1.
    """
    pi_l = 3.14159265358979323846  # lgl_module.f90:22
    nodes = np.zeros(n)
    weights = np.zeros(n)
    if n == 1:
        return np.array([0.0]), np.array([2.0])
    if n == 2:
        return np.array([-1.0, 1.0]), np.array([1.0, 1.0])
    nodes[0], nodes[-1] = -1.0, 1.0
    weights[0] = 2.0 / float(n * (n - 1))
    weights[-1] = weights[0]
    for i in range(2, n):
        x = -math.cos(pi_l * (i - 1) / (n - 1))
        for _ in range(100):
            x_old = x
            _, dp, d2p = _legendre_d(n - 1, x)
            x = x_old - dp / d2p
            if abs(x - x_old) < 1.0e-15:
                break
        nodes[i - 1] = x
        p = _legendre(n - 1, x)
        weights[i - 1] = 2.0 / (float(n * (n - 1)) * p * p)
    return nodes, weights


def differentiation_matrix(nodes: np.ndarray, guard: bool = True) -> np.ndarray:
    """differentiation_matrix, lgl_module.f90:211-263 (Lagrange products).

    D[i,i] = sum_{k!=i} 1/(x_i-x_k); D[i,j] = prod_{k!=i,j}(x_i-x_k) /
    prod_{k!=j}(x_j-x_k), set to 0 if |denominator| <= 1e-15 (the reference
    guard, lgl_module.f90:247-251) unless ``guard`` is False.
    """
    n = len(nodes)
    d = np.zeros((n, n))
    if n == 1:
        return d
    for i in range(n):
        for j in range(n):
            if i == j:
                s = 0.0
                for k in range(n):
                    if k != i:
                        s += 1.0 / (nodes[i] - nodes[k])
                d[i, i] = s
            else:
                prod1 = 1.0
                prod2 = 1.0
                for k in range(n):
                    if k != i and k != j:
                        prod1 *= nodes[i] - nodes[k]
                    if k != j:
                        prod2 *= nodes[j] - nodes[k]
                d[i, j] = prod1 / prod2 if (abs(prod2) > 1.0e-15 or not guard) else 0.0
    return d


# --------------------------------------------------------------------------
# Grid / spectral setup (setup_grid_3d 3D:728-753, setup_spectral_3d 769-809)
# --------------------------------------------------------------------------
@dataclass
class Grid:
    nx: int
    ny: int
    nz: int
    xlen: float
    ylen: float
    alpha: float
    beta: float
    ybar: float
    xw: np.ndarray
    xsq: np.ndarray
    yw: np.ndarray
    ysq: np.ndarray
    zpts: np.ndarray
    zwts: np.ndarray
    d1: np.ndarray
    d2: np.ndarray

    @property
    def nxhp(self) -> int:
        return self.nx // 2 + 1


def setup_grid(cfg: Config) -> Grid:
    nx, ny, nz = cfg.nx, cfg.ny, cfg.nz
    alpha = 2.0 * PI / cfg.xlen  # 3D:740 (overrides the namelist alpha)
    beta = 2.0 * PI / cfg.ylen   # 3D:741
    ybar = 2.0                   # 3D:742
    nxhp = nx // 2 + 1
    xw = np.arange(nxhp, dtype=np.float64) * alpha  # 3D:780-783
    yw = np.empty(ny)
    for j in range(1, ny + 1):                       # 3D:789-796
        if j <= ny // 2 + 1:
            yw[j - 1] = float(j - 1) * 2.0 * PI / cfg.ylen
        else:
            yw[j - 1] = float(j - 1 - ny) * 2.0 * PI / cfg.ylen
    zpts, zwts = lgl_nodes_weights(nz)
    d1 = differentiation_matrix(zpts, cfg.lgl_dmatrix_guard)
    d2 = d1 @ d1  # 3D:801
    return Grid(nx, ny, nz, cfg.xlen, cfg.ylen, alpha, beta, ybar,
                xw, xw ** 2, yw, yw ** 2, zpts, zwts, d1, d2)


# --------------------------------------------------------------------------
# FFT wrapper (fftw3_dns_module.f90:100-131), all z-planes at once
# --------------------------------------------------------------------------
def r2c(f: np.ndarray) -> np.ndarray:
    """fftw3_forward_2d_dns per plane: unnormalised r2c, [..,ny,nx] -> [..,ny,nx/2+1]."""
    return np.fft.rfft2(f, axes=(-2, -1))


def c2r(fh: np.ndarray, nx: int, ny: int) -> np.ndarray:
    """fftw3_backward_2d_dns per plane: c2r then / (nx*ny)."""
    return np.fft.irfft2(fh, s=(ny, nx), axes=(-2, -1))


# --------------------------------------------------------------------------
# Derivatives (compute_derivatives_3d 3D:2321-2407), divergence (1858-1879)
# --------------------------------------------------------------------------
def ddz(g: Grid, f: np.ndarray) -> np.ndarray:
    """dfdz(i,j,:) = (2/ybar) * matmul(d1, f(i,j,:)) (3D:2351-2357)."""
    return (2.0 / g.ybar) * np.einsum("kn,nji->kji", g.d1, f, optimize=True)


def ddx(g: Grid, f: np.ndarray) -> np.ndarray:
    """c2r(r2c(f) * (0, xw(i))) per plane (3D:2380-2387)."""
    return c2r(r2c(f) * (1j * g.xw)[None, None, :], g.nx, g.ny)


def ddy(g: Grid, f: np.ndarray) -> np.ndarray:
    """c2r(r2c(f) * (0, yw(j))) per plane (3D:2390-2397)."""
    return c2r(r2c(f) * (1j * g.yw)[None, :, None], g.nx, g.ny)


def derivatives(g: Grid, f: np.ndarray):
    return ddx(g, f), ddy(g, f), ddz(g, f)


def divergence(g: Grid, fx, fy, fz) -> np.ndarray:
    """compute_divergence_3d: dfx/dx + dfy/dy + dfz/dz (3D:1858-1879)."""
    return ddx(g, fx) + ddy(g, fy) + ddz(g, fz)


def laplacian(g: Grid, f: np.ndarray) -> np.ndarray:
    """compute_laplacian_3d (3D:1564-1606): (2/ybar)^2 d2 f^ - (xsq+ysq) f^."""
    fh = r2c(f)
    zs = 2.0 / g.ybar
    lap = np.einsum("kn,nji->kji", g.d2, fh, optimize=True) * zs ** 2
    ksq = g.xsq[None, :] + g.ysq[:, None]
    lap = lap - ksq[None, :, :] * fh
    return c2r(lap, g.nx, g.ny)


def stiffness(g: Grid) -> np.ndarray:
    """S_kn = sum_m d1(m,k) d1(m,n) zwts(m) * (2/ybar) (3D:1467-1471, 1688)."""
    return (g.d1.T * g.zwts[None, :]) @ g.d1 * (2.0 / g.ybar)


def dealias_mask(g: Grid) -> np.ndarray:
    """apply_dealias_truncation keep-mask, [ny][nxhp] (3D:1163-1193)."""
    nx, ny = g.nx, g.ny
    kx_max = (nx // 2) * 2 // 3
    ky_max = (ny // 2) * 2 // 3
    keep = np.ones((ny, nx // 2 + 1), dtype=bool)
    for j in range(1, ny + 1):
        for i in range(1, nx // 2 + 2):
            if (i - 1) > kx_max:
                keep[j - 1, i - 1] = False
                continue
            if j <= ny // 2 + 1:
                if (j - 1) > ky_max:
                    keep[j - 1, i - 1] = False
            elif abs(j - 1 - ny) > ky_max:
                keep[j - 1, i - 1] = False
    return keep


# --------------------------------------------------------------------------
# State
# --------------------------------------------------------------------------
@dataclass
class PIState:
    """PI controller globals (3D:75-89), initialised in read_input_3d (3D:623-635)."""

    current_pressure_gradient: float
    current_bulk_velocity: float = 0.0
    bulk_velocity_error: float = 0.0
    bulk_velocity_error_integral: float = 0.0
    bulk_velocity_error_prev: float = 0.0
    pressure_gradient_sum: float = 0.0
    pressure_gradient_count: int = 0
    avg_pressure_gradient: float = 0.0


@dataclass
class State:
    u: np.ndarray
    v: np.ndarray
    w: np.ndarray
    p_total: np.ndarray
    gpx: np.ndarray  # grad_p_prev_x
    gpy: np.ndarray  # grad_p_prev_y
    gpz: np.ndarray  # grad_p_prev_z (computed, never consumed)
    pi: PIState
    time: float = 0.0
    istep: int = 0
    extras: dict = field(default_factory=dict)

    def copy(self) -> "State":
        return State(self.u.copy(), self.v.copy(), self.w.copy(), self.p_total.copy(),
                     self.gpx.copy(), self.gpy.copy(), self.gpz.copy(),
                     replace(self.pi), self.time, self.istep, dict(self.extras))


def analytical_perturbation(g: Grid, amp: float, mx: int, my: int):
    """generate_analytical_perturbations, perturbation_analytical_simple.f90:24-105.

    psi = sin(kx x) sin(ky y)(1-z^2); u' = -ky sin cos (1-z^2),
    v' = kx cos sin (1-z^2), w' = 0; scaled so max |u'| (pointwise vector
    norm) = amp unless that max is <= 1e-12 (then left at zero, :120-133);
    walls zeroed (:138-155).
    """
    nx, ny, nz = g.nx, g.ny, g.nz
    kx = 2.0 * PI * mx / g.xlen
    ky = 2.0 * PI * my / g.ylen
    x = np.arange(nx) * g.xlen / nx
    y = np.arange(ny) * g.ylen / ny
    damp = 1.0 - g.zpts ** 2
    sx, cx = np.sin(kx * x), np.cos(kx * x)
    sy, cy = np.sin(ky * y), np.cos(ky * y)
    up = -ky * damp[:, None, None] * (cy[None, :, None] * sx[None, None, :])
    vp = kx * damp[:, None, None] * (sy[None, :, None] * cx[None, None, :])
    wp = np.zeros_like(up)
    cur = np.max(np.sqrt(up ** 2 + vp ** 2 + wp ** 2))
    if cur > 1.0e-12:
        s = amp / cur
        up, vp, wp = up * s, vp * s, wp * s
    for a in (up, vp, wp):
        a[0] = 0.0
        a[-1] = 0.0
    return up, vp, wp


def splitmix64_uniform(seed: int, n: int) -> np.ndarray:
    """n uniforms in [0, 1) from SplitMix64 (Steele, Lea and Flood 2014):
    output i = mix(seed + (i+1) * 0x9E3779B97F4A7C15), top 53 bits."""
    gamma = np.uint64(0x9E3779B97F4A7C15)
    s = np.uint64(seed % (1 << 64)) + (np.arange(n, dtype=np.uint64) + np.uint64(1)) * gamma
    z = (s ^ (s >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * 2.0 ** -53


def integrate_w_column(z: np.ndarray, div: np.ndarray) -> np.ndarray:
    """integrate_with_boundary_conditions_fallback (perturbation_module.f90:
    470-517) for one column: trapezoid integral of -div from w(-1) = 0,
    quadratic correction to w(+1) = 0, sin^2 tapers (with 3.14159)."""
    nz = len(z)
    up = np.zeros(nz)
    for k in range(1, nz):
        up[k] = up[k - 1] - 0.5 * (div[k] + div[k - 1]) * (z[k] - z[k - 1])
    total = up[-1]
    zn = (z - z[0]) / (z[-1] - z[0])
    w = up - total * (zn * (2.0 - zn))
    w[0] = 0.0
    w[-1] = 0.0
    for k in range(2, min(4, nz - 1) + 1):           # Fortran levels
        w[k - 1] *= math.sin(0.5 * 3.14159 * float(k - 1) / 3.0) ** 2
    for k in range(max(nz - 3, 2), nz):
        w[k - 1] *= math.sin(0.5 * 3.14159 * float(nz - k) / 3.0) ** 2
    return w


def random_solenoidal_perturbation(cfg: Config, g: Grid):
    """generate_channel_solenoidal_perturbations (perturbation_module.f90:
    42-176) with SplitMix64 draws in place of the clock-seeded random_number:
    four uniforms per mode (Re u, Im u, Re v, Im v; k, j, i order), damping
    by 0.1 beyond half the smaller Nyquist wavenumber, projection onto
    kx u + ky v = 0 separately for the real and imaginary parts, zero mean
    mode, c2r per plane; w from integrating -(du/dx + dv/dy) per column (or
    zero); walls zeroed and the interior damped by (1 - z^2)^2
    (enforce_channel_walls :276-320); energy scaled to amplitude * 0.5 * 1.5^2
    (scale_to_amplitude :325-372)."""
    nx, ny, nz, nxhp = g.nx, g.ny, g.nz, g.nxhp
    pi = 4.0 * math.atan(1.0)
    r = splitmix64_uniform(cfg.perturbation_seed, 4 * nz * ny * nxhp).reshape(nz, ny, nxhp, 4) - 0.5
    uh = r[..., 0] + 1j * r[..., 1]
    vh = r[..., 2] + 1j * r[..., 3]
    kx = 2.0 * pi * np.arange(nxhp) / cfg.xlen
    jj = np.arange(1, ny + 1)
    ky = 2.0 * pi * np.where(jj <= ny // 2 + 1, jj - 1, jj - 1 - ny) / cfg.ylen
    KX, KY = np.meshgrid(kx, ky)                       # [ny][nxhp]
    kp = KX * KX + KY * KY
    damp = np.where(np.sqrt(kp) > 0.5 * min(2.0 * pi * nx / cfg.xlen, 2.0 * pi * ny / cfg.ylen), 0.1, 1.0)
    ur, ui, vr, vi = uh.real * damp, uh.imag * damp, vh.real * damp, vh.imag * damp
    proj = kp > 1.0e-12
    kps = np.where(proj, kp, 1.0)
    kv = KX * ur + KY * vr
    ur = np.where(proj, ur - KX * kv / kps, ur)
    vr = np.where(proj, vr - KY * kv / kps, vr)
    kv = KX * ui + KY * vi
    ui = np.where(proj, ui - KX * kv / kps, ui)
    vi = np.where(proj, vi - KY * kv / kps, vi)
    uh = ur + 1j * ui
    vh = vr + 1j * vi
    uh[:, 0, 0] = 0.0
    vh[:, 0, 0] = 0.0
    up = c2r(uh, nx, ny)
    vp = c2r(vh, nx, ny)
    if cfg.zero_w_perturbations:
        wp = np.zeros_like(up)
    else:
        dxy = ddx(g, up) + ddy(g, vp)
        wp = np.empty_like(up)
        for j in range(ny):
            for i in range(nx):
                wp[:, j, i] = integrate_w_column(g.zpts, dxy[:, j, i])
    d = (1.0 - g.zpts ** 2) ** 2
    d[0] = d[-1] = 0.0
    up, vp, wp = (a * d[:, None, None] for a in (up, vp, wp))
    cur = 0.5 * (np.sum(up ** 2) + np.sum(vp ** 2) + np.sum(wp ** 2)) / float(nx * ny * nz)
    target = cfg.perturbation_amplitude * (0.5 * 1.5 ** 2)
    sc = math.sqrt(target / cur) if cur > 1.0e-15 else 1.0
    return up * sc, vp * sc, wp * sc


def philox4x32_10(ctr, key):
    """Philox4x32-10 (Salmon, Moraes, Dror and Shaw, SC'11) on arrays of
    counters ctr = (c0, c1, c2, c3) (uint32 arrays) with key (k0, k1)."""
    m32 = np.uint64(0xFFFFFFFF)
    c0, c1, c2, c3 = (np.asarray(x, dtype=np.uint64) for x in ctr)
    k0, k1 = np.uint64(key[0]), np.uint64(key[1])
    for r in range(10):
        if r:
            k0 = (k0 + np.uint64(0x9E3779B9)) & m32
            k1 = (k1 + np.uint64(0xBB67AE85)) & m32
        p0 = np.uint64(0xD2511F53) * c0
        p1 = np.uint64(0xCD9E8D57) * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & m32
        hi1, lo1 = p1 >> np.uint64(32), p1 & m32
        c0, c1, c2, c3 = (hi1 ^ c1 ^ k0) & m32, lo1, (hi0 ^ c3 ^ k1) & m32, lo0
    return c0, c1, c2, c3


def philox_noise(seed: int, shape, comp: int, amplitude: float) -> np.ndarray:
    """Uniform noise in [-amplitude, amplitude) for component comp at every
    point of `shape` (C order index n): counter (n low, n high, comp, 0), key
    (seed low, seed high), 53 bits from the first two outputs."""
    n = np.arange(int(np.prod(shape)), dtype=np.uint64)
    s = int(seed) % (1 << 64)
    x0, x1, _, _ = philox4x32_10((n & np.uint64(0xFFFFFFFF), n >> np.uint64(32),
                                  np.full(n.shape, comp, np.uint64), np.zeros(n.shape, np.uint64)),
                                 (s & 0xFFFFFFFF, s >> 32))
    u = ((x0 >> np.uint64(5)) * np.uint64(67108864) + (x1 >> np.uint64(6))).astype(np.float64) * 2.0 ** -53
    return (amplitude * (2.0 * u - 1.0)).reshape(shape)


def initial_state(cfg: Config, g: Grid, noise=None) -> State:
    """initialize_fields_3d (3D:909-962) with the analytical perturbation.

    ``noise``: optional (nu, nv, nw) arrays added after the perturbation and
    before the final wall reset.  This is not a reference feature; it is used
    only by the large seeded white-noise workload.
    """
    shape = (g.nz, g.ny, g.nx)
    u = np.broadcast_to((cfg.u_centerline * (1.0 - g.zpts ** 2))[:, None, None], shape).copy()
    v = np.zeros(shape)
    w = np.zeros(shape)
    if cfg.enable_perturbations:
        if cfg.use_analytical_perturbations:
            up, vp, wp = analytical_perturbation(g, cfg.perturbation_amplitude,
                                                 cfg.analytical_mode_x, cfg.analytical_mode_y)
        else:
            up, vp, wp = random_solenoidal_perturbation(cfg, g)
        u, v, w = u + up, v + vp, w + wp
    if noise is None and cfg.noise_amplitude > 0.0:
        noise = tuple(philox_noise(cfg.perturbation_seed, shape, c, cfg.noise_amplitude) for c in range(3))
    if noise is not None:
        u, v, w = u + noise[0], v + noise[1], w + noise[2]
    if cfg.enable_perturbations or noise is not None:
        for a in (u, v, w):  # apply_boundary_conditions_3d (3D:3253)
            a[0] = 0.0
            a[-1] = 0.0
    z = np.zeros(shape)
    pi = PIState(current_pressure_gradient=cfg.target_pressure_gradient,
                 avg_pressure_gradient=cfg.target_pressure_gradient)
    return State(u, v, w, z.copy(), z.copy(), z.copy(), z.copy(), pi)


# --------------------------------------------------------------------------
# The time step (3D:286-361), one subroutine per reference subroutine
# --------------------------------------------------------------------------
def calculate_bulk_velocity(g: Grid, u: np.ndarray) -> float:
    """calculate_bulk_velocity_3d (3D:2434-2464): sum u*w_k / (nx*ny*sum w_k)."""
    vol = 0.0
    wsum = 0.0
    for k in range(g.nz):
        vol += float(np.sum(u[k])) * g.zwts[k]
        wsum += g.zwts[k]
    return vol / (float(g.nx * g.ny) * wsum)


def update_pressure_gradient(cfg: Config, g: Grid, st: State, istep: int) -> None:
    """update_pressure_gradient_3d (3D:2488-2549), positional PI with anti-windup."""
    pi = st.pi
    if istep % cfg.controller_update_freq != 0:
        return
    pi.current_bulk_velocity = calculate_bulk_velocity(g, st.u)
    pi.bulk_velocity_error = cfg.target_bulk_velocity - pi.current_bulk_velocity
    kp = cfg.controller_gain
    ki = 0.05 * cfg.controller_gain
    base = 3.0 / cfg.re
    unclamped = base + kp * pi.bulk_velocity_error + ki * pi.bulk_velocity_error_integral
    clamped = max(0.0, min(10.0, unclamped))
    if abs(clamped - unclamped) < 1.0e-12:
        if istep <= cfg.controller_update_freq:
            pi.bulk_velocity_error_integral += pi.bulk_velocity_error * cfg.dt
        else:
            pi.bulk_velocity_error_integral += 0.5 * cfg.dt * (pi.bulk_velocity_error_prev
                                                               + pi.bulk_velocity_error)
    pi.bulk_velocity_error_prev = pi.bulk_velocity_error
    pi.current_pressure_gradient = clamped
    pi.pressure_gradient_sum += clamped
    pi.pressure_gradient_count += 1
    pi.avg_pressure_gradient = pi.pressure_gradient_sum / float(pi.pressure_gradient_count)


def jacgs(A: np.ndarray, b: np.ndarray, tol: float, maxit: int = 500) -> np.ndarray:
    """jacgs (DNS_pressure_BC_2D.f90:2361-2476) on a batch of real systems
    A[s] x[s] = b[s]: Jacobi-preconditioned conjugate gradients from x = 0,
    small = 1e-30 guards, at most `maxit` iterations; a system stops when its
    residual 2-norm is <= tol * (initial residual 2-norm) (the reference tests
    the absolute norm against tol).  Converged systems are left unchanged."""
    small = 1.0e-30
    d = np.diagonal(A, axis1=1, axis2=2)
    dinv = np.where(np.abs(d) > small, 1.0 / np.where(d == 0.0, 1.0, d), 1.0)
    x = np.zeros_like(b)
    r = b.copy()
    q = r * dinv
    p = q.copy()
    res0 = np.sqrt(np.sum(r * r, axis=1))
    active = res0 > 0.0
    for _ in range(maxit):
        if not active.any():
            break
        ap = np.einsum("sij,sj->si", A, p)
        qdr = np.sum(q * r, axis=1)
        alfa = qdr / (np.sum(p * ap, axis=1) + small)
        a = active[:, None]
        x = np.where(a, x + alfa[:, None] * p, x)
        r = np.where(a, r - alfa[:, None] * ap, r)
        q = r * dinv
        beta = np.sum(q * r, axis=1) / (qdr + small)
        p = np.where(a, q + beta[:, None] * p, p)
        res1 = np.sqrt(np.sum(r * r, axis=1))
        active = active & ~(res1 <= tol * res0)
    return x


def _solve_real_systems(A: np.ndarray, b: np.ndarray, tol: float) -> np.ndarray:
    """jacgs on complex right-hand sides: real and imaginary parts apart."""
    xr = jacgs(A, np.ascontiguousarray(b.real), tol)
    xi = jacgs(A, np.ascontiguousarray(b.imag), tol)
    return xr + 1j * xi


def nonlinear_source(cfg: Config, g: Grid, u, v, w):
    """compute_source_terms_3d_standard (3D:1054-1098) and, with the 2/3 rule,
    the filtering of compute_source_terms_3d_dealiased (3D:1233-1261):
    S = u x omega (the gradient part is absorbed into p)."""
    ux, uy, uz = derivatives(g, u)
    vx, vy, vz = derivatives(g, v)
    wx, wy, wz = derivatives(g, w)
    ox = wy - vz  # 3D:1077-1079
    oy = uz - wx
    oz = vx - uy
    su = v * oz - w * oy  # 3D:1089-1091
    sv = w * ox - u * oz
    sw = u * oy - v * ox
    if cfg.use_dealias_23_rule:  # compute_source_terms_3d_dealiased (3D:1233-1261)
        keep = dealias_mask(g)
        su = c2r(np.where(keep, r2c(su), 0.0), g.nx, g.ny)
        sv = c2r(np.where(keep, r2c(sv), 0.0), g.nx, g.ny)
        sw = c2r(np.where(keep, r2c(sw), 0.0), g.nx, g.ny)
    return su, sv, sw


def jst4_source(cfg: Config, g: Grid, st: State):
    """runge_kutta_convection (DNS_pressure_BC_2D.f90:931-1014) lifted to 3D:
    for irk = 4, 3, 2 the stage state is u^n + (1/irk) dt S(previous stage
    state) with the walls zeroed (apply_wall_bc); the source of the step is S
    of the last stage state (the 2D routine keeps the irk = 1 evaluation and
    resets u to u^n)."""
    cu, cv, cw = st.u, st.v, st.w
    for irk in (4, 3, 2):
        su, sv, sw = nonlinear_source(cfg, g, cu, cv, cw)
        a = (1.0 / float(irk)) * cfg.dt
        cu, cv, cw = st.u + a * su, st.v + a * sv, st.w + a * sw
        for f in (cu, cv, cw):
            f[0] = 0.0
            f[-1] = 0.0
    return nonlinear_source(cfg, g, cu, cv, cw)


def compute_source_terms(cfg: Config, g: Grid, st: State):
    """compute_source_terms_3d (3D:1032-1045) -> (su, sv, sw)."""
    if cfg.convection_scheme == 1:
        su, sv, sw = jst4_source(cfg, g, st)
    else:
        su, sv, sw = nonlinear_source(cfg, g, st.u, st.v, st.w)
    # apply_flow_control_forcing (3D:1107-1148); method 2 is called with the
    # namelist istart, not the step number (3D:1118)
    if cfg.flow_control_method == 1:
        st.pi.current_pressure_gradient = cfg.target_pressure_gradient
    elif cfg.flow_control_method == 2:
        update_pressure_gradient(cfg, g, st, cfg.istart)
    su = su + st.pi.current_pressure_gradient
    return su, sv, sw


def solve_viscous_helmholtz(cfg: Config, g: Grid, rhs: np.ndarray, theta: float,
                            bc1: np.ndarray, bc2: np.ndarray) -> np.ndarray:
    """solve_viscous_helmholtz (3D:1425-1521), including its lifting.

    Rows 1 and nz become identity rows but columns 1 and nz are kept, so the
    wall data is subtracted twice from the interior equations (3D:1494-1502).
    """
    nz = g.nz
    factor = theta * cfg.dt / cfg.re
    rh = r2c(rhs)                       # [nz][ny][nxhp]
    b1 = r2c(bc1)                       # [ny][nxhp]
    b2 = r2c(bc2)
    S = stiffness(g)
    ksq = g.xsq[None, :] + g.ysq[:, None]  # [ny][nxhp]
    ny, nxhp = ksq.shape
    half = g.ybar / 2.0
    # batched matrices [ny*nxhp, nz, nz]
    H = np.broadcast_to(S * factor, (ny * nxhp, nz, nz)).copy()
    diag = (1.0 + factor * ksq.reshape(-1))[:, None] * (g.zwts * half)[None, :]
    idx = np.arange(nz)
    H[:, idx, idx] += diag
    b = (rh.reshape(nz, -1).T * (g.zwts * half)[None, :]).astype(np.complex128)
    b1f = b1.reshape(-1)
    b2f = b2.reshape(-1)
    b[:, 1:nz - 1] -= H[:, 1:nz - 1, 0] * b1f[:, None] + H[:, 1:nz - 1, nz - 1] * b2f[:, None]
    b[:, 0] = b1f
    b[:, nz - 1] = b2f
    if cfg.linear_solver == 1:
        # jacgs on the interior system: the identity rows fix x_1, x_nz and the
        # kept columns subtract the wall data a second time
        r = b[:, 1:nz - 1] - (H[:, 1:nz - 1, 0] * b1f[:, None] + H[:, 1:nz - 1, nz - 1] * b2f[:, None])
        xi = _solve_real_systems(np.ascontiguousarray(H[:, 1:nz - 1, 1:nz - 1]), r, cfg.cgstol)
        x = np.concatenate([b1f[:, None], xi, b2f[:, None]], axis=1)
        return c2r(x.T.reshape(nz, ny, nxhp), g.nx, g.ny)
    H[:, 0, :] = 0.0
    H[:, 0, 0] = 1.0
    H[:, nz - 1, :] = 0.0
    H[:, nz - 1, nz - 1] = 1.0
    x = np.linalg.solve(H.astype(np.complex128), b[:, :, None])[:, :, 0]
    fh = x.T.reshape(nz, ny, nxhp)
    return c2r(fh, g.nx, g.ny)


def viscous_step(cfg: Config, g: Grid, st: State, su, sv, sw):
    """viscous_step_3d (3D:1285-1332) -> (u*, v*, w*)."""
    theta = 0.5 if cfg.use_crank_nicolson else 1.0
    dt = cfg.dt
    rhs_u = st.u + dt * su
    rhs_v = st.v + dt * sv
    rhs_w = st.w + dt * sw
    if theta < 1.0:  # add_explicit_diffusion (3D:1355-1381), factor fixed at 0.5
        fac = 0.5 * dt / cfg.re
        rhs_u = rhs_u + fac * laplacian(g, st.u)
        rhs_v = rhs_v + fac * laplacian(g, st.v)
        rhs_w = rhs_w + fac * laplacian(g, st.w)
    zero = np.zeros((g.ny, g.nx))
    us = solve_viscous_helmholtz(cfg, g, rhs_u, theta, -dt * st.gpx[0], -dt * st.gpx[-1])
    vs = solve_viscous_helmholtz(cfg, g, rhs_v, theta, -dt * st.gpy[0], -dt * st.gpy[-1])
    ws = solve_viscous_helmholtz(cfg, g, rhs_w, theta, zero, zero)
    return us, vs, ws


def _poisson_matrices(g: Grid) -> np.ndarray:
    """Per-mode Galerkin Poisson operators P = -S - diag(k^2 w ybar/2) (3D:1684-1692)."""
    nz = g.nz
    S = stiffness(g)
    ksq = (g.xsq[None, :] + g.ysq[:, None]).reshape(-1)
    P = np.broadcast_to(-S, (ksq.size, nz, nz)).copy()
    idx = np.arange(nz)
    P[:, idx, idx] -= ksq[:, None] * (g.zwts * (g.ybar / 2.0))[None, :]
    # mode (1,1) pin (3D:1702-1711)
    P[0, 0, :] = 0.0
    P[0, :, 0] = 0.0
    P[0, 0, 0] = 1.0
    return P.astype(np.complex128)


def solve_pressure(cfg: Config, g: Grid, us, vs, ws) -> np.ndarray:
    """solve_pressure_3d (3D:1631): standard (1654-1733) or weak form (1749-1835)."""
    nz = g.nz
    ny, nxhp = g.ny, g.nxhp
    half = g.ybar / 2.0
    P = _poisson_matrices(g)
    if not cfg.use_weak_form_divergence:
        div = divergence(g, us, vs, ws) / cfg.dt
        dh = r2c(div)
        b = dh.reshape(nz, -1).T * (0.5 * g.ybar * g.zwts)[None, :]
    else:
        uh, vh, wh = r2c(us), r2c(vs), r2c(ws)
        horiz = (1j * g.xw)[None, None, :] * uh + (1j * g.yw)[None, :, None] * vh
        b = -(horiz.reshape(nz, -1).T) * (g.zwts * half)[None, :]
        # sum_m d1(m,k) * w_hat(m) * zwts(m) * (2/ybar)
        vert = np.einsum("mk,mj->jk", g.d1 * g.zwts[:, None], wh.reshape(nz, -1)) * (2.0 / g.ybar)
        b = (b - vert) / cfg.dt
    b = b.astype(np.complex128)
    b[0, 0] = 0.0
    x = np.linalg.solve(P, b[:, :, None])[:, :, 0]
    if cfg.linear_solver == 1:
        # jacgs on every non-pinned mode: (S + k^2 w ybar/2) phi = -b
        x[1:] = _solve_real_systems(np.ascontiguousarray(-P[1:].real), -b[1:], cfg.cgstol)
    return c2r(x.T.reshape(nz, ny, nxhp), g.nx, g.ny)


def pressure_correction(cfg: Config, g: Grid, st: State, us, vs, ws, phi) -> None:
    """pressure_correction_3d (3D:1903-1929)."""
    px, py, pz = derivatives(g, phi)
    st.u = us - cfg.dt * px
    st.v = vs - cfg.dt * py
    st.w = ws - cfg.dt * pz
    st.p_total = st.p_total + phi
    st.gpx, st.gpy, st.gpz = derivatives(g, st.p_total)


def apply_boundary_conditions(st: State) -> None:
    """apply_boundary_conditions_3d (3D:1953-1972): wall planes := 0."""
    for a in (st.u, st.v, st.w):
        a[0] = 0.0
        a[-1] = 0.0


def step(cfg: Config, g: Grid, st: State) -> State:
    """One pass of the time loop body (3D:286-361) without IO; mutates ``st``."""
    st.istep += 1
    st.time = st.time + cfg.dt
    su, sv, sw = compute_source_terms(cfg, g, st)
    us, vs, ws = viscous_step(cfg, g, st, su, sv, sw)
    phi = solve_pressure(cfg, g, us, vs, ws)
    pressure_correction(cfg, g, st, us, vs, ws, phi)
    apply_boundary_conditions(st)
    return st


# --------------------------------------------------------------------------
# Diagnostics (output_diagnostics_3d 3D:2094-2146, check_divergence_3d 2171-2190)
# --------------------------------------------------------------------------
def diagnostics(cfg: Config, g: Grid, st: State) -> dict:
    umax = float(np.max(np.abs(st.u)))
    vmax = float(np.max(np.abs(st.v)))
    wmax = float(np.max(np.abs(st.w)))
    fac = (g.xlen / g.nx) * (g.ylen / g.ny) * (g.ybar / 2.0)
    e2 = st.u * st.u + st.v * st.v + st.w * st.w
    energy = float(np.sum(0.5 * e2 * fac * g.zwts[:, None, None])) / (g.xlen * g.ylen * g.ybar)
    out = dict(umax=umax, vmax=vmax, wmax=wmax, energy=energy,
               dpdx=st.pi.current_pressure_gradient,
               dpdx_avg=st.pi.avg_pressure_gradient)
    if cfg.flow_control_method == 2:
        out["u_bulk"] = calculate_bulk_velocity(g, st.u)
    else:
        out["u_bulk"] = st.pi.current_bulk_velocity
    return out


def max_divergence(g: Grid, st: State) -> float:
    return float(np.max(np.abs(divergence(g, st.u, st.v, st.w))))


def run(cfg: Config, nsteps: int, record_every: int = 1, noise=None):
    """Set up, run ``nsteps`` steps, return (grid, final state, history)."""
    g = setup_grid(cfg)
    st = initial_state(cfg, g, noise=noise)
    hist = []
    for _ in range(nsteps):
        step(cfg, g, st)
        if st.istep % record_every == 0:
            d = diagnostics(cfg, g, st)
            d["step"] = st.istep
            hist.append(d)
    return g, st, hist


# --------------------------------------------------------------------------
# Output files: the numbers and text of write_time_series_data (3D:2702-2748),
# write_flow_statistics (3D:2849-2952), write_spanwise_averaged_profile
# (3D:2799-2841) and write_velocity_field_snapshot (3D:2756-2791)
# --------------------------------------------------------------------------
def flow_statistics(cfg: Config, g: Grid, st: State) -> dict:
    """The values write_flow_statistics / write_time_series_data write, by
    the reference's physical-space loops (as numpy sums)."""
    d = diagnostics(cfg, g, st)
    nxny = float(g.nx * g.ny)
    if cfg.flow_control_method == 2:
        bulk = calculate_bulk_velocity(g, st.u)                              # 3D:2872
    else:
        bulk = float(np.sum(st.u * g.zwts[:, None, None])) / nxny / 2.0     # 3D:2874-2889
    nu = 1.0 / cfg.re
    dl = float(np.sum((st.u[1] - st.u[0]) / (g.zpts[1] - g.zpts[0]))) / nxny        # 3D:2898-2905
    du = float(np.sum((st.u[-1] - st.u[-2]) / (g.zpts[-1] - g.zpts[-2]))) / nxny    # 3D:2909-2916
    tl, tu = nu * dl, nu * du
    ut = math.sqrt((abs(tl) + abs(tu)) / 2.0)
    return dict(umax=d["umax"], vmax=d["vmax"], wmax=d["wmax"], energy=d["energy"], bulk_velocity=bulk,
                dpdx=d["dpdx"], dpdx_avg=d["dpdx_avg"], wall_shear_lower=tl, wall_shear_upper=tu,
                friction_velocity_avg=ut, re_tau=ut * cfg.re, time=st.time, step=st.istep,
                flow_control_method=cfg.flow_control_method)


def spanwise_profile(g: Grid, st: State):
    """Plane means of u, v, w per level k (3D:2817-2834)."""
    n = float(g.nx * g.ny)
    return tuple(np.sum(a, axis=(1, 2)) / n for a in (st.u, st.v, st.w))


def fortran_es(v: float, w: int, d: int) -> str:
    """gfortran's ESw.d: one nonzero digit, d decimals, exponent E+dd (three
    digits without the letter beyond +-99), right-aligned in w; '*' * w when
    the text does not fit; "Infinity" when it fits, else "Inf".  Rounding is
    to nearest on the exact binary value."""
    from decimal import ROUND_HALF_EVEN, Decimal, localcontext
    if math.isnan(v):
        s = "NaN"
    elif math.isinf(v):
        s = ("-" if v < 0 else "") + ("Infinity" if w >= 8 + (v < 0) else "Inf")
    else:
        with localcontext() as ctx:
            ctx.prec = 1200
            ctx.Emin, ctx.Emax = -2000, 2000
            x = Decimal(v)
            sign = "-" if x.is_signed() else ""
            x = abs(x)
            if x == 0:
                mant, e = Decimal(0).quantize(Decimal(1).scaleb(-d)), 0
            else:
                e = x.adjusted()
                mant = (x.scaleb(-e)).quantize(Decimal(1).scaleb(-d), rounding=ROUND_HALF_EVEN)
                if mant >= 10:
                    e += 1
                    mant = (x.scaleb(-e)).quantize(Decimal(1).scaleb(-d), rounding=ROUND_HALF_EVEN)
        es = ("E%+03d" % e) if abs(e) <= 99 else ("%+04d" % e)
        s = f"{sign}{mant}{es}"
    return s.rjust(w) if len(s) <= w else "*" * w


def fortran_f(v: float, w: int, d: int) -> str:
    """gfortran's Fw.d (leading zero kept when it fits)."""
    from decimal import ROUND_HALF_EVEN, Decimal, localcontext
    if not math.isfinite(v):
        return fortran_es(v, w, d)
    with localcontext() as ctx:
        ctx.prec = 1200
        ctx.Emin, ctx.Emax = -2000, 2000
        x = Decimal(v).quantize(Decimal(1).scaleb(-d), rounding=ROUND_HALF_EVEN)
        s = f"{x:f}"  # a negative value that rounds to zero keeps its sign
    return s.rjust(w) if len(s) <= w else "*" * w


def time_series_row(s: dict) -> str:
    """One row of output_time_series.dat (3D:2740-2744)."""
    cols = [s["time"], s["umax"], s["vmax"], s["wmax"], s["energy"]]
    cols += [s["dpdx_avg"], s["bulk_velocity"]] if s["flow_control_method"] == 2 else [s["dpdx"]]
    return f"{s['step']:8d}" + "".join(fortran_es(c, 15, 6) for c in cols)


def flow_statistics_text(s: dict) -> str:
    """flow_statistics.dat (3D:2925-2951)."""
    es = lambda x: fortran_es(x, 15, 6)
    pg = s["dpdx_avg"] if s["flow_control_method"] == 2 else s["dpdx"]
    lines = ["# DNS 3D Flow Statistics Summary", f"# Time step: {s['step']}", "# Time: " + fortran_f(s["time"], 12, 6),
             "", "# Maximum velocities:", "u_max = " + es(s["umax"]), "v_max = " + es(s["vmax"]),
             "w_max = " + es(s["wmax"]), "", "# Energy and bulk flow:", "kinetic_energy = " + es(s["energy"]),
             "bulk_velocity = " + es(s["bulk_velocity"]), "pressure_gradient = " + es(pg), "",
             "# Wall shear stress:", "tau_wall_lower = " + es(s["wall_shear_lower"]),
             "tau_wall_upper = " + es(s["wall_shear_upper"]),
             "friction_velocity_avg = " + es(s["friction_velocity_avg"]), "re_tau = " + es(s["re_tau"])]
    return "\n".join(lines) + "\n"


def spanwise_profile_text(istep: int, time: float, z, ua, va, wa) -> str:
    """spanwise_profile_NNNNN.dat (3D:2812-2835)."""
    lines = ["# DNS 3D Spanwise-Averaged Velocity Profile", f"# Time step: {istep}",
             "# Time: " + fortran_f(time, 12, 6), "# Columns: k, z, u_avg, v_avg, w_avg"]
    for k in range(len(z)):
        lines.append(f"{k + 1:6d}" + "".join(fortran_es(float(a[k]), 15, 6) for a in (z, ua, va, wa)))
    return "\n".join(lines) + "\n"


def velocity_snapshot_text(istep: int, time: float, xlen: float, ylen: float, z, u, v, w) -> str:
    """velocity_field_NNNNN.dat (3D:2769-2786): k outer, i fastest."""
    nz, ny, nx = u.shape
    lines = ["# DNS 3D Velocity Field Snapshot", f"# Time step: {istep}", "# Time: " + fortran_f(time, 12, 6),
             "# Columns: i, j, k, x, y, z, u, v, w"]
    for k in range(nz):
        for j in range(ny):
            y = float(j) * ylen / float(ny)
            for i in range(nx):
                x = float(i) * xlen / float(nx)
                lines.append(f"{i + 1:6d}{j + 1:6d}{k + 1:6d}" + "".join(
                    fortran_es(float(c), 15, 6) for c in (x, y, z[k], u[k, j, i], v[k, j, i], w[k, j, i])))
    return "\n".join(lines) + "\n"
