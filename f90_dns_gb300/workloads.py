"""Named channel-flow workloads (namelist values of read_input_3d).

All runs use the analytical stream-function perturbation of
``perturbation_analytical_simple.f90`` on the base profile U = 1 - z^2
(``u_centerline = 1``), Crank-Nicolson, the 2/3 filter and the standard
(collocation) pressure right-hand side, on x in [0, 4 pi), y in [0, 2 pi).
A constant forcing ``target_pressure_gradient = +2/Re`` keeps that profile
steady: the reference adds the value to the x-momentum source
(DNS_pressure_BC_3D.f90:1129), i.e. it is -dp/dx.

Grids with nz >= 58 set ``lgl_dmatrix_guard = 0``: the reference's own
differentiation matrix degenerates there (lgl_module.f90:247-251) and its
pressure solve stops.
"""
from __future__ import annotations

import math

import numpy as np

PI = 4.0 * math.atan(1.0)

_BASE = dict(
    xlen=4.0 * PI, ylen=2.0 * PI, u_centerline=1.0, use_crank_nicolson=True,
    enable_perturbations=True, use_analytical_perturbations=True, zero_w_perturbations=False,
    use_dealias_23_rule=True, use_weak_form_divergence=False, istart=0,
    controller_gain=0.15, controller_update_freq=7,
)


def _wl(**kw) -> dict:
    d = dict(_BASE)
    d.update(kw)
    d.setdefault("lgl_dmatrix_guard", d["nz"] < 58)
    d.setdefault("nwrt", d.get("nsteps", 1))
    d.setdefault("restart_write_freq", max(1000, d.get("nsteps", 1)))
    return d


WORKLOADS = {
    # 32x32x33, Re 180, dt 0.002, constant forcing 2/Re, amplitude 0.01, mode (1,1), 100 steps
    "channel_32x32x33_re180_dpdx": _wl(
        nx=32, ny=32, nz=33, re=180.0, dt=0.002, flow_control_method=1,
        target_pressure_gradient=2.0 / 180.0, perturbation_amplitude=0.01,
        analytical_mode_x=1, analytical_mode_y=1, nsteps=100),
    # 128x128x65, Re 180, dt 0.002, PI control to U_bulk = 2/3, amplitude 0.05, mode (2,1), 1000 steps
    "channel_128x128x65_re180_pi": _wl(
        nx=128, ny=128, nz=65, re=180.0, dt=0.002, flow_control_method=2,
        target_bulk_velocity=2.0 / 3.0, target_pressure_gradient=2.0 / 180.0,
        perturbation_amplitude=0.05, analytical_mode_x=2, analytical_mode_y=1, nsteps=1000),
    # 256x256x97 serving-stream large request
    "channel_256x256x97_re180_dpdx": _wl(
        nx=256, ny=256, nz=97, re=180.0, dt=0.002, flow_control_method=1,
        target_pressure_gradient=2.0 / 180.0, perturbation_amplitude=0.02,
        analytical_mode_x=1, analytical_mode_y=1, nsteps=200),
    # 512x384x129, Re 180, dt 0.001, PI to 2/3, amplitude 0.08, mode (2,2), 2000 steps,
    # plus seeded white noise of amplitude 1e-3 on u, v, w (Philox, seed 0)
    "channel_512x384x129_re180_pi": _wl(
        nx=512, ny=384, nz=129, re=180.0, dt=0.001, flow_control_method=2,
        target_bulk_velocity=2.0 / 3.0, target_pressure_gradient=2.0 / 180.0,
        perturbation_amplitude=0.08, analytical_mode_x=2, analytical_mode_y=2, nsteps=2000,
        noise_amplitude=1.0e-3, perturbation_seed=0),
}


def ensemble_draws(n: int = 64, seed: int = 0) -> list[dict]:
    """Seeded parameter sweep: nx, ny in {32,48,64,96}, nz in {33,49,65},
    Re ~ U[100,300], amplitude log-uniform [0.005, 0.08], mode_x in {1,2,3},
    mode_y in {0,1,2} (mode_y = 0 gives no perturbation at all, as in the
    reference), dt 0.002, constant forcing 2/Re, 500 steps."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        re = float(rng.uniform(100.0, 300.0))
        out.append(_wl(
            nx=int(rng.choice([32, 48, 64, 96])), ny=int(rng.choice([32, 48, 64, 96])),
            nz=int(rng.choice([33, 49, 65])), re=re, dt=0.002, flow_control_method=1,
            target_pressure_gradient=2.0 / re,
            perturbation_amplitude=float(math.exp(rng.uniform(math.log(0.005), math.log(0.08)))),
            analytical_mode_x=int(rng.choice([1, 2, 3])), analytical_mode_y=int(rng.choice([0, 1, 2])),
            nsteps=500))
    return out


def point_count(wl: dict) -> int:
    return int(wl["nx"]) * int(wl["ny"]) * int(wl["nz"])
