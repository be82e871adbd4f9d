"""Shared helpers for the parity tests: oracle config conversion and error norms."""
import numpy as np

from oracle import dns3d_ref as ref


def oracle_config(wl: dict) -> ref.Config:
    names = set(ref.Config.__dataclass_fields__)
    kw = {k: v for k, v in wl.items() if k in names}
    for k in ("use_crank_nicolson", "enable_perturbations", "use_analytical_perturbations",
              "zero_w_perturbations", "use_dealias_23_rule", "use_weak_form_divergence",
              "lgl_dmatrix_guard"):
        if k in kw:
            kw[k] = bool(kw[k])
    return ref.Config(**kw)


def _fields(st):
    return {k: (st[k] if isinstance(st, dict) else getattr(st, k)) for k in ("u", "v", "w", "p_total")}


def component_errors(gpu: dict, st, floor: float = 1e-4) -> dict:
    """Max abs difference per field, each relative to that field's own max|.|.
    For u, v, w the scale is floored at ``floor`` x the velocity scale
    U = max(|u|,|v|,|w|): a component far below U (w starts at zero) is held
    to an absolute error of tol x floor x U, since round-off in the coupled
    step is a fraction of U, not of the small component."""
    ref_f = _fields(st)
    U = max(np.max(np.abs(ref_f[k])) for k in ("u", "v", "w"))
    out = {}
    for k in ("u", "v", "w", "p_total"):
        a = ref_f[k]
        own = float(np.max(np.abs(a)))
        sc = max(own, floor * U) if k != "p_total" else max(own, 1e-300)
        out[k] = float(np.max(np.abs(gpu[k] - a)) / sc)
    return out


def velocity_errors(gpu: dict, st) -> dict:
    """Per-field errors of :func:`component_errors`: u, v, w each on its own
    scale (floored at 1e-4 U), p_total on max|p_total|."""
    return component_errors(gpu, st)


def scaled_velocity_errors(gpu: dict, st) -> dict:
    """Max abs difference per component scaled by the velocity scale
    U = max(|u|,|v|,|w|): the norm of the stated errors of the approximate
    forms (mixed precision, iterative solves stopped at a tolerance)."""
    ref_f = _fields(st)
    U = max(np.max(np.abs(ref_f[k])) for k in ("u", "v", "w"))
    out = {k: float(np.max(np.abs(gpu[k] - ref_f[k])) / U) for k in ("u", "v", "w")}
    out["p_total"] = float(np.max(np.abs(gpu["p_total"] - ref_f["p_total"])) / max(np.max(np.abs(ref_f["p_total"])), 1e-300))
    return out
