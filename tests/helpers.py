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


def velocity_errors(gpu: dict, st) -> dict:
    """Max abs difference per component, scaled by the reference velocity scale
    max(|u|,|v|,|w|) (the relative-error definition the parity bar uses)."""
    scale = max(np.max(np.abs(st.u)), np.max(np.abs(st.v)), np.max(np.abs(st.w)))
    out = {}
    for k, a in (("u", st.u), ("v", st.v), ("w", st.w)):
        out[k] = float(np.max(np.abs(gpu[k] - a)) / scale)
    pscale = max(np.max(np.abs(st.p_total)), 1e-300)
    out["p_total"] = float(np.max(np.abs(gpu["p_total"] - st.p_total)) / pscale)
    return out
