"""ctypes binding of the C/OpenMP restatement (oracle/dns3d_cpu.c).

TEST INFRASTRUCTURE AND CPU BASELINE ONLY: loaded by the tests and by the CPU
legs of bench.py; the product library never calls it.  The config is the
numpy restatement's ``Config`` (dns3d_ref.py)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_cpu

_lib = None


class CpuConfig(C.Structure):
    _fields_ = [(n, C.c_int) for n in (
        "nx", "ny", "nz", "istart", "use_crank_nicolson", "flow_control_method", "controller_update_freq",
        "enable_perturbations", "use_analytical_perturbations", "analytical_mode_x", "analytical_mode_y",
        "use_weak_form_divergence", "use_dealias_23_rule", "lgl_dmatrix_guard")] + [(n, C.c_double) for n in (
        "dt", "re", "xlen", "ylen", "u_centerline", "target_pressure_gradient", "target_bulk_velocity",
        "controller_gain", "perturbation_amplitude")]


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(build_cpu.build())
        vp, ip, dp = C.c_void_p, C.c_int, C.POINTER(C.c_double)
        lib.cpu_create.argtypes = [C.POINTER(CpuConfig), ip]
        lib.cpu_create.restype = vp
        lib.cpu_destroy.argtypes = [vp]
        lib.cpu_step.argtypes = [vp, ip]
        lib.cpu_step.restype = ip
        lib.cpu_get_state.argtypes = [vp, vp, vp, vp, vp, vp]
        lib.cpu_set_state.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        lib.cpu_diagnostics.argtypes = [vp, dp]
        lib.cpu_threads.argtypes = [vp]
        lib.cpu_threads.restype = ip
        lib.cpu_r2c_plane.argtypes = [ip, ip, vp, vp]
        lib.cpu_c2r_plane.argtypes = [ip, ip, vp, vp]
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class CpuChannel:
    """One run of the C restatement; same step semantics as dns3d_ref.step."""

    def __init__(self, cfg, threads: int = 0):
        c = CpuConfig()
        for n, _ in CpuConfig._fields_:
            setattr(c, n, type(getattr(c, n))(getattr(cfg, n)) if isinstance(getattr(c, n), float)
                    else int(getattr(cfg, n)))
        self.lib = load()
        # the C restatement builds the analytical initial condition itself;
        # the random perturbation and the white noise come from dns3d_ref
        special = (cfg.enable_perturbations and not cfg.use_analytical_perturbations) or \
            getattr(cfg, "noise_amplitude", 0.0) > 0.0
        if special:
            c.enable_perturbations = 0
        self.h = self.lib.cpu_create(C.byref(c), int(threads))
        if not self.h:
            raise RuntimeError("cpu_create failed")
        self.shape = (cfg.nz, cfg.ny, cfg.nx)
        if special:
            from . import dns3d_ref as ref
            st = ref.initial_state(cfg, ref.setup_grid(cfg))
            self.set_state(u=st.u, v=st.v, w=st.w)

    @property
    def threads(self) -> int:
        return self.lib.cpu_threads(self.h)

    def step(self, n: int = 1) -> None:
        if self.lib.cpu_step(self.h, int(n)):
            raise RuntimeError("singular operator (the reference stops in zgesv)")

    def get_state(self) -> dict:
        out = {k: np.empty(self.shape) for k in ("u", "v", "w", "p_total")}
        pi = np.empty(7)
        self.lib.cpu_get_state(self.h, *[_p(out[k]) for k in ("u", "v", "w", "p_total")], _p(pi))
        out["pi"] = pi
        return out

    def set_state(self, u=None, v=None, w=None, p_total=None, gpx=None, gpy=None) -> None:
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (u, v, w, p_total, gpx, gpy)]
        self.lib.cpu_set_state(self.h, *[_p(a) for a in arrs])

    def diagnostics(self) -> dict:
        o = np.empty(8)
        self.lib.cpu_diagnostics(self.h, o.ctypes.data_as(C.POINTER(C.c_double)))
        return dict(zip(("umax", "vmax", "wmax", "energy", "dpdx", "u_bulk", "dpdx_avg", "max_div"), map(float, o)))

    def close(self) -> None:
        if self.h:
            self.lib.cpu_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


def r2c_plane(f: np.ndarray) -> np.ndarray:
    ny, nx = f.shape
    out = np.empty((ny, nx // 2 + 1), dtype=np.complex128)
    load().cpu_r2c_plane(nx, ny, _p(np.ascontiguousarray(f, dtype=np.float64)), _p(out))
    return out


def c2r_plane(F: np.ndarray, nx: int) -> np.ndarray:
    ny = F.shape[0]
    out = np.empty((ny, nx))
    load().cpu_c2r_plane(nx, ny, _p(np.ascontiguousarray(F, dtype=np.complex128)), _p(out))
    return out
