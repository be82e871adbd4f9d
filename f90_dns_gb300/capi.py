"""ctypes binding of ``libdns3d_gpu.so`` and a host-side mirror of the
reference's time-loop interface.

The reference program (``DNS_pressure_BC_3D.f90``) advances the flow with five
argument-less subroutines called in a fixed order from its time loop
(DNS_pressure_BC_3D.f90:314-326).  :class:`ChannelDNS` exposes the same five
names as methods over one GPU handle, plus ``step(n)`` for the fused,
graph-replayed loop body, state transfer and diagnostics.

There is no CPU fallback: if the shared library is missing or no GPU is
present, constructing :class:`ChannelDNS` raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, fields as dc_fields

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libdns3d_gpu.so")

DNS3D_OK = 0
DNS3D_E_INVALID = 1
DNS3D_E_OOM = 2
DNS3D_E_SINGULAR = 3
DNS3D_E_NONFINITE = 4
DNS3D_E_CUDA = 5
DNS3D_E_UNSUPPORTED = 6
DNS3D_E_IO = 7
DNS3D_E_NODEVICE = 8
DNS3D_E_TIMEOUT = 9
DNS3D_E_CANCELLED = 10
REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = 0, 1, 2, 3
PREC_FP64 = 0
PREC_MIXED = 1

#: every symbol declared in include/dns3d_capi.h
EXPORTED_SYMBOLS = (
    "dns3d_config_defaults", "dns3d_config_read_namelist", "dns3d_create", "dns3d_destroy",
    "dns3d_initialize_fields", "dns3d_set_state", "dns3d_get_state", "dns3d_set_clock",
    "dns3d_compute_source_terms", "dns3d_viscous_step", "dns3d_solve_pressure",
    "dns3d_pressure_correction", "dns3d_apply_boundary_conditions", "dns3d_step",
    "dns3d_synchronize", "dns3d_query", "dns3d_diagnostics", "dns3d_output_diagnostics", "dns3d_check_divergence",
    "dns3d_projection_residual", "dns3d_footprint_bytes", "dns3d_strerror",
    "dns3d_last_error", "dns3d_step_timed", "dns3d_profile_kernels", "dns3d_launches_per_step",
    "dns3d_measure_fp64_tflops", "dns3d_check_conversions", "dns3d_flow_stats_noalloc",
    "dns3d_ensemble_create", "dns3d_ensemble_destroy", "dns3d_ensemble_size", "dns3d_ensemble_run",
    "dns3d_ensemble_step", "dns3d_ensemble_step_timed", "dns3d_ensemble_info",
    "dns3d_batch_create", "dns3d_batch_step", "dns3d_batch_synchronize", "dns3d_batch_query", "dns3d_batch_info",
    "dns3d_batch_destroy",
    "dns3d_server_opts_defaults", "dns3d_server_create", "dns3d_server_submit", "dns3d_server_poll",
    "dns3d_server_wait", "dns3d_server_result_state", "dns3d_server_release", "dns3d_server_get_stats",
    "dns3d_server_destroy", "dns3d_restart_write", "dns3d_restart_read", "dns3d_save_restart",
    "dns3d_load_restart", "dns3d_get_config", "dns3d_get_clock", "dns3d_lgl_nodes_weights",
    "dns3d_flow_statistics", "dns3d_output_init", "dns3d_output_time_series_row",
    "dns3d_output_flow_statistics", "dns3d_output_spanwise_profile", "dns3d_output_velocity_snapshot",
    "dns3d_output_simulation_summary", "dns3d_write_time_series_data", "dns3d_write_flow_statistics",
    "dns3d_write_spanwise_averaged_profile", "dns3d_write_velocity_field_snapshot",
    "dns3d_autotune", "dns3d_set_tiles",
)

TILE_KERNELS = ("vorticity", "viscous", "pressure", "correction", "divergence", "vorticity_mixed",
                "viscous_mixed", "pressure_mixed")


class CConfig(C.Structure):
    """``dns3d_config`` (field order of include/dns3d_capi.h)."""

    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("istart", C.c_int), ("nsteps", C.c_int), ("nwrt", C.c_int), ("restart_write_freq", C.c_int),
        ("dt", C.c_double),
        ("re", C.c_double), ("xlen", C.c_double), ("ylen", C.c_double), ("u_centerline", C.c_double),
        ("use_crank_nicolson", C.c_int),
        ("flow_control_method", C.c_int),
        ("target_pressure_gradient", C.c_double), ("target_bulk_velocity", C.c_double),
        ("controller_gain", C.c_double),
        ("controller_update_freq", C.c_int),
        ("enable_perturbations", C.c_int),
        ("perturbation_amplitude", C.c_double),
        ("zero_w_perturbations", C.c_int), ("use_analytical_perturbations", C.c_int),
        ("analytical_mode_x", C.c_int), ("analytical_mode_y", C.c_int),
        ("use_weak_form_divergence", C.c_int),
        ("use_dealias_23_rule", C.c_int),
        ("lgl_dmatrix_guard", C.c_int),
        ("precision", C.c_int),
        ("device", C.c_int),
        ("perturbation_seed", C.c_longlong),
        ("convection_scheme", C.c_int), ("linear_solver", C.c_int),
        ("cgstol", C.c_double),
        ("noise_amplitude", C.c_double),
        ("poisson_refinement", C.c_int), ("pad_", C.c_int),
    ]


class CPIState(C.Structure):
    _fields_ = [
        ("current_pressure_gradient", C.c_double), ("current_bulk_velocity", C.c_double),
        ("bulk_velocity_error", C.c_double), ("bulk_velocity_error_integral", C.c_double),
        ("bulk_velocity_error_prev", C.c_double), ("pressure_gradient_sum", C.c_double),
        ("avg_pressure_gradient", C.c_double), ("pressure_gradient_count", C.c_int),
        ("pad_", C.c_int),
    ]


class CDiag(C.Structure):
    _fields_ = [
        ("umax", C.c_double), ("vmax", C.c_double), ("wmax", C.c_double), ("energy", C.c_double),
        ("u_bulk", C.c_double), ("dpdx", C.c_double), ("dpdx_avg", C.c_double),
        ("max_div", C.c_double), ("time", C.c_double), ("step", C.c_int), ("pad_", C.c_int),
    ]


class CKernelTime(C.Structure):
    _fields_ = [("name", C.c_char_p), ("launches", C.c_int), ("pad_", C.c_int), ("total_ms", C.c_double)]


class CServerOpts(C.Structure):
    _fields_ = [("max_bytes", C.c_ulonglong), ("max_runs", C.c_int), ("steps_per_round", C.c_int),
                ("device", C.c_int), ("pad_", C.c_int)]


class CRequestInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("error", C.c_int), ("steps_done", C.c_int), ("nsteps", C.c_int),
                ("bytes", C.c_ulonglong), ("t_submit", C.c_double), ("t_start", C.c_double),
                ("t_finish", C.c_double), ("diag", CDiag)]


class CServerStats(C.Structure):
    _fields_ = [("queued", C.c_int), ("running", C.c_int), ("bytes_in_use", C.c_ulonglong),
                ("point_steps_done", C.c_ulonglong), ("uptime_s", C.c_double)]


class CRestartHeader(C.Structure):
    _fields_ = [("istep", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("time", C.c_double), ("dt", C.c_double), ("re", C.c_double), ("alpha", C.c_double),
                ("beta", C.c_double)]


class CFlowStats(C.Structure):
    """``dns3d_flow_stats``: the numbers of the reference's output files."""

    _fields_ = [
        ("umax", C.c_double), ("vmax", C.c_double), ("wmax", C.c_double), ("energy", C.c_double),
        ("bulk_velocity", C.c_double), ("dpdx", C.c_double), ("dpdx_avg", C.c_double),
        ("wall_shear_lower", C.c_double), ("wall_shear_upper", C.c_double),
        ("friction_velocity_avg", C.c_double), ("re_tau", C.c_double), ("time", C.c_double),
        ("step", C.c_int), ("flow_control_method", C.c_int),
    ]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


class Dns3DError(RuntimeError):
    """A non-zero status from the C-ABI (the reference would ``stop`` here)."""

    def __init__(self, code: int, where: str, detail: str = ""):
        self.code = code
        msg = f"{where}: {strerror(code)} (status {code})"
        if detail:
            msg += f": {detail}"
        super().__init__(msg)


_lib = None


def load_library(path: str | None = None) -> C.CDLL:
    """Load ``libdns3d_gpu.so`` (built by ``f90_dns_gb300.build``)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"{p} is missing: build it with `python -m f90_dns_gb300.build`")
    lib = C.CDLL(p)
    vp, ip, dp = C.c_void_p, C.c_int, C.POINTER(C.c_double)
    hp = C.c_void_p
    lib.dns3d_config_defaults.argtypes = [C.POINTER(CConfig)]
    lib.dns3d_config_read_namelist.argtypes = [C.c_char_p, C.POINTER(CConfig)]
    lib.dns3d_create.argtypes = [C.POINTER(CConfig), C.POINTER(hp)]
    lib.dns3d_destroy.argtypes = [hp]
    lib.dns3d_initialize_fields.argtypes = [hp]
    lib.dns3d_set_state.argtypes = [hp] + [vp] * 8 + [C.POINTER(CPIState)]
    lib.dns3d_get_state.argtypes = [hp] + [vp] * 8 + [C.POINTER(CPIState)]
    lib.dns3d_set_clock.argtypes = [hp, ip, C.c_double]
    for n in ("dns3d_compute_source_terms", "dns3d_viscous_step", "dns3d_solve_pressure",
              "dns3d_pressure_correction", "dns3d_apply_boundary_conditions", "dns3d_synchronize"):
        getattr(lib, n).argtypes = [hp]
    lib.dns3d_step.argtypes = [hp, ip]
    lib.dns3d_diagnostics.argtypes = [hp, C.POINTER(CDiag)]
    lib.dns3d_output_diagnostics.argtypes = [hp, C.POINTER(CDiag)]
    lib.dns3d_check_divergence.argtypes = [hp, C.POINTER(C.c_double)]
    lib.dns3d_projection_residual.argtypes = [hp, C.POINTER(C.c_double)]
    lib.dns3d_footprint_bytes.argtypes = [C.POINTER(CConfig), C.POINTER(C.c_ulonglong)]
    lib.dns3d_strerror.argtypes = [ip]
    lib.dns3d_strerror.restype = C.c_char_p
    lib.dns3d_step_timed.argtypes = [hp, ip, C.POINTER(C.c_double)]
    lib.dns3d_profile_kernels.argtypes = [hp, ip, C.POINTER(CKernelTime), ip, C.POINTER(C.c_int)]
    lib.dns3d_launches_per_step.argtypes = [hp, C.POINTER(C.c_int)]
    lib.dns3d_measure_fp64_tflops.argtypes = [ip, C.POINTER(C.c_double)]
    lib.dns3d_check_conversions.argtypes = [ip, C.c_longlong, C.POINTER(C.c_ulonglong)]
    lib.dns3d_flow_stats_noalloc.argtypes = [vp, vp, vp, ip, ip, ip, vp, vp]
    lib.dns3d_ensemble_create.argtypes = [C.POINTER(CConfig), ip, C.POINTER(hp)]
    lib.dns3d_ensemble_destroy.argtypes = [hp]
    lib.dns3d_ensemble_size.argtypes = [hp, C.POINTER(C.c_int)]
    lib.dns3d_ensemble_run.argtypes = [hp, ip, C.POINTER(hp)]
    lib.dns3d_ensemble_step.argtypes = [hp, ip]
    lib.dns3d_ensemble_step_timed.argtypes = [hp, ip, C.POINTER(C.c_double)]
    lib.dns3d_ensemble_info.argtypes = [hp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.dns3d_batch_create.argtypes = [C.POINTER(hp), ip, ip, C.POINTER(hp)]
    lib.dns3d_batch_step.argtypes = [hp, ip]
    lib.dns3d_batch_synchronize.argtypes = [hp]
    lib.dns3d_batch_query.argtypes = [hp, C.POINTER(C.c_int)]
    lib.dns3d_query.argtypes = [hp, C.POINTER(C.c_int)]
    lib.dns3d_batch_info.argtypes = [hp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.dns3d_batch_destroy.argtypes = [hp]
    lib.dns3d_server_opts_defaults.argtypes = [C.POINTER(CServerOpts)]
    lib.dns3d_server_create.argtypes = [C.POINTER(CServerOpts), C.POINTER(hp)]
    lib.dns3d_server_submit.argtypes = [hp, C.POINTER(CConfig), ip, ip, C.POINTER(C.c_longlong)]
    lib.dns3d_server_poll.argtypes = [hp, C.c_longlong, C.POINTER(CRequestInfo)]
    lib.dns3d_server_wait.argtypes = [hp, C.c_longlong, C.c_double, C.POINTER(CRequestInfo)]
    lib.dns3d_server_result_state.argtypes = [hp, C.c_longlong, vp, vp, vp, vp]
    lib.dns3d_server_release.argtypes = [hp, C.c_longlong]
    lib.dns3d_server_get_stats.argtypes = [hp, C.POINTER(CServerStats)]
    lib.dns3d_server_destroy.argtypes = [hp]
    lib.dns3d_restart_write.argtypes = [C.c_char_p, C.POINTER(CRestartHeader)] + [vp] * 7 + [C.POINTER(CPIState)]
    lib.dns3d_restart_read.argtypes = [C.c_char_p, C.POINTER(CRestartHeader)] + [vp] * 7 + [C.POINTER(CPIState)]
    lib.dns3d_save_restart.argtypes = [hp, C.c_char_p, ip, C.c_double]
    lib.dns3d_load_restart.argtypes = [hp, C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    lib.dns3d_get_config.argtypes = [hp, C.POINTER(CConfig)]
    lib.dns3d_get_clock.argtypes = [hp, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    lib.dns3d_lgl_nodes_weights.argtypes = [ip, vp, vp]
    lib.dns3d_flow_statistics.argtypes = [hp, C.POINTER(CFlowStats), vp, vp, vp]
    lib.dns3d_output_init.argtypes = [C.c_char_p]
    lib.dns3d_output_time_series_row.argtypes = [C.c_char_p, C.POINTER(CFlowStats)]
    lib.dns3d_output_flow_statistics.argtypes = [C.c_char_p, C.POINTER(CFlowStats)]
    lib.dns3d_output_spanwise_profile.argtypes = [C.c_char_p, ip, C.c_double, ip, vp, vp, vp, vp]
    lib.dns3d_output_velocity_snapshot.argtypes = [C.c_char_p, ip, C.c_double, ip, ip, ip, C.c_double,
                                                   C.c_double, vp, vp, vp, vp]
    lib.dns3d_output_simulation_summary.argtypes = [C.c_char_p, C.POINTER(CConfig), C.c_char_p, C.c_char_p,
                                                    C.c_char_p, ip, ip, C.c_double]
    for n in ("dns3d_write_time_series_data", "dns3d_write_flow_statistics",
              "dns3d_write_spanwise_averaged_profile", "dns3d_write_velocity_field_snapshot"):
        getattr(lib, n).argtypes = [hp, C.c_char_p]
    lib.dns3d_autotune.argtypes = [hp, ip, C.POINTER(C.c_int), ip]
    lib.dns3d_set_tiles.argtypes = [hp, C.POINTER(C.c_int), ip]
    lib.dns3d_last_error.argtypes = [hp]
    lib.dns3d_last_error.restype = C.c_char_p
    for n in EXPORTED_SYMBOLS:
        if n not in ("dns3d_strerror", "dns3d_last_error"):
            getattr(lib, n).restype = ip
    del dp
    if path is None:
        _lib = lib
    return lib


def strerror(code: int) -> str:
    try:
        return load_library().dns3d_strerror(code).decode()
    except Exception:  # pragma: no cover - library absent
        return f"status {code}"


def default_config(**overrides) -> CConfig:
    """``dns3d_config`` with the reference defaults (3D:571-603) and overrides."""
    cfg = CConfig()
    rc = load_library().dns3d_config_defaults(C.byref(cfg))
    if rc:
        raise Dns3DError(rc, "dns3d_config_defaults")
    for k, v in overrides.items():
        if not hasattr(cfg, k):
            raise KeyError(k)
        setattr(cfg, k, int(v) if isinstance(v, bool) else v)
    return cfg


def read_namelist(path: str, base: CConfig | None = None) -> CConfig:
    """Parse an ``input.dat`` with the eight namelist groups of read_input_3d."""
    cfg = base if base is not None else default_config()
    rc = load_library().dns3d_config_read_namelist(os.fsencode(path), C.byref(cfg))
    if rc:
        raise Dns3DError(rc, "dns3d_config_read_namelist", path)
    return cfg


def config_from(obj, **overrides) -> CConfig:
    """Build a ``dns3d_config`` from any object/dict carrying namelist names."""
    cfg = default_config()
    src = obj if isinstance(obj, dict) else {f.name: getattr(obj, f.name) for f in dc_fields(obj)}
    names = {n for n, _ in CConfig._fields_}
    for k, v in src.items():
        if k in names:
            setattr(cfg, k, int(v) if isinstance(v, bool) else v)
    for k, v in overrides.items():
        setattr(cfg, k, int(v) if isinstance(v, bool) else v)
    return cfg


def measure_fp64_tflops(device: int = 0) -> float:
    out = C.c_double(0.0)
    rc = load_library().dns3d_measure_fp64_tflops(int(device), C.byref(out))
    if rc:
        raise Dns3DError(rc, "dns3d_measure_fp64_tflops")
    return float(out.value)


def footprint_bytes(cfg: CConfig) -> int:
    out = C.c_ulonglong(0)
    rc = load_library().dns3d_footprint_bytes(C.byref(cfg), C.byref(out))
    if rc:
        raise Dns3DError(rc, "dns3d_footprint_bytes")
    return int(out.value)


@dataclass
class Diagnostics:
    umax: float
    vmax: float
    wmax: float
    energy: float
    u_bulk: float
    dpdx: float
    dpdx_avg: float
    max_div: float
    time: float
    step: int


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class ChannelDNS:
    """One channel-flow run resident on a GPU (the reference program's state).

    Arrays are numpy ``float64`` of shape ``(nz, ny, nx)``: the memory order of
    the reference's Fortran ``u(nx,ny,nz)``.
    """

    def __init__(self, cfg: CConfig, _handle=None):
        self.lib = load_library()
        self.cfg = cfg
        self._owned = _handle is None
        if _handle is not None:
            self._h = _handle
        else:
            self._h = C.c_void_p()
            rc = self.lib.dns3d_create(C.byref(cfg), C.byref(self._h))
            if rc:
                raise Dns3DError(rc, "dns3d_create")
        self.shape = (cfg.nz, cfg.ny, cfg.nx)

    # -- lifetime -------------------------------------------------------------
    def close(self) -> None:
        if self._h and self._owned:
            self.lib.dns3d_destroy(self._h)
        self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int, where: str) -> None:
        if rc:
            raise Dns3DError(rc, where, self.lib.dns3d_last_error(self._h).decode())

    # -- the reference's five time-loop subroutines (3D:314-326) -------------
    def compute_source_terms_3d(self) -> None:
        self._check(self.lib.dns3d_compute_source_terms(self._h), "compute_source_terms_3d")

    def viscous_step_3d(self) -> None:
        self._check(self.lib.dns3d_viscous_step(self._h), "viscous_step_3d")

    def solve_pressure_3d(self) -> None:
        self._check(self.lib.dns3d_solve_pressure(self._h), "solve_pressure_3d")

    def pressure_correction_3d(self) -> None:
        self._check(self.lib.dns3d_pressure_correction(self._h), "pressure_correction_3d")

    def apply_boundary_conditions_3d(self) -> None:
        self._check(self.lib.dns3d_apply_boundary_conditions(self._h), "apply_boundary_conditions_3d")

    # -- fused loop body --------------------------------------------------------
    def step(self, nsteps: int = 1) -> None:
        self._check(self.lib.dns3d_step(self._h, int(nsteps)), "dns3d_step")

    def step_timed(self, nsteps: int) -> float:
        """Run ``nsteps`` graph replays bracketed by CUDA events; device ms."""
        ms = C.c_double(0.0)
        self._check(self.lib.dns3d_step_timed(self._h, int(nsteps), C.byref(ms)), "dns3d_step_timed")
        return float(ms.value)

    def profile_kernels(self, nsteps: int) -> dict:
        """Per-kernel {name: (launches, total_ms)} over ``nsteps`` eager loop bodies."""
        buf = (CKernelTime * 64)()
        n = C.c_int(0)
        self._check(self.lib.dns3d_profile_kernels(self._h, int(nsteps), buf, 64, C.byref(n)),
                    "dns3d_profile_kernels")
        return {buf[i].name.decode(): (buf[i].launches, buf[i].total_ms) for i in range(n.value)}

    def launches_per_step(self) -> int:
        n = C.c_int(0)
        self._check(self.lib.dns3d_launches_per_step(self._h, C.byref(n)), "dns3d_launches_per_step")
        return int(n.value)

    def synchronize(self) -> None:
        self._check(self.lib.dns3d_synchronize(self._h), "dns3d_synchronize")

    def initialize_fields_3d(self) -> None:
        self._check(self.lib.dns3d_initialize_fields(self._h), "initialize_fields_3d")

    def set_clock(self, step: int, time: float) -> None:
        self._check(self.lib.dns3d_set_clock(self._h, int(step), float(time)), "dns3d_set_clock")

    # -- state ------------------------------------------------------------------
    def get_state(self, walls: bool = True) -> dict:
        nz, ny, nx = self.shape
        out = {k: np.empty(self.shape) for k in ("u", "v", "w", "p_total")}
        gp = {k: np.empty((ny, nx)) for k in ("gpx_w1", "gpx_w2", "gpy_w1", "gpy_w2")} if walls else {}
        pi = CPIState()
        rc = self.lib.dns3d_get_state(self._h, _ptr(out["u"]), _ptr(out["v"]), _ptr(out["w"]),
                                      _ptr(out["p_total"]), _ptr(gp.get("gpx_w1")),
                                      _ptr(gp.get("gpx_w2")), _ptr(gp.get("gpy_w1")),
                                      _ptr(gp.get("gpy_w2")), C.byref(pi))
        self._check(rc, "dns3d_get_state")
        out.update(gp)
        out["pi"] = {n: getattr(pi, n) for n, _ in CPIState._fields_ if n != "pad_"}
        return out

    def get_state_into(self, u=None, v=None, w=None, p_total=None) -> None:
        """Copy u, v, w, p_total into caller-owned contiguous float64 arrays
        (e.g. pinned host buffers); None skips a field."""
        for a in (u, v, w, p_total):
            if a is not None and (a.dtype != np.float64 or not a.flags.c_contiguous or a.shape != self.shape):
                raise ValueError("arrays must be C-contiguous float64 of shape (nz, ny, nx)")
        rc = self.lib.dns3d_get_state(self._h, _ptr(u), _ptr(v), _ptr(w), _ptr(p_total),
                                      None, None, None, None, None)
        self._check(rc, "dns3d_get_state")

    def set_state(self, u=None, v=None, w=None, p_total=None, gpx_w1=None, gpx_w2=None,
                  gpy_w1=None, gpy_w2=None, pi: dict | None = None) -> None:
        def arr(a, shape):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.float64)
            if a.shape != shape:
                raise ValueError(f"expected shape {shape}, got {a.shape}")
            return a
        nz, ny, nx = self.shape
        f = [arr(x, self.shape) for x in (u, v, w, p_total)]
        g = [arr(x, (ny, nx)) for x in (gpx_w1, gpx_w2, gpy_w1, gpy_w2)]
        cpi = None
        if pi is not None:
            cpi = CPIState()
            for k, val in pi.items():
                setattr(cpi, k, val)
        rc = self.lib.dns3d_set_state(self._h, *[_ptr(x) for x in f], *[_ptr(x) for x in g],
                                      C.byref(cpi) if cpi is not None else None)
        self._check(rc, "dns3d_set_state")

    def save_restart(self, path: str, istep: int, time: float) -> None:
        """Write the state as a restart file in the reference's format."""
        self._check(self.lib.dns3d_save_restart(self._h, os.fsencode(path), int(istep), float(time)),
                    "dns3d_save_restart")

    def load_restart(self, path: str) -> tuple:
        """Load a restart file; returns (istep, time).  grad_p_prev stays zero,
        as in the reference's restart."""
        st, tm = C.c_int(0), C.c_double(0.0)
        self._check(self.lib.dns3d_load_restart(self._h, os.fsencode(path), C.byref(st), C.byref(tm)),
                    "dns3d_load_restart")
        return int(st.value), float(tm.value)

    def autotune(self, force: bool = False) -> dict:
        """Re-run the tile autotuner; returns the widths in use per kernel."""
        t = (C.c_int * len(TILE_KERNELS))()
        self._check(self.lib.dns3d_autotune(self._h, int(force), t, len(TILE_KERNELS)), "dns3d_autotune")
        return dict(zip(TILE_KERNELS, list(t)))

    def tiles(self) -> dict:
        """Tile widths in use per kernel (no tuning)."""
        t = (C.c_int * len(TILE_KERNELS))()
        self._check(self.lib.dns3d_autotune(self._h, -1, t, len(TILE_KERNELS)), "dns3d_autotune")
        return dict(zip(TILE_KERNELS, list(t)))

    def set_tiles(self, **widths) -> None:
        """Set tile widths by kernel name (0 = built-in heuristic)."""
        cur = self.tiles()
        cur.update(widths)
        t = (C.c_int * len(TILE_KERNELS))(*[int(cur[k]) for k in TILE_KERNELS])
        self._check(self.lib.dns3d_set_tiles(self._h, t, len(TILE_KERNELS)), "dns3d_set_tiles")

    def get_clock(self) -> tuple:
        st, tm = C.c_int(0), C.c_double(0.0)
        self._check(self.lib.dns3d_get_clock(self._h, C.byref(st), C.byref(tm)), "dns3d_get_clock")
        return int(st.value), float(tm.value)

    def flow_statistics(self, profiles: bool = False):
        """The numbers of write_flow_statistics / write_time_series_data
        (dict), and with ``profiles`` the plane means u_avg, v_avg, w_avg
        per level (arrays of nz)."""
        st = CFlowStats()
        nz = self.shape[0]
        prof = [np.empty(nz) for _ in range(3)] if profiles else [None] * 3
        rc = self.lib.dns3d_flow_statistics(self._h, C.byref(st), *[_ptr(a) for a in prof])
        if rc and rc != DNS3D_E_NONFINITE:
            self._check(rc, "dns3d_flow_statistics")
        out = st.as_dict()
        if profiles:
            out.update(u_avg=prof[0], v_avg=prof[1], w_avg=prof[2])
        return out

    def write_time_series_data(self, out_dir: str) -> None:
        self._write("dns3d_write_time_series_data", out_dir)

    def write_flow_statistics(self, out_dir: str) -> None:
        self._write("dns3d_write_flow_statistics", out_dir)

    def write_spanwise_averaged_profile(self, out_dir: str) -> None:
        self._write("dns3d_write_spanwise_averaged_profile", out_dir)

    def write_velocity_field_snapshot(self, out_dir: str) -> None:
        self._write("dns3d_write_velocity_field_snapshot", out_dir)

    def _write(self, fn: str, out_dir: str) -> None:
        rc = getattr(self.lib, fn)(self._h, os.fsencode(out_dir))
        if rc and rc != DNS3D_E_NONFINITE:
            self._check(rc, fn)

    def diagnostics(self) -> Diagnostics:
        d = CDiag()
        rc = self.lib.dns3d_diagnostics(self._h, C.byref(d))
        self._check(rc, "dns3d_diagnostics")
        return Diagnostics(d.umax, d.vmax, d.wmax, d.energy, d.u_bulk, d.dpdx, d.dpdx_avg,
                           d.max_div, d.time, d.step)

    def output_diagnostics_3d(self) -> Diagnostics:
        """output_diagnostics_3d alone (max_div = 0)."""
        d = CDiag()
        rc = self.lib.dns3d_output_diagnostics(self._h, C.byref(d))
        self._check(rc, "dns3d_output_diagnostics")
        return Diagnostics(d.umax, d.vmax, d.wmax, d.energy, d.u_bulk, d.dpdx, d.dpdx_avg,
                           d.max_div, d.time, d.step)

    def projection_residual(self) -> float:
        """Relative residual max|b - P phi| / max|b| of the last pressure
        solve's Galerkin Poisson system (the divergence the projection
        controls)."""
        v = C.c_double(0.0)
        self._check(self.lib.dns3d_projection_residual(self._h, C.byref(v)), "dns3d_projection_residual")
        return v.value

    def check_divergence_3d(self) -> float:
        """check_divergence_3d: max |div u| of the current state."""
        v = C.c_double(0.0)
        rc = self.lib.dns3d_check_divergence(self._h, C.byref(v))
        self._check(rc, "dns3d_check_divergence")
        return v.value


BATCH_TUNE = 1


class Batch:
    """Joint stepping of existing runs (``dns3d_batch``): every stage of the
    step is one ragged kernel launch over all eligible runs of a precision.
    The runs stay owned by the caller and must outlive the batch."""

    def __init__(self, runs, tune: bool = True):
        self.lib = load_library()
        self.runs = list(runs)
        arr = (C.c_void_p * len(self.runs))(*[r._h for r in self.runs])
        self._b = C.c_void_p()
        rc = self.lib.dns3d_batch_create(arr, len(self.runs), BATCH_TUNE if tune else 0, C.byref(self._b))
        if rc:
            msg = "; ".join(m for m in (self.lib.dns3d_last_error(r._h).decode() for r in self.runs) if m)
            raise Dns3DError(rc, "dns3d_batch_create", msg)

    def step(self, nsteps: int = 1) -> None:
        rc = self.lib.dns3d_batch_step(self._b, int(nsteps))
        if rc:
            raise Dns3DError(rc, "dns3d_batch_step")

    def synchronize(self) -> None:
        rc = self.lib.dns3d_batch_synchronize(self._b)
        if rc:
            raise Dns3DError(rc, "dns3d_batch_synchronize")

    def info(self) -> tuple[int, int]:
        """(kernel launches per step, runs in ragged launches)."""
        n, r = C.c_int(0), C.c_int(0)
        rc = self.lib.dns3d_batch_info(self._b, C.byref(n), C.byref(r))
        if rc:
            raise Dns3DError(rc, "dns3d_batch_info")
        return n.value, r.value

    def close(self) -> None:
        if self._b:
            self.lib.dns3d_batch_destroy(self._b)
            self._b = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Ensemble:
    """Independent runs of any grids advanced together: each stage of the
    step is one ragged kernel launch over all runs of a precision (runs with
    options outside the ragged stages keep their own launches), one CUDA graph
    per step.  ``run(i)`` is a view of run i (a :class:`ChannelDNS` that the
    ensemble owns)."""

    def __init__(self, cfgs):
        self.lib = load_library()
        self.cfgs = list(cfgs)
        arr = (CConfig * len(self.cfgs))(*self.cfgs)
        self._e = C.c_void_p()
        rc = self.lib.dns3d_ensemble_create(arr, len(self.cfgs), C.byref(self._e))
        if rc:
            raise Dns3DError(rc, "dns3d_ensemble_create")
        self._views = []
        for i, cfg in enumerate(self.cfgs):
            h = C.c_void_p()
            self._check(self.lib.dns3d_ensemble_run(self._e, i, C.byref(h)), "dns3d_ensemble_run")
            self._views.append(ChannelDNS(cfg, _handle=h))

    def _check(self, rc, where):
        if rc:
            msgs = []
            for i, v in enumerate(getattr(self, "_views", [])):
                m = self.lib.dns3d_last_error(v._h).decode() if v._h else ""
                if m:
                    msgs.append(f"run {i}: {m}")
            raise Dns3DError(rc, where, "; ".join(msgs))

    def __len__(self):
        return len(self.cfgs)

    def run(self, i: int) -> ChannelDNS:
        return self._views[i]

    def step(self, nsteps: int = 1) -> None:
        self._check(self.lib.dns3d_ensemble_step(self._e, int(nsteps)), "dns3d_ensemble_step")

    def step_timed(self, nsteps: int) -> float:
        ms = C.c_double(0.0)
        self._check(self.lib.dns3d_ensemble_step_timed(self._e, int(nsteps), C.byref(ms)),
                    "dns3d_ensemble_step_timed")
        return float(ms.value)

    def info(self) -> tuple[int, int]:
        """(kernel launches per step, runs in ragged launches)."""
        n, r = C.c_int(0), C.c_int(0)
        self._check(self.lib.dns3d_ensemble_info(self._e, C.byref(n), C.byref(r)), "dns3d_ensemble_info")
        return n.value, r.value

    def close(self) -> None:
        if self._e:
            for v in self._views:
                v._h = C.c_void_p()
            self.lib.dns3d_ensemble_destroy(self._e)
            self._e = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


@dataclass
class RequestInfo:
    status: int
    error: int
    steps_done: int
    nsteps: int
    bytes: int
    t_submit: float
    t_start: float
    t_finish: float
    diag: Diagnostics

    @property
    def latency(self) -> float:
        return self.t_finish - self.t_submit


def _info(ci: CRequestInfo) -> RequestInfo:
    d = ci.diag
    return RequestInfo(ci.status, ci.error, ci.steps_done, ci.nsteps, int(ci.bytes), ci.t_submit, ci.t_start,
                       ci.t_finish, Diagnostics(d.umax, d.vmax, d.wmax, d.energy, d.u_bulk, d.dpdx, d.dpdx_avg,
                                                d.max_div, d.time, d.step))


class Server:
    """Continuous-batching request loop over one GPU (see dns3d_server_* in
    include/dns3d_capi.h): submit runs, wait or poll, read final state."""

    def __init__(self, max_bytes: int | None = None, max_runs: int | None = None,
                 steps_per_round: int | None = None, device: int = 0):
        self.lib = load_library()
        o = CServerOpts()
        self.lib.dns3d_server_opts_defaults(C.byref(o))
        if max_bytes is not None:
            o.max_bytes = int(max_bytes)
        if max_runs is not None:
            o.max_runs = int(max_runs)
        if steps_per_round is not None:
            o.steps_per_round = int(steps_per_round)
        o.device = device
        self.opts = o
        self._s = C.c_void_p()
        rc = self.lib.dns3d_server_create(C.byref(o), C.byref(self._s))
        if rc:
            raise Dns3DError(rc, "dns3d_server_create")
        self._shapes = {}

    def submit(self, cfg: CConfig, nsteps: int, keep_state: bool = False) -> int:
        rid = C.c_longlong(0)
        rc = self.lib.dns3d_server_submit(self._s, C.byref(cfg), int(nsteps), int(keep_state), C.byref(rid))
        if rc:
            raise Dns3DError(rc, "dns3d_server_submit")
        self._shapes[rid.value] = (cfg.nz, cfg.ny, cfg.nx)
        return int(rid.value)

    def poll(self, rid: int) -> RequestInfo:
        ci = CRequestInfo()
        rc = self.lib.dns3d_server_poll(self._s, rid, C.byref(ci))
        if rc:
            raise Dns3DError(rc, "dns3d_server_poll")
        return _info(ci)

    def wait(self, rid: int, timeout: float = -1.0) -> RequestInfo:
        ci = CRequestInfo()
        rc = self.lib.dns3d_server_wait(self._s, rid, float(timeout), C.byref(ci))
        if rc:
            raise Dns3DError(rc, "dns3d_server_wait")
        return _info(ci)

    def result_state(self, rid: int) -> dict:
        shp = self._shapes[rid]
        out = {k: np.empty(shp) for k in ("u", "v", "w", "p_total")}
        rc = self.lib.dns3d_server_result_state(self._s, rid, *[_ptr(out[k]) for k in ("u", "v", "w", "p_total")])
        if rc:
            raise Dns3DError(rc, "dns3d_server_result_state")
        return out

    def release(self, rid: int) -> None:
        rc = self.lib.dns3d_server_release(self._s, rid)
        if rc:
            raise Dns3DError(rc, "dns3d_server_release")

    def stats(self) -> dict:
        st = CServerStats()
        self.lib.dns3d_server_get_stats(self._s, C.byref(st))
        return {n: getattr(st, n) for n, _ in CServerStats._fields_}

    def close(self) -> None:
        if self._s:
            self.lib.dns3d_server_destroy(self._s)
            self._s = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def restart_write(path: str, istep: int, time: float, dt: float, re: float, alpha: float, beta: float,
                  u, v, w, un=None, vn=None, wn=None, p_total=None, pi: dict | None = None) -> None:
    """Encode a restart file (no GPU); arrays (nz, ny, nx) float64."""
    nz, ny, nx = np.shape(u)
    hdr = CRestartHeader(istep, nx, ny, nz, time, dt, re, alpha, beta)
    arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (u, v, w, un, vn, wn, p_total)]
    cpi = None
    if pi is not None:
        cpi = CPIState()
        for k, val in pi.items():
            setattr(cpi, k, val)
    rc = load_library().dns3d_restart_write(os.fsencode(path), C.byref(hdr), *[_ptr(a) for a in arrs],
                                            C.byref(cpi) if cpi is not None else None)
    if rc:
        raise Dns3DError(rc, "dns3d_restart_write", path)


def restart_read(path: str, nx: int, ny: int, nz: int) -> dict:
    """Decode a restart file written for an nx x ny x nz grid (no GPU)."""
    hdr = CRestartHeader(0, nx, ny, nz, 0.0, 0.0, 0.0, 0.0, 0.0)
    out = {k: np.empty((nz, ny, nx)) for k in ("u", "v", "w", "un", "vn", "wn", "p_total")}
    pi = CPIState()
    rc = load_library().dns3d_restart_read(os.fsencode(path), C.byref(hdr),
                                           *[_ptr(out[k]) for k in ("u", "v", "w", "un", "vn", "wn", "p_total")],
                                           C.byref(pi))
    if rc:
        raise Dns3DError(rc, "dns3d_restart_read", path)
    out.update({n: getattr(hdr, n) for n, _ in CRestartHeader._fields_})
    out["pi"] = {n: getattr(pi, n) for n, _ in CPIState._fields_ if n != "pad_"}
    return out


# ---------------------------------------------------------------- output files

def lgl_nodes_weights(nz: int):
    """LGL nodes (ascending from -1) and weights of lgl_module.f90:30-80."""
    z, w = np.empty(nz), np.empty(nz)
    rc = load_library().dns3d_lgl_nodes_weights(int(nz), _ptr(z), _ptr(w))
    if rc:
        raise Dns3DError(rc, "dns3d_lgl_nodes_weights")
    return z, w


def _flow_stats(st) -> CFlowStats:
    if isinstance(st, CFlowStats):
        return st
    c = CFlowStats()
    for n, _ in CFlowStats._fields_:
        if n in st:
            setattr(c, n, st[n])
    return c


def _out_call(fn: str, *args) -> None:
    rc = getattr(load_library(), fn)(*args)
    if rc:
        raise Dns3DError(rc, fn)


def output_init(out_dir: str) -> None:
    """output_time_series.dat and flow_statistics.dat with their headers."""
    _out_call("dns3d_output_init", os.fsencode(out_dir))


def output_time_series_row(out_dir: str, stats) -> None:
    _out_call("dns3d_output_time_series_row", os.fsencode(out_dir), C.byref(_flow_stats(stats)))


def output_flow_statistics(out_dir: str, stats) -> None:
    _out_call("dns3d_output_flow_statistics", os.fsencode(out_dir), C.byref(_flow_stats(stats)))


def output_spanwise_profile(out_dir: str, istep: int, time: float, z, u_avg, v_avg, w_avg) -> None:
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (z, u_avg, v_avg, w_avg)]
    _out_call("dns3d_output_spanwise_profile", os.fsencode(out_dir), int(istep), float(time), len(arrs[0]),
              *[_ptr(a) for a in arrs])


def output_velocity_snapshot(out_dir: str, istep: int, time: float, xlen: float, ylen: float, z, u, v, w) -> None:
    """velocity_field_NNNNN.dat from arrays (nz, ny, nx)."""
    nz, ny, nx = np.shape(u)
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (z, u, v, w)]
    _out_call("dns3d_output_velocity_snapshot", os.fsencode(out_dir), int(istep), float(time), nx, ny, nz,
              float(xlen), float(ylen), *[_ptr(a) for a in arrs])


def output_simulation_summary(out_dir: str, cfg: CConfig, input_filename: str = "", output_directory=None,
                              restart_filename: str = "restart.dat", restarted: bool = False,
                              restart_step: int = 0, restart_time: float = 0.0) -> None:
    _out_call("dns3d_output_simulation_summary", os.fsencode(out_dir), C.byref(cfg), os.fsencode(input_filename),
              None if output_directory is None else os.fsencode(output_directory), os.fsencode(restart_filename),
              int(bool(restarted)), int(restart_step), float(restart_time))
