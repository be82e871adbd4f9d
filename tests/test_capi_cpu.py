"""CPU: the C-ABI library builds for sm_103a, loads, exports every symbol the
header declares, matches the header's struct layouts, and its host logic
(defaults, namelist reader, validation, error codes) behaves -- all without
touching a GPU."""
import ctypes as C
import os
import re
import subprocess

import pytest

from f90_dns_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "dns3d_capi.h")
GOLDEN = os.path.join(ROOT, "tests", "golden")


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dns3d_\w+)\s*\(", text)))


def test_library_exports_every_header_symbol(built_lib):
    names = header_functions()
    assert len(names) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", capi.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\sT\s(dns3d_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    assert set(names) == set(capi.EXPORTED_SYMBOLS)
    for n in names:
        assert getattr(built_lib, n) is not None


def test_library_contains_sm103a_code(built_lib):
    # the build passes exactly one -gencode for sm_103a; the fatbin section must exist
    out = subprocess.run(["readelf", "-S", capi.LIB_PATH], capture_output=True, text=True).stdout
    assert ".nv_fatbin" in out


STRUCTS = {
    "dns3d_restart_header": capi.CRestartHeader,
    "dns3d_server_opts": capi.CServerOpts,
    "dns3d_request_info": capi.CRequestInfo,
    "dns3d_server_stats": capi.CServerStats,
    "dns3d_config": capi.CConfig,
    "dns3d_pi_state": capi.CPIState,
    "dns3d_diag": capi.CDiag,
    "dns3d_kernel_time": capi.CKernelTime,
}


def test_struct_layouts_match_header(tmp_path):
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "dns3d_capi.h"', "int main(void){"]
    for cname, cls in STRUCTS.items():
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for line in res:
        if line.strip():
            a, b, c = line.split()
            got[(a, b)] = int(c)
    for cname, cls in STRUCTS.items():
        assert got[(cname, "sizeof")] == C.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)


def test_config_defaults_match_reference(built_lib):
    c = capi.default_config()
    # read_input_3d defaults (DNS_pressure_BC_3D.f90:571-603)
    assert (c.nx, c.ny, c.nz) == (128, 32, 33)
    assert c.istart == 0 and c.nsteps == 1000 and c.nwrt == 100 and c.restart_write_freq == 1000
    assert c.re == 180.0 and c.dt == 0.01 and c.u_centerline == 1.5
    assert abs(c.xlen - 2 * 3.141592653589793) < 1e-15 and c.use_crank_nicolson == 1
    assert c.flow_control_method == 1 and c.target_pressure_gradient == 0.03
    assert c.target_bulk_velocity == 1.0 and c.controller_gain == 0.15 and c.controller_update_freq == 7
    assert c.enable_perturbations == 0 and c.perturbation_amplitude == 0.01
    assert c.analytical_mode_x == 1 and c.analytical_mode_y == 1
    assert c.use_weak_form_divergence == 0 and c.use_dealias_23_rule == 0 and c.lgl_dmatrix_guard == 1


def test_namelist_reader(built_lib):
    c = capi.read_namelist(os.path.join(GOLDEN, "input_channel_32x32x33.dat"))
    assert (c.nx, c.ny, c.nz) == (32, 32, 33)
    assert c.dt == 2.0e-3 and c.nsteps == 100 and c.nwrt == 10
    assert c.re == 180.0 and c.u_centerline == 1.0 and c.use_crank_nicolson == 1
    assert abs(c.xlen - 12.566370614359172) < 1e-15 and abs(c.ylen - 6.283185307179586) < 1e-15
    assert c.flow_control_method == 1 and abs(c.target_pressure_gradient - 2 / 180) < 1e-17
    assert c.enable_perturbations == 1 and c.use_analytical_perturbations == 1
    assert c.use_dealias_23_rule == 1 and c.use_weak_form_divergence == 0


def test_namelist_partial_and_errors(built_lib, tmp_path):
    p = tmp_path / "partial.dat"
    p.write_text("&grid\n nx_input = 64, nz_input = 17\n/\n&flow_control\n flow_control_method = 2,\n"
                 " target_bulk_velocity = 0.6667\n/\n")
    c = capi.read_namelist(str(p))
    assert (c.nx, c.ny, c.nz) == (64, 32, 17)  # ny keeps its default
    assert c.flow_control_method == 2 and c.target_bulk_velocity == 0.6667
    seeded = tmp_path / "seeded.dat"
    seeded.write_text("&perturbations\n enable_perturbations = .true., use_analytical_perturbations = .false.,\n"
                      " perturbation_seed = 12345678901\n/\n")
    c = capi.read_namelist(str(seeded))
    assert c.perturbation_seed == 12345678901 and c.enable_perturbations == 1
    assert c.use_analytical_perturbations == 0
    bad = tmp_path / "bad.dat"
    bad.write_text("&grid\n nx_input = sixty\n/\n")
    with pytest.raises(capi.Dns3DError) as ei:
        capi.read_namelist(str(bad))
    assert ei.value.code == capi.DNS3D_E_IO
    with pytest.raises(capi.Dns3DError) as ei:
        capi.read_namelist(str(tmp_path / "missing.dat"))
    assert ei.value.code == capi.DNS3D_E_IO


@pytest.mark.parametrize("over,code", [
    (dict(flow_control_method=3), capi.DNS3D_E_INVALID),
    (dict(flow_control_method=2, controller_gain=0.0), capi.DNS3D_E_INVALID),
    (dict(flow_control_method=2, target_bulk_velocity=-1.0), capi.DNS3D_E_INVALID),
    (dict(flow_control_method=2, controller_update_freq=0), capi.DNS3D_E_INVALID),
    (dict(nx=100), capi.DNS3D_E_UNSUPPORTED),   # nx/2 = 50 is not 2^a 3^b
    (dict(ny=40), capi.DNS3D_E_UNSUPPORTED),
    (dict(nz=200), capi.DNS3D_E_UNSUPPORTED),
    (dict(precision=7), capi.DNS3D_E_UNSUPPORTED),
    (dict(dt=0.0), capi.DNS3D_E_INVALID),
])
def test_create_rejects_bad_config(built_lib, over, code):
    cfg = capi.default_config(**over)
    h = C.c_void_p()
    assert built_lib.dns3d_create(C.byref(cfg), C.byref(h)) == code
    assert not h.value


def _has_gpu():
    try:
        cudart = C.CDLL("libcudart.so")
        n = C.c_int(0)
        return cudart.cudaGetDeviceCount(C.byref(n)) == 0 and n.value > 0
    except OSError:
        return False


@pytest.mark.skipif(_has_gpu(), reason="a GPU is present")
def test_create_without_gpu_fails_loudly(built_lib):
    with pytest.raises(capi.Dns3DError) as ei:
        capi.ChannelDNS(capi.default_config(nx=32, ny=32, nz=17))
    assert ei.value.code == capi.DNS3D_E_NODEVICE


def test_noalloc_argument_checks_without_gpu(built_lib):
    buf = (C.c_double * 8)()
    p = C.cast(buf, C.c_void_p)
    assert built_lib.dns3d_flow_stats_noalloc(None, p, p, 4, 4, 9, p, None) == capi.DNS3D_E_INVALID
    assert built_lib.dns3d_flow_stats_noalloc(p, p, p, 4, 4, 130, p, None) == capi.DNS3D_E_UNSUPPORTED


def test_footprint_and_strerror(built_lib):
    small = capi.footprint_bytes(capi.default_config(nx=32, ny=32, nz=33))
    big = capi.footprint_bytes(capi.default_config(nx=128, ny=128, nz=65))
    assert 0 < small < big
    # 17 spectral + 6 physical fields and the 2 sets of folded per-mode inverses dominate
    assert big > 2 * 65 * 65 * (33 * 33 + 32 * 32) * 8
    assert capi.strerror(capi.DNS3D_E_SINGULAR) == "singular per-mode operator"
    assert capi.strerror(12345) == "unknown error"


def test_null_handle_is_rejected(built_lib):
    for n in ("dns3d_compute_source_terms", "dns3d_viscous_step", "dns3d_solve_pressure",
              "dns3d_pressure_correction", "dns3d_apply_boundary_conditions", "dns3d_destroy"):
        assert getattr(built_lib, n)(None) == capi.DNS3D_E_INVALID
    assert built_lib.dns3d_step(None, 1) == capi.DNS3D_E_INVALID


@pytest.mark.skipif(_has_gpu(), reason="a GPU is present")
def test_server_host_logic_without_gpu(built_lib):
    """Queueing, failure reporting, waits and shutdown of the serving loop work
    on a host without a GPU: every request fails with DNS3D_E_NODEVICE."""
    cfg = capi.default_config(nx=32, ny=32, nz=17)
    with capi.Server(max_runs=2) as srv:
        ids = [srv.submit(cfg, 5) for _ in range(4)]
        infos = [srv.wait(i, timeout=30.0) for i in ids]
        for inf in infos:
            assert inf.status == capi.REQ_FAILED and inf.error == capi.DNS3D_E_NODEVICE
            assert inf.t_finish >= inf.t_submit >= 0.0
        st = srv.stats()
        assert st["queued"] == 0 and st["running"] == 0 and st["bytes_in_use"] == 0
        srv.release(ids[0])
        with pytest.raises(capi.Dns3DError):
            srv.poll(ids[0])


def test_server_rejects_request_larger_than_budget(built_lib):
    cfg = capi.default_config(nx=128, ny=128, nz=65, lgl_dmatrix_guard=0)
    with capi.Server(max_bytes=1 << 20) as srv:
        with pytest.raises(capi.Dns3DError) as ei:
            srv.submit(cfg, 10)
        assert ei.value.code == capi.DNS3D_E_OOM


def test_ctypes_structs_match_the_c_layout(tmp_path):
    """Every struct the Python binding mirrors has the C compiler's size and
    field offsets (a mismatch would make the library read past the end)."""
    import ctypes as C
    import shutil
    import subprocess

    from f90_dns_gb300 import capi
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no gcc")
    pairs = [("dns3d_config", capi.CConfig), ("dns3d_pi_state", capi.CPIState), ("dns3d_diag", capi.CDiag),
             ("dns3d_kernel_time", capi.CKernelTime), ("dns3d_server_opts", capi.CServerOpts),
             ("dns3d_request_info", capi.CRequestInfo), ("dns3d_server_stats", capi.CServerStats),
             ("dns3d_restart_header", capi.CRestartHeader), ("dns3d_flow_stats", capi.CFlowStats)]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "dns3d_capi.h"', 'int main(void) {']
    for cname, py in pairs:
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([gcc, "-I", inc, str(src), "-o", str(exe)], check=True)
    got = dict(ln.split() for ln in subprocess.run([str(exe)], capture_output=True, text=True,
                                                    check=True).stdout.splitlines())
    for cname, py in pairs:
        assert int(got[cname]) == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(got[f"{cname}.{f}"]) == getattr(py, f).offset, (cname, f)
