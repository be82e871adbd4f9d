"""CPU: restart files in the reference's format (write_restart_file_3d,
DNS_pressure_BC_3D.f90:2976-3038): an independent struct-level encoder that
follows the reference's write sequence must produce the same bytes."""
import struct

import numpy as np
import pytest

from f90_dns_gb300 import capi


def reference_layout_bytes(istep, time, dt, nx, ny, nz, re, alpha, beta, fields, pis):
    # write(...) 'DNS3D_RESTART_v1.0' / istep, time, dt / nx, ny, nz / re, alpha, beta /
    # u / v / w / un / vn / wn / p_total / 4 PI scalars -- stream, little-endian
    b = b"DNS3D_RESTART_v1.0" + struct.pack("<idd", istep, time, dt) + struct.pack("<iii", nx, ny, nz)
    b += struct.pack("<ddd", re, alpha, beta)
    for f in fields:
        b += np.asarray(f, dtype="<f8").tobytes(order="C")
    return b + struct.pack("<dddd", *pis)


def test_restart_bytes_match_reference_layout(built_lib, tmp_path):
    rng = np.random.default_rng(0)
    nz, ny, nx = 5, 4, 6
    fields = [rng.standard_normal((nz, ny, nx)) for _ in range(7)]
    pi = dict(current_pressure_gradient=0.0166, current_bulk_velocity=0.66, bulk_velocity_error_integral=1e-4,
              bulk_velocity_error_prev=-2e-5)
    path = tmp_path / "restart.dat"
    capi.restart_write(str(path), 42, 0.084, 0.002, 180.0, 0.5, 1.0, *fields, pi=pi)
    want = reference_layout_bytes(42, 0.084, 0.002, nx, ny, nz, 180.0, 0.5, 1.0, fields,
                                  [pi[k] for k in ("current_pressure_gradient", "current_bulk_velocity",
                                                   "bulk_velocity_error_integral", "bulk_velocity_error_prev")])
    assert path.read_bytes() == want
    back = capi.restart_read(str(path), nx, ny, nz)
    assert back["istep"] == 42 and back["time"] == 0.084 and back["dt"] == 0.002 and back["re"] == 180.0
    for k, f in zip(("u", "v", "w", "un", "vn", "wn", "p_total"), fields):
        assert np.array_equal(back[k], f)
    assert back["pi"]["bulk_velocity_error_prev"] == -2e-5


def test_restart_read_errors_and_short_file(built_lib, tmp_path):
    nz, ny, nx = 3, 2, 4
    f = [np.ones((nz, ny, nx))] * 7
    path = tmp_path / "r.dat"
    capi.restart_write(str(path), 1, 0.1, 0.1, 100.0, 1.0, 1.0, *f)
    with pytest.raises(capi.Dns3DError) as ei:  # grid mismatch: the reference ignores the file
        capi.restart_read(str(path), nx + 2, ny, nz)
    assert ei.value.code == capi.DNS3D_E_INVALID
    bad = tmp_path / "bad.dat"
    bad.write_bytes(b"NOT_A_RESTART_FILE" + path.read_bytes()[18:])
    with pytest.raises(capi.Dns3DError) as ei:
        capi.restart_read(str(bad), nx, ny, nz)
    assert ei.value.code == capi.DNS3D_E_IO
    short = tmp_path / "short.dat"
    short.write_bytes(path.read_bytes()[:-32])  # no PI scalars: the reader keeps its defaults
    back = capi.restart_read(str(short), nx, ny, nz)
    assert np.array_equal(back["p_total"], f[6])
