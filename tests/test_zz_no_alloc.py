"""dns3d_flow_stats_noalloc: the allocation-free statistics entry point.

It serves callers that may not let a library allocate device memory (their own
pool owns the GPU, or their memory budget is fixed), so it must give the same
max|u|, max|v|, max|w| and kinetic energy as dns3d_diagnostics() on a handle
while using only its built-in scratch array.  Two calls in a row check that
the second call is not affected by what the first left in that shared array.
This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from f90_dns_gb300 import ChannelDNS, config_from
from f90_dns_gb300.workloads import WORKLOADS

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _noalloc_stats(lib, u, v, w):
    torch = pytest.importorskip("torch")
    nz, ny, nx = u.shape
    du, dv, dw = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (u, v, w))
    out = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    rc = lib.dns3d_flow_stats_noalloc(C.c_void_p(du.data_ptr()), C.c_void_p(dv.data_ptr()),
                                      C.c_void_p(dw.data_ptr()), nx, ny, nz, C.c_void_p(out.data_ptr()),
                                      C.c_void_p(stream.cuda_stream))
    assert rc == 0, rc
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _close(a, b):
    return abs(a - b) <= RTOL * max(abs(a), abs(b), 1e-300)


def test_noalloc_stats_match_diagnostics_twice(built_lib):
    wl = dict(WORKLOADS["channel_32x32x33_re180_dpdx"], nx=48, ny=32, nz=33)
    rng = np.random.default_rng(11)
    shp = (33, 32, 48)
    with ChannelDNS(config_from(wl)) as d:
        u = rng.standard_normal(shp)
        v = 0.1 * rng.standard_normal(shp)
        w = 0.01 * rng.standard_normal(shp)
        d.set_state(u=u, v=v, w=w)
        for call in range(2):
            st = d.get_state(walls=False)
            ref = d.diagnostics()
            got = _noalloc_stats(built_lib, st["u"], st["v"], st["w"])
            for i, k in enumerate(("umax", "vmax", "wmax", "energy")):
                assert _close(got[i], getattr(ref, k)), (call, k, got[i], getattr(ref, k))
            d.step(1)  # second call sees a different state


def test_noalloc_rejects_oversized_nz(built_lib):
    torch = pytest.importorskip("torch")
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    assert built_lib.dns3d_flow_stats_noalloc(p, p, p, 2, 2, 4000, p, None) == 6  # DNS3D_E_UNSUPPORTED


def test_noalloc_reports_nan(built_lib):
    """A NaN in a field must reach out4: the maxima keep NaN, so a blown-up
    state is not reported with finite maxima."""
    rng = np.random.default_rng(5)
    shp = (17, 8, 16)
    u, v, w = (rng.standard_normal(shp) for _ in range(3))
    v[3, 2, 5] = np.nan
    got = _noalloc_stats(built_lib, u, v, w)
    assert np.isfinite(got[0]) and np.isnan(got[1]) and np.isfinite(got[2]) and np.isnan(got[3]), got
    v[3, 2, 5] = 0.0
    got = _noalloc_stats(built_lib, u, v, w)  # the shared scratch keeps no NaN from the call before
    assert np.all(np.isfinite(got)), got
