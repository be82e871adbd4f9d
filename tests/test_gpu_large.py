"""GPU: the large single run (512x384x129, PI control, dt 0.001, amplitude 0.08,
modes (2,2), seeded white noise 1e-3) -- the oracle is too slow at this size,
so the checks are size-independent properties; the white-noise initial
condition itself is pinned against the oracle on a small grid."""
import numpy as np
import pytest

from f90_dns_gb300 import ChannelDNS, config_from
from f90_dns_gb300.capi import PREC_MIXED
from f90_dns_gb300.workloads import WORKLOADS
from oracle import dns3d_ref as ref
from tests.helpers import oracle_config, velocity_errors

pytestmark = pytest.mark.gpu

BIG = WORKLOADS["channel_512x384x129_re180_pi"]


def test_white_noise_ic_matches_oracle_small(built_lib):
    wl = dict(BIG, nx=32, ny=24, nz=33, lgl_dmatrix_guard=True, perturbation_seed=5)
    with ChannelDNS(config_from(wl)) as d:
        g0 = d.get_state()
        d.step(10)
        gst = d.get_state()
    cfg = oracle_config(wl)
    g = ref.setup_grid(cfg)
    st = ref.initial_state(cfg, g)
    # the noise itself: the library's Philox stream is the oracle's
    for k in ("u", "v", "w"):
        assert np.max(np.abs(g0[k] - getattr(st, k))) <= 1e-14  # transform round trip of set_state
    assert np.max(np.abs(g0["w"][1:-1])) > 0.5e-3
    for _ in range(10):
        ref.step(cfg, g, st)
    err = velocity_errors(gst, st)
    assert max(err["u"], err["v"], err["w"]) <= 1e-10, err


@pytest.mark.parametrize("precision", [0, PREC_MIXED])
def test_large_run_properties(built_lib, precision):
    with ChannelDNS(config_from(BIG, precision=precision, noise_amplitude=0.0)) as d:
        d0 = d.diagnostics()
    with ChannelDNS(config_from(BIG, precision=precision)) as d:
        d.step(20)
        dg = d.diagnostics()
        st = d.get_state(walls=False)
    assert np.isfinite(dg.energy) and dg.step == 20
    # walls stay no-slip, the PI controller keeps the bulk velocity near its target
    for k in ("u", "v", "w"):
        assert np.max(np.abs(st[k][0])) == 0.0 and np.max(np.abs(st[k][-1])) == 0.0
    assert abs(dg.u_bulk - 2.0 / 3.0) < 2e-3
    assert 0.0 <= dg.dpdx <= 10.0
    # energy changes only slowly over 20 steps of dt 0.001
    assert abs(dg.energy - d0.energy) < 0.02 * d0.energy
    assert dg.vmax < 0.2 and dg.wmax < 0.2
