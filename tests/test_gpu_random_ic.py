"""GPU: the random solenoidal initial perturbation (perturbation_module.f90:
42-176, seeded) built by the library against the oracle's restatement, and
the first steps from it.  Bar: the fields agree to 1e-12 of the velocity
scale (transform round-off only), the 20-step runs to the FP64 parity bar
1e-10."""
import numpy as np
import pytest

from f90_dns_gb300 import ChannelDNS, config_from
from f90_dns_gb300.capi import PREC_MIXED
from f90_dns_gb300.workloads import WORKLOADS
from oracle import dns3d_ref as ref
from tests.helpers import oracle_config, velocity_errors

pytestmark = pytest.mark.gpu

C1 = WORKLOADS["channel_32x32x33_re180_dpdx"]


def _wl(**kw):
    wl = dict(C1, nx=32, ny=24, nz=17, use_analytical_perturbations=False, perturbation_amplitude=0.01,
              perturbation_seed=20250813)
    wl.update(kw)
    return wl


@pytest.mark.parametrize("zero_w", [False, True])
def test_random_initial_condition_matches_oracle(built_lib, zero_w):
    wl = _wl(zero_w_perturbations=zero_w)
    cfg = oracle_config(wl)
    g = ref.setup_grid(cfg)
    st = ref.initial_state(cfg, g)
    with ChannelDNS(config_from(wl)) as d:
        got = d.get_state()
    scale = max(np.max(np.abs(st.u)), np.max(np.abs(st.v)), np.max(np.abs(st.w)))
    for k in ("u", "v", "w"):
        assert np.max(np.abs(got[k] - getattr(st, k))) <= 1e-12 * scale, k
    assert (np.max(np.abs(got["w"])) == 0.0) == zero_w
    assert np.max(np.abs(got["v"])) > 1e-3


def test_random_seed_changes_the_field(built_lib):
    with ChannelDNS(config_from(_wl())) as a, ChannelDNS(config_from(_wl(perturbation_seed=7))) as b:
        ua, ub = a.get_state()["u"], b.get_state()["u"]
    assert np.max(np.abs(ua - ub)) > 1e-3


def test_steps_from_random_ic_match_oracle(built_lib):
    wl = _wl(perturbation_amplitude=0.05)
    with ChannelDNS(config_from(wl)) as d:
        d.step(20)
        got = d.get_state()
    cfg = oracle_config(wl)
    _, st, _ = ref.run(cfg, 20, record_every=20)
    err = velocity_errors(got, st)
    assert max(err["u"], err["v"], err["w"]) <= 1e-10, err


def test_mixed_from_random_ic(built_lib):
    wl = _wl(perturbation_amplitude=0.05)
    with ChannelDNS(config_from(wl)) as a, ChannelDNS(config_from(wl, precision=PREC_MIXED)) as b:
        a.step(20)
        b.step(20)
        sa, sb = a.get_state(), b.get_state()
    scale = max(np.max(np.abs(sa[k])) for k in ("u", "v", "w"))
    assert max(np.max(np.abs(sa[k] - sb[k])) for k in ("u", "v", "w")) <= 1e-6 * scale
