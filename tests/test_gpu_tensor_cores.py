"""GPU: the Crank-Nicolson viscous solve and the z-derivatives of the
vorticity, the pressure right-hand side and the projection on the tensor cores
(emulated FP64: 8 FP16 digit slices of the operators and right-hand sides,
exact FP32 tcgen05 accumulation, integer combination; about 2^-53 of the
operand scales) keep the plain path's parity bar against the oracle, agree
with the FP64-pipe kernels, and give the same bits in a batch as alone."""
import numpy as np
import pytest

from f90_dns_gb300 import ChannelDNS, Ensemble, config_from
from f90_dns_gb300.workloads import WORKLOADS, ensemble_draws
from oracle import dns3d_ref as ref
from tests.helpers import oracle_config, velocity_errors

pytestmark = pytest.mark.gpu

TOL = 1e-10
C1 = WORKLOADS["channel_32x32x33_re180_dpdx"]
C2 = WORKLOADS["channel_128x128x65_re180_pi"]


def _names(d):
    return set(d.profile_kernels(1))


@pytest.mark.parametrize("wl", [C1, dict(C1, nx=16, ny=24, nz=65, lgl_dmatrix_guard=False, flow_control_method=2,
                                          target_bulk_velocity=2.0 / 3.0, controller_gain=0.5,
                                          controller_update_freq=1),
                                dict(C1, nx=16, ny=16, nz=97, lgl_dmatrix_guard=False),
                                dict(C1, nx=16, ny=16, nz=129, lgl_dmatrix_guard=False, flow_control_method=2,
                                     target_bulk_velocity=2.0 / 3.0, perturbation_amplitude=0.05),
                                dict(C1, nx=24, ny=16, nz=17)])
def test_tensor_core_viscous_matches_oracle(built_lib, monkeypatch, wl):
    monkeypatch.setenv("DNS3D_TENSOR_CORES", "1")
    with ChannelDNS(config_from(wl)) as d:
        assert {"viscous_helmholtz_tc", "vorticity_tc", "pressure_poisson_tc", "pressure_correction_tc"} <= _names(d)
    with ChannelDNS(config_from(wl)) as d:
        d.step(50)
        gst = d.get_state()
        gdiag = d.diagnostics()
    cfg = oracle_config(wl)
    g, st, hist = ref.run(cfg, 50, record_every=50)
    err = velocity_errors(gst, st)
    assert max(err["u"], err["v"], err["w"]) <= TOL, err
    assert err["p_total"] <= TOL, err
    assert abs(gdiag.energy - hist[-1]["energy"]) <= TOL * hist[-1]["energy"]


def test_tensor_core_viscous_agrees_with_fp64_pipe(built_lib, monkeypatch):
    wl = dict(C2, nx=64, ny=64, noise_amplitude=0.0)
    out = {}
    for mode, names in (("1", {"viscous_helmholtz_tc", "vorticity_tc", "pressure_poisson_tc", "pressure_correction_tc"}),
                        ("0", {"viscous_helmholtz", "vorticity", "pressure_poisson", "pressure_correction"})):
        monkeypatch.setenv("DNS3D_TENSOR_CORES", mode)
        with ChannelDNS(config_from(wl)) as d:
            assert names <= _names(d)
        with ChannelDNS(config_from(wl)) as d:
            d.step(1)
            one = d.get_state(walls=False)
            d.step(9)
            out[mode] = (one, d.get_state(walls=False), d.diagnostics())
    scale = max(np.max(np.abs(out["0"][1][k])) for k in ("u", "v", "w"))
    # about 2^-53 of the row and column scales per product (the FP64-pipe
    # kernels: 2^-53 of each term), K = 65 terms: ~1e-14 of the velocity
    # scale per step
    for i, bound in ((0, 3e-13), (1, 2e-12)):
        for k in ("u", "v", "w"):
            assert np.max(np.abs(out["1"][i][k] - out["0"][i][k])) <= bound * scale, (i, k)
    assert abs(out["1"][2].energy - out["0"][2].energy) <= 1e-12 * out["0"][2].energy


def test_tensor_core_runs_in_batches_bitwise(built_lib, monkeypatch):
    monkeypatch.setenv("DNS3D_TENSOR_CORES", "1")
    draws = ensemble_draws(4, seed=13)
    cfgs = [config_from(d) for d in draws]
    with Ensemble(cfgs) as ens:
        ens.step(3)
        states = [ens.run(i).get_state(walls=False) for i in range(len(ens))]
    for cfg, st in zip(cfgs, states):
        with ChannelDNS(cfg) as d:
            assert {"viscous_helmholtz_tc", "vorticity_tc", "pressure_poisson_tc", "pressure_correction_tc"} <= _names(d)
        with ChannelDNS(cfg) as d:
            d.step(3)
            solo = d.get_state(walls=False)
        for k in ("u", "v", "w", "p_total"):
            assert np.array_equal(st[k], solo[k]), (cfg.nx, cfg.ny, cfg.nz, k)


def test_tensor_core_wait_runs_out_and_reports(built_lib, monkeypatch):
    """Failure detection without a GPU fault: with the MMA commit withheld
    (DNS3D_TC_TEST_STALL=1) every tensor-core kernel's bounded completion wait
    runs out; the kernels write nothing, free their TMEM and return, and
    diagnostics report DNS3D_E_TIMEOUT.  The context stays usable."""
    from f90_dns_gb300 import Dns3DError
    from f90_dns_gb300.capi import DNS3D_E_TIMEOUT
    wl = dict(C1, nx=16, ny=16)
    monkeypatch.setenv("DNS3D_TENSOR_CORES", "1")
    monkeypatch.setenv("DNS3D_TC_TEST_STALL", "1")
    with ChannelDNS(config_from(wl)) as d:
        d.step(1)
        with pytest.raises(Dns3DError) as ei:
            d.diagnostics()
        assert ei.value.code == DNS3D_E_TIMEOUT
    monkeypatch.delenv("DNS3D_TC_TEST_STALL")
    with ChannelDNS(config_from(wl)) as d:
        d.step(2)
        assert np.isfinite(d.diagnostics().energy)


def test_tensor_core_forms_at_the_largest_supported_nz(built_lib, monkeypatch):
    """Each folded block is its own M = 128 MMA, so every supported nz (up to
    129) keeps the tensor-core forms when forced; nz = 127 against the oracle."""
    monkeypatch.setenv("DNS3D_TENSOR_CORES", "1")
    wl = dict(C1, nx=16, ny=16, nz=127, lgl_dmatrix_guard=False)
    with ChannelDNS(config_from(wl)) as d:
        names = _names(d)
    assert {"viscous_helmholtz_tc", "vorticity_tc", "pressure_poisson_tc", "pressure_correction_tc"} <= names
    with ChannelDNS(config_from(wl)) as d:
        d.step(10)
        gst = d.get_state()
    _, st, _ = ref.run(oracle_config(wl), 10, record_every=10)
    err = velocity_errors(gst, st)
    assert max(err.values()) <= TOL, err
