"""GPU: an ensemble (or a batch of existing runs) with different grids,
parameters and precisions advanced together gives, for every run, exactly the
state of that run advanced alone: the ragged stage launches run each run's own
kernel bodies, and runs outside them keep their own launches."""
import numpy as np
import pytest

from f90_dns_gb300 import Batch, ChannelDNS, Ensemble, config_from
from f90_dns_gb300.capi import PREC_MIXED
from f90_dns_gb300.workloads import ensemble_draws

pytestmark = pytest.mark.gpu


def test_ensemble_runs_equal_solo_runs(built_lib):
    draws = ensemble_draws(6, seed=3)
    cfgs = [config_from(d, precision=(PREC_MIXED if i % 2 else 0)) for i, d in enumerate(draws)]
    with Ensemble(cfgs) as ens:
        ens.step(5)
        ens.step(3)
        mixed_states = [ens.run(i).get_state(walls=False) for i in range(len(ens))]
        assert all(ens.run(i).diagnostics().step == 8 for i in range(len(ens)))
    for cfg, st in zip(cfgs, mixed_states):
        with ChannelDNS(cfg) as d:
            d.step(8)
            solo = d.get_state(walls=False)
        for k in ("u", "v", "w", "p_total"):
            assert np.array_equal(st[k], solo[k]), (cfg.nx, cfg.ny, cfg.nz, k)


def test_ensemble_state_io_between_steps(built_lib):
    draws = ensemble_draws(3, seed=5)
    cfgs = [config_from(d) for d in draws]
    with Ensemble(cfgs) as ens:
        ens.step(2)
        r = ens.run(1)
        st = r.get_state()
        r.set_state(u=st["u"] * 0.5)
        ens.step(1)
        d = r.diagnostics()
        assert d.step == 3 and np.isfinite(d.energy)


def test_handles_of_different_grids_coexist(built_lib):
    """A small grid's handle created after a large one must not restrict the
    large one's kernels (launch limits are per kernel function)."""
    big = dict(ensemble_draws(1, seed=1)[0], nx=96, ny=96, nz=65, lgl_dmatrix_guard=False)
    small = dict(big, nx=32, ny=32, nz=17, lgl_dmatrix_guard=True)
    with ChannelDNS(config_from(big)) as a, ChannelDNS(config_from(small)) as b:
        a.step(2)
        b.step(2)
        a.compute_source_terms_3d()
        a.viscous_step_3d()
        a.synchronize()


def _solo(cfg, nsteps):
    with ChannelDNS(cfg) as d:
        d.step(nsteps)
        return d.get_state(walls=False), d.diagnostics()


def test_ensemble_ragged_launches_and_loose_runs(built_lib):
    """Runs with the jst4 scheme, the jacgs solver or a transform length
    without compile-time kernels keep their own launches beside the ragged
    stages; every run still equals its solo run bitwise."""
    draws = ensemble_draws(5, seed=7)
    cfgs = [config_from(d, precision=(PREC_MIXED if i % 2 else 0)) for i, d in enumerate(draws)]
    cfgs.append(config_from(draws[0], convection_scheme=1))
    cfgs.append(config_from(draws[1], linear_solver=1))
    cfgs.append(config_from(draws[2], nx=24, ny=12, nz=17))  # lengths 12: generic kernels
    with Ensemble(cfgs) as ens:
        launches, ragged = ens.info()
        ens.step(4)
        states = [ens.run(i).get_state(walls=False) for i in range(len(ens))]
    assert ragged == 5
    # nine stage launches per FP64 group, eleven per mixed group, plus the loose runs' own launches
    assert launches > 20
    for cfg, st in zip(cfgs, states):
        solo, _ = _solo(cfg, 4)
        for k in ("u", "v", "w", "p_total"):
            assert np.array_equal(st[k], solo[k]), (cfg.nx, cfg.ny, cfg.nz, cfg.precision, k)


def test_ensemble_launches_per_step_independent_of_size(built_lib):
    for n in (2, 12):
        cfgs = [config_from(d, precision=PREC_MIXED) for d in ensemble_draws(n, seed=2)]
        with Ensemble(cfgs) as ens:
            launches, ragged = ens.info()
        assert (launches, ragged) == (11, n)  # nine stages + the mixed mode (0,0) pair


def test_batch_over_existing_runs_with_pi_control(built_lib):
    """A batch over caller-owned handles, PI-controlled runs included: the
    tile tuning at creation leaves the controller state untouched, and tuned
    and untuned batches give the solo results."""
    draws = ensemble_draws(4, seed=9)
    cfgs = [config_from(d, precision=(PREC_MIXED if i % 2 else 0), flow_control_method=2,
                        target_bulk_velocity=2.0 / 3.0, controller_gain=0.5, controller_update_freq=1)
            for i, d in enumerate(draws)]
    for tune in (True, False):
        runs = [ChannelDNS(c) for c in cfgs]
        try:
            for r in runs:
                r.step(1)  # the controller has state before the batch is made
            with Batch(runs, tune=tune) as b:
                b.step(3)
                b.synchronize()
            for r in runs:
                r.step(1)  # the runs' own launches after the batch
            got = [(r.get_state(walls=False), r.diagnostics()) for r in runs]
        finally:
            for r in runs:
                r.close()
        for cfg, (st, dg) in zip(cfgs, got):
            solo, sdg = _solo(cfg, 5)
            assert dg.step == 5
            assert dg.dpdx == sdg.dpdx
            for k in ("u", "v", "w", "p_total"):
                assert np.array_equal(st[k], solo[k]), (tune, cfg.nx, cfg.ny, cfg.nz, k)
