"""GPU: an ensemble of runs with different grids, parameters and precisions
advanced together gives, for every run, exactly the state of that run
advanced alone (same kernels; the graph only overlaps them)."""
import numpy as np
import pytest

from f90_dns_gb300 import ChannelDNS, Ensemble, config_from
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
