"""GPU: served runs (continuous batching, runs admitted as memory frees up,
the runs of a full round stepped as one ragged batch) give exactly the result
of each run alone."""
import numpy as np
import pytest

from f90_dns_gb300 import ChannelDNS, Server, config_from, footprint_bytes
from f90_dns_gb300.capi import PREC_MIXED, REQ_DONE
from f90_dns_gb300.workloads import ensemble_draws

pytestmark = pytest.mark.gpu


def test_served_results_equal_alone(built_lib):
    draws = ensemble_draws(5, seed=11)
    cfgs = [config_from(d, precision=(PREC_MIXED if i % 2 else 0)) for i, d in enumerate(draws)]
    steps = [7, 13, 5, 9, 11]
    # budget for about two runs at a time: later requests wait for memory
    budget = int(sorted(footprint_bytes(c) for c in cfgs)[-1] * 2.1)
    with Server(max_bytes=budget, steps_per_round=4) as srv:
        ids = [srv.submit(c, n, keep_state=True) for c, n in zip(cfgs, steps)]
        infos = [srv.wait(i, timeout=300.0) for i in ids]
        states = [srv.result_state(i) for i in ids]
        assert srv.stats()["bytes_in_use"] == 0
    for inf, n in zip(infos, steps):
        assert inf.status == REQ_DONE and inf.steps_done == n and inf.diag.step == n
    # at most ~two footprints were resident at any time: some request started late
    assert max(i.t_start for i in infos) > min(i.t_finish for i in infos) - 1e-9
    for cfg, n, st in zip(cfgs, steps, states):
        with ChannelDNS(cfg) as d:
            d.step(n)
            solo = d.get_state(walls=False)
        for k in ("u", "v", "w", "p_total"):
            assert np.array_equal(st[k], solo[k]), (cfg.nx, cfg.ny, cfg.nz, k)


def test_served_batches_rebuilt_as_runs_finish(built_lib):
    """Ten runs admitted together step as one batch; the batch is rebuilt as
    runs finish (uneven step counts, a short last round each) and every
    result is still the run's solo result."""
    draws = ensemble_draws(10, seed=4)
    cfgs = [config_from(d, precision=(PREC_MIXED if i % 3 else 0)) for i, d in enumerate(draws)]
    steps = [3 + 2 * i for i in range(10)]
    with Server(steps_per_round=4) as srv:
        ids = [srv.submit(c, n, keep_state=True) for c, n in zip(cfgs, steps)]
        infos = [srv.wait(i, timeout=300.0) for i in ids]
        states = [srv.result_state(i) for i in ids]
    for inf, n in zip(infos, steps):
        assert inf.status == REQ_DONE and inf.steps_done == n
    for cfg, n, st in zip(cfgs, steps, states):
        with ChannelDNS(cfg) as d:
            d.step(n)
            solo = d.get_state(walls=False)
        for k in ("u", "v", "w", "p_total"):
            assert np.array_equal(st[k], solo[k]), (cfg.nx, cfg.ny, cfg.nz, k)


def test_large_and_small_runs_overlap(built_lib):
    """A large run (at least 2^20 points: its own launches, never in a batch)
    beside small batched runs, every unit getting its next chunk as soon as its
    last one completes: every result is the run's solo result, and
    dns3d_query reports a handle done once its work has completed."""
    import ctypes as C
    small = [config_from(d, precision=PREC_MIXED) for d in ensemble_draws(4, seed=21)]
    large = config_from(dict(ensemble_draws(1, seed=22)[0], nx=128, ny=96, nz=97, lgl_dmatrix_guard=False),
                        precision=PREC_MIXED)
    with Server(steps_per_round=5) as srv:
        lid = srv.submit(large, 60, keep_state=True)
        sids = [srv.submit(c, 12, keep_state=True) for c in small]
        sinfo = [srv.wait(i, timeout=300.0) for i in sids]
        linfo = srv.wait(lid, timeout=300.0)
        states = [srv.result_state(i) for i in sids] + [srv.result_state(lid)]
    assert all(i.status == REQ_DONE for i in sinfo + [linfo])
    for cfg, n, st in zip(small + [large], [12] * 4 + [60], states):
        with ChannelDNS(cfg) as d:
            d.step(n)
            done = C.c_int(-1)
            assert d.lib.dns3d_query(d._h, C.byref(done)) == 0 and done.value in (0, 1)
            solo = d.get_state(walls=False)
            assert d.lib.dns3d_query(d._h, C.byref(done)) == 0 and done.value == 1
        for k in ("u", "v", "w", "p_total"):
            assert np.array_equal(st[k], solo[k]), (cfg.nx, cfg.ny, cfg.nz, k)
