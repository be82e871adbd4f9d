"""GPU: the FP64 plane transforms in 64-bit block fixed point.

For grids with compile-time transform kernels the FP64 path runs its r2c and
c2r plane transforms on the integer pipes (fft_ct.cu); DNS3D_FFT_FP64=1 keeps
them on the FP64 pipe.  Bars:
  * a set_state -> get_state round trip (r2c then c2r of every plane) returns
    every plane to 4e-15 of that plane's own largest value, whatever the
    planes' magnitudes (1e-30 .. 1e6, an all-zero plane), on power-of-two and
    radix-3 lengths;
  * 20 steps with either transform agree to 1e-13 of the velocity scale, and
    both match the oracle to 1e-10 (the parity bar);
  * batches of runs with either transform equal their solo runs bitwise.
"""
import numpy as np
import pytest

from f90_dns_gb300 import Batch, ChannelDNS, config_from
from f90_dns_gb300.workloads import WORKLOADS
from oracle import dns3d_ref as ref
from tests.helpers import oracle_config, velocity_errors

pytestmark = pytest.mark.gpu

C1 = WORKLOADS["channel_32x32x33_re180_dpdx"]


@pytest.mark.parametrize("nx,ny,nz", [(32, 32, 17), (128, 128, 9), (96, 48, 9), (48, 192, 7), (512, 384, 5)])
@pytest.mark.parametrize("fp64_pipe", ["0", "1"])
def test_round_trip_per_plane_scale(built_lib, monkeypatch, nx, ny, nz, fp64_pipe):
    monkeypatch.setenv("DNS3D_FFT_FP64", fp64_pipe)
    rng = np.random.default_rng(nx + ny + nz)
    scales = np.array([10.0 ** e for e in np.linspace(-30, 6, nz)])
    scales[nz // 2] = 0.0
    fields = {k: rng.standard_normal((nz, ny, nx)) * scales[:, None, None] for k in ("u", "v", "w", "p_total")}
    with ChannelDNS(config_from(dict(C1, nx=nx, ny=ny, nz=nz))) as d:
        d.set_state(**fields)
        back = d.get_state(walls=False)
    for k, a in fields.items():
        pmax = np.max(np.abs(a), axis=(1, 2))
        err = np.max(np.abs(back[k] - a), axis=(1, 2))
        assert err[nz // 2] == 0.0, k
        rel = err[pmax > 0] / pmax[pmax > 0]
        assert np.max(rel) <= 4e-15, (k, float(np.max(rel)))


def _steps(monkeypatch, wl, n, fp64_pipe):
    monkeypatch.setenv("DNS3D_FFT_FP64", fp64_pipe)
    with ChannelDNS(config_from(wl)) as d:
        d.step(n)
        return d.get_state()


@pytest.mark.parametrize("grid", [(32, 32, 33), (96, 48, 25)])
def test_fixed_point_and_fp64_transforms_agree(built_lib, monkeypatch, grid):
    nx, ny, nz = grid
    wl = dict(C1, nx=nx, ny=ny, nz=nz)
    fx = _steps(monkeypatch, wl, 20, "0")
    f64 = _steps(monkeypatch, wl, 20, "1")
    scale = max(np.max(np.abs(f64[k])) for k in ("u", "v", "w"))
    for k in ("u", "v", "w"):
        assert np.max(np.abs(fx[k] - f64[k])) <= 1e-13 * scale, k
    cfg = oracle_config(wl)
    g = ref.setup_grid(cfg)
    st = ref.initial_state(cfg, g)
    for _ in range(20):
        ref.step(cfg, g, st)
    for run in (fx, f64):
        err = velocity_errors(run, st)
        assert max(err["u"], err["v"], err["w"]) <= 1e-10, err


@pytest.mark.parametrize("fp64_pipe", ["0", "1"])
def test_batches_bitwise_with_either_transform(built_lib, monkeypatch, fp64_pipe):
    monkeypatch.setenv("DNS3D_FFT_FP64", fp64_pipe)
    grids = [(32, 32, 17), (48, 24, 9), (64, 96, 13)]
    cfgs = [config_from(dict(C1, nx=a, ny=b, nz=c)) for a, b, c in grids]
    solo = []
    for cfg in cfgs:
        with ChannelDNS(cfg) as d:
            d.step(3)
            solo.append(d.get_state())
    runs = [ChannelDNS(cfg) for cfg in cfgs]
    try:
        with Batch(runs) as b:
            b.step(3)
        for r, s in zip(runs, solo):
            st = r.get_state()
            for k in ("u", "v", "w", "p_total"):
                assert np.array_equal(st[k], s[k]), (r.shape, k)
    finally:
        for r in runs:
            r.close()


def test_pinned_host_buffers_in_place(built_lib, monkeypatch):
    """Pinned host buffers are read and written in place by the transform
    kernels (no staging copies); the state and the diagnostics equal, bit for
    bit, those of pageable buffers and of the staged path (DNS3D_ZERO_COPY=0)."""
    torch = pytest.importorskip("torch")
    wl = dict(C1, nx=64, ny=48, nz=17)
    shape = (17, 48, 64)
    rng = np.random.default_rng(17)
    init = {k: rng.standard_normal(shape) for k in ("u", "v", "w", "p_total")}

    def run(zero_copy, pinned):
        monkeypatch.setenv("DNS3D_ZERO_COPY", zero_copy)
        alloc = ((lambda: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()) if pinned
                 else (lambda: np.empty(shape)))
        with ChannelDNS(config_from(wl)) as d:
            bufs = {k: alloc() for k in init}
            for k in bufs:
                bufs[k][...] = init[k]
            d.set_state(**bufs)
            d.step(2)
            out = {k: alloc() for k in init}
            d.get_state_into(out["u"], out["v"], out["w"], out["p_total"])
            diag = d.diagnostics()
        return {k: np.array(v) for k, v in out.items()}, diag

    ref_state, ref_diag = run("0", False)
    for zc, pinned in (("1", True), ("0", True), ("1", False)):
        st, dg = run(zc, pinned)
        for k in init:
            assert np.array_equal(st[k], ref_state[k]), (zc, pinned, k)
        assert (dg.energy, dg.max_div, dg.umax) == (ref_diag.energy, ref_diag.max_div, ref_diag.umax)
