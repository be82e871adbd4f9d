"""GPU: the tile autotuner.  Widths change only the schedule of the mode-tile
kernels, so runs with tuned, built-in and hand-set widths are bitwise equal;
unfitting widths are refused."""
import numpy as np
import pytest

from f90_dns_gb300 import ChannelDNS, Dns3DError, config_from
from f90_dns_gb300.capi import DNS3D_E_INVALID, PREC_MIXED, TILE_KERNELS
from f90_dns_gb300.workloads import WORKLOADS

pytestmark = pytest.mark.gpu

WL = dict(WORKLOADS["channel_32x32x33_re180_dpdx"], nx=48, ny=32, nz=33)


@pytest.mark.parametrize("prec", [0, PREC_MIXED])
def test_tile_widths_do_not_change_results(built_lib, prec):
    states = []
    for widths in (None, dict(vorticity=4, viscous=4, pressure=8, correction=16, vorticity_mixed=4,
                              viscous_mixed=4, pressure_mixed=8),
                   dict(vorticity=32, viscous=8, pressure=32, correction=64, vorticity_mixed=64,
                        viscous_mixed=16, pressure_mixed=32)):
        with ChannelDNS(config_from(WL, precision=prec)) as d:
            if widths:
                d.set_tiles(**widths)
                got = d.tiles()
                assert all(got[k] == v for k, v in widths.items())
            d.step(5)
            states.append(d.get_state())
    for s in states[1:]:
        for k in ("u", "v", "w", "p_total"):
            np.testing.assert_array_equal(s[k], states[0][k])


def test_autotune_reports_fitting_widths(built_lib):
    with ChannelDNS(config_from(WL)) as d:
        t = d.autotune(force=True)
        assert set(t) == set(TILE_KERNELS)
        assert all(w in (4, 8, 16, 32, 64) or w > 0 for w in t.values())
        with pytest.raises(Dns3DError) as ei:
            d.set_tiles(viscous=4096)
        assert ei.value.code == DNS3D_E_INVALID
