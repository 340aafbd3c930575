"""Sweep schedules of the tile relaxations (tt_cuda_set_relax_schedule):
fill, reconstruct and gwdt give the same bits under every schedule,
including the two that order tile visits by value; the oracle pins
schedule 0 (tests/test_gpu_parity.py)."""
import numpy as np
import pytest

from conftest import same_float

pytestmark = pytest.mark.gpu


def _cases():
    from libtopotoolbox_gb300 import dems

    out = []
    d, bc, _ = dems.plain_4096(seed=41, size=700)
    out.append(("rounded_pits_700", d, bc))
    d, bc, _ = dems.plain_16384(seed=42, size=900)
    d2, bc2, _ = dems.nan_to_outlets(d, bc)
    out.append(("nodata_ninf_900", d2, bc2))
    out.append(("nodata_nan_900", d, bc))
    d = dems.pcg4d_dem((333, 517), 9)
    out.append(("pcg4d_333x517", d, dems.border_bc(d.shape)))
    return out


@pytest.mark.parametrize("sched", [1, 2, 3, 4, 5])
def test_schedules_same_bits(gpu, port, sched):
    from libtopotoolbox_gb300 import _native as N
    from libtopotoolbox_gb300 import api

    lib = N.lib()
    for name, dem, bc in _cases():
        lib.tt_cuda_set_relax_schedule(0)
        f0 = api.fillsinks(dem, bc)
        fl, _ = api.identifyflats(f0)
        costs, _ = api.gwdt_computecosts(fl, dem, f0)
        d0 = api.gwdt(costs, fl)
        r0 = api.reconstruct(np.asfortranarray(dem - np.float32(5)), dem)
        lib.tt_cuda_set_relax_schedule(sched)
        try:
            assert same_float(api.fillsinks(dem, bc), f0), (name, "fill")
            assert same_float(api.gwdt(costs, fl), d0), (name, "gwdt")
            assert same_float(api.reconstruct(np.asfortranarray(dem - np.float32(5)), dem), r0), (name, "reconstruct")
            assert same_float(api.d8_pipeline(dem, bc)["dist"], d0), (name, "pipeline")
        finally:
            lib.tt_cuda_set_relax_schedule(-1)
        assert same_float(f0, port.fillsinks(dem, bc)), (name, "oracle")
