"""GPU parity of the public grayscale reconstruction (include/topotoolbox.h:1056,
1070; src/reconstruct.c:270-312) against the oracle, which is pinned to the
compiled reference on the same cases (tests/test_oracle_pins.py).

Markers are arbitrary (below the mask by random amounts, -INF but for a few
seeds, above the mask in places) and masks hold NaN holes and plateaus.
Results must be bit-exact (signed zeros compare equal), through the
host-pointer entry points, the hybrid form with its convergence flag, and
the device-pointer form.
"""
import numpy as np
import pytest

from conftest import reconstruct_cases, same_float

pytestmark = pytest.mark.gpu

RECON = reconstruct_cases()


@pytest.mark.parametrize("idx", range(len(RECON)))
def test_reconstruct(gpu, port, idx):
    from libtopotoolbox_gb300 import api

    name, marker, mask = RECON[idx]
    exp = port.reconstruct(marker, mask)
    m0 = marker.copy(order="F")
    got = api.reconstruct(marker, mask)
    assert np.array_equal(marker, m0, equal_nan=True), "input marker was modified"
    assert same_float(got, exp), name
    got_h, flag = api.reconstruct_hybrid(marker, mask)
    assert flag == 0, name
    assert same_float(got_h, exp), name


@pytest.mark.parametrize("idx", range(len(RECON)))
def test_reconstruct_dev(gpu, port, idx):
    torch = gpu
    from libtopotoolbox_gb300.api import dev

    name, marker, mask = RECON[idx]
    exp = port.reconstruct(marker, mask)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).cuda()  # noqa: E731
    d_marker, d_mask = t(marker), t(mask)
    mask0 = d_mask.clone()
    dev.reconstruct(d_marker, d_mask)
    torch.cuda.synchronize()
    assert torch.equal(torch.nan_to_num(d_mask, 7.0), torch.nan_to_num(mask0, 7.0))
    assert same_float(d_marker.cpu().numpy().T, exp), name


def test_reconstruct_equals_fill(gpu, port):
    """fillsinks is -reconstruct(-dem) with the marker seeded from bc
    (src/fillsinks.c:23-48): the public reconstruction reproduces it."""
    from libtopotoolbox_gb300 import api, dems

    dem, bc, _ = dems.plain_4096(seed=31, size=300)
    marker = np.where(bc == 1, -dem, -np.inf).astype(np.float32)
    got = -api.reconstruct(np.asfortranarray(marker), np.asfortranarray(-dem))
    assert same_float(got, port.fillsinks(dem, bc))
