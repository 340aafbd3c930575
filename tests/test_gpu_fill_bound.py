"""Sink filling from the coarse upper bound (the fill of the 4 x 4 max-pooled
DEM, src/fillsinks.c:23-77 reached from another start) against the oracle.

The bounded start runs by default only on grids of 12288 pixels a side and
more; here a child process lowers that threshold (TT_CUDA_FILL_BOUND_MIN,
read once per process) so that small grids take it too, with the cases the
bound has to treat conservatively: NaN pixels (a cell holding one is never
passable nor a seed), seeds inside such cells, -INF outlets, ragged sizes
whose last cells are partial, and two bounded levels.  Every result must
equal the oracle bit for bit.
"""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import same_float

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def _cases():
    from libtopotoolbox_gb300 import dems

    out = []
    for k, shp in enumerate([(300, 257), (517, 1029), (1024, 1024), (33, 4000)]):
        dem = dems.pcg4d_dem(shp, 20 + k)
        bc = dems.border_bc(shp)
        rng = np.random.default_rng(k)
        if k in (1, 2):  # NaN disks, some seeds inside them
            m, n = shp
            ii, jj = np.meshgrid(np.arange(m), np.arange(n), indexing="ij")
            for _ in range(6):
                ci, cj, r = rng.integers(0, m), rng.integers(0, n), rng.integers(3, 20)
                dem[(ii - ci) ** 2 + (jj - cj) ** 2 < r * r] = np.nan
            bc[rng.random(shp) < 0.002] = 1
        if k == 3:  # -INF outlets with bc = 1, the nodata convention of the workloads
            hole = rng.random(shp) < 0.01
            dem[hole] = -np.inf
            bc[hole] = 1
        out.append((np.asfortranarray(dem.astype(np.float32)), np.asfortranarray(bc)))
    return out


def test_bounded_fill_matches_oracle(gpu, port, tmp_path):
    cases = _cases()
    np.savez(tmp_path / "in.npz", **{f"dem{k}": d for k, (d, _) in enumerate(cases)},
             **{f"bc{k}": b for k, (_, b) in enumerate(cases)})
    code = (
        "import sys, numpy as np; sys.path.insert(0, %r)\n"
        "from libtopotoolbox_gb300 import api\n"
        "z = np.load(%r)\n"
        "out = {}\n"
        "for k in range(%d):\n"
        "    out[f'f{k}'] = api.fillsinks(z[f'dem{k}'], z[f'bc{k}'])\n"
        "import torch\n"
        "from libtopotoolbox_gb300.api import dev\n"
        "t = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).cuda()\n"
        "with dev.deferred():\n"
        "    f = dev.fillsinks(t(z['dem2']), t(z['bc2']))\n"
        "out['deferred2'] = f.cpu().numpy().T\n"
        "np.savez(%r, **out)\n"
    ) % (str(ROOT), str(tmp_path / "in.npz"), len(cases), str(tmp_path / "out.npz"))
    env = dict(os.environ, TT_CUDA_FILL_BOUND_MIN="32")  # bounded at every level >= 32
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    got = np.load(tmp_path / "out.npz")
    for k, (dem, bc) in enumerate(cases):
        assert same_float(got[f"f{k}"], port.fillsinks(dem, bc)), f"case {k} {dem.shape}"
    # the same under deferred status (the coarse runs record nothing)
    assert same_float(got["deferred2"], got["f2"])
