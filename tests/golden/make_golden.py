"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference's own hot-path C sources (compiled by
`make -C oracle ref` from the reference checkout) on small seeded DEMs and
stores inputs and every output of the D8 path as .npz files.  The fixtures
pin the CPU oracle on hosts where the reference sources are absent.

    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import pyoracle  # noqa: E402
from libtopotoolbox_gb300 import dems  # noqa: E402


def main():
    if pyoracle.build_ref() is None:
        raise SystemExit("reference sources not found")
    ref = pyoracle.Oracle("ref")
    cases = []
    for s in (0, 1):
        d = dems.pcg4d_dem((100, 200), s)
        cases.append((f"pcg4d_100x200_seed{s}", d, dems.border_bc(d.shape), s & 1))
    d, bc, _ = dems.plain_512(seed=21, size=96)
    cases.append(("fractal_noise_96", d, bc, 1))
    d, bc, _ = dems.plain_4096(seed=22, size=96)
    cases.append(("fractal_rounded_96", d, bc, 0))
    d, bc, _ = dems.plain_16384(seed=23, size=128)
    d2, bc2, _ = dems.nan_to_outlets(d, bc)
    cases.append(("fractal_nodata_128", d2, bc2, 1))
    for name, dem, bc, hybrid in cases:
        r = ref.pipeline(dem, bc, hybrid=bool(hybrid))
        az, alt, cs = 3.9269908, 1.0471976, 30.0
        hs = ref.hillshade_fused(np.nan_to_num(dem), az, alt, cs)
        np.savez_compressed(HERE / f"{name}.npz", dem=dem, bc=bc, hybrid=hybrid, az=az, alt=alt,
                            cs=cs, hillshade=hs, **r)
        print("wrote", name)


if __name__ == "__main__":
    main()
