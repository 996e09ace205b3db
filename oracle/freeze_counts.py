"""Write profiles/algorithmic_counts.json: the per-unit algorithmic operation
counts (oracle/flops.py) of the batched and multilayer workloads, which
bench.py divides by the measured kernel times for their FP32 rooflines.

MEASUREMENT INFRASTRUCTURE.  Run from the repository root:

    python oracle/freeze_counts.py
"""

from __future__ import annotations

import json
import math
import pathlib
import sys

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parents[1]


def batched_counts(num_configs: int = 4, rays: int = 2000) -> dict:
    """Mean per-ray counts over the first configurations of the batched
    spectrograph workload (seed 3), on the rays its Philox stream draws."""
    sys.path.insert(0, str(ROOT))
    from optika_gb300 import configs
    from oracle import batch as OB
    from oracle import flops as F

    systems, _, _ = configs.spectrograph_batch(4096, seed=3)
    acc = {}
    for c in range(num_configs):
        g = OB.batch_inputs(3, c, rays, *configs.SPEC_WAVELENGTH, *configs.SPEC_FIELD_HALF,
                            configs.SPEC_PUPIL_HALF)
        g = {k: g[k].astype(np.float64) for k in ("wavelength", "field_x", "field_y",
                                                   "pupil_x", "pupil_y")}
        for k, v in F.count_rayfunction(systems[c], g).items():
            acc[k] = acc.get(k, 0.0) + v / num_configs
    return acc


def multilayer_counts(num_mirrors: int = 4, samples: int = 3000) -> dict:
    """Mean per-sample counts (R and T, s and p) over mirrors of the
    multilayer workload (seed 4): 40-bilayer periodic stacks by binary
    powering of the period matrix."""
    sys.path.insert(0, str(ROOT))
    import bench
    from oracle import flops as F

    mirrors = bench._mirrors(4, num_mirrors)
    rng = np.random.default_rng(1)
    wl = rng.uniform(12.0, 15.0, samples)
    cos = np.cos(rng.uniform(0.0, 20.0 * math.pi / 180.0, samples))
    acc = {}
    for m in mirrors:
        for k, v in F.count_multilayer(m.layers, m.substrate, wl, cos).items():
            acc[k] = acc.get(k, 0.0) + v / num_mirrors
    return acc


def main() -> None:
    out = {
        "batched-spectrograph": {"unit": "ray", **{k: round(v, 1)
                                                    for k, v in batched_counts().items()}},
        "multilayer-periodic": {"unit": "sample (s and p)",
                                **{k: round(v, 1) for k, v in multilayer_counts().items()}},
        "counted_by": "oracle/flops.py (non-trivial real operations of the reference's "
                      "formulas), python oracle/freeze_counts.py",
    }
    dst = ROOT / "profiles" / "algorithmic_counts.json"
    dst.write_text(json.dumps(out, indent=1) + "\n")
    print(dst.read_text())


if __name__ == "__main__":
    main()
