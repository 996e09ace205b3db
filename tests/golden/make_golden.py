"""Generate ``multilayer_imd.npz`` from the reference's IMD golden data.

The reference pins ``multilayer_efficiency`` against IMD output files
(optika/materials/_tests/test_multilayers.py:178-287, data in
optika/materials/_tests/_data/*.txt, normal incidence, rtol 1e-4), computed
with the optical constants of optika/chemicals/nk/*.nk.  This script reads
both from a checkout of the reference given on the command line, keeps every
``STEP``-th wavelength, and stores per case the IMD efficiency and, for each
chemical of the stack, n and k linearly interpolated at those wavelengths
(the reference's ``na.interp`` of the table, optika/chemicals/_chemicals.py:
138-142).  Run it where the reference is available:

    python tests/golden/make_golden.py /path/to/optika
"""

from __future__ import annotations

import pathlib
import sys

import numpy as np

STEP = 5

CASES = {
    # name: (IMD file, [(chemical, thickness nm)], substrate chemical, is_mirror,
    #        erf interface width on every layer and the substrate, nm)
    "Si": ("Si.txt", [], "Si", False, 0.0),
    "SiO2_50A": ("SiO2.txt", [("SiO2", 5.0)], "Si", False, 0.0),
    "SiO2_100A": ("SiO2_100A.txt", [("SiO2", 10.0)], "Si", False, 0.0),
    "SiC_Cr": ("SiC_Cr.txt", [("SiC", 25.0), ("Cr", 5.0)], "SiO2", True, 0.0),
    # the reference marks this one xfail: "IMD incorrectly uses the vacuum
    # wavelength" in its roughness factor (test_multilayers.py:225-245)
    "SiC_Cr_Rough": ("SiC_Cr_Rough.txt", [("SiC", 25.0), ("Cr", 5.0)], "SiO2", True, 2.0),
}


def read_columns(path: pathlib.Path) -> np.ndarray:
    rows = []
    for line in path.read_text().splitlines():
        s = line.strip()
        if not s or s.startswith(";"):
            continue
        rows.append([float(v) for v in s.split()])
    return np.asarray(rows, dtype=np.float64)


def main(ref: pathlib.Path) -> None:
    data_dir = ref / "optika" / "materials" / "_tests" / "_data"
    nk_dir = ref / "optika" / "chemicals" / "nk"
    out = {}
    for name, (fname, layers, substrate, is_mirror, sigma) in CASES.items():
        a = read_columns(data_dir / fname)
        wl_nm = a[::STEP, 0] / 10.0
        eff = a[::STEP, 1]
        out[f"{name}/wavelength"] = wl_nm
        out[f"{name}/efficiency"] = eff
        out[f"{name}/is_mirror"] = np.array(is_mirror)
        out[f"{name}/interface_width"] = np.array(sigma)
        out[f"{name}/thickness"] = np.array([t for _, t in layers], dtype=np.float64)
        chems = [c for c, _ in layers] + [substrate]
        for i, chem in enumerate(chems):
            t = read_columns(nk_dir / f"{chem}.nk")
            w = t[:, 0] / 10.0
            out[f"{name}/n{i}"] = np.interp(wl_nm, w, t[:, 1])
            out[f"{name}/k{i}"] = np.interp(wl_nm, w, t[:, 2])
        out[f"{name}/num_chemicals"] = np.array(len(chems))
    dst = pathlib.Path(__file__).resolve().parent / "multilayer_imd.npz"
    np.savez_compressed(dst, **out)
    print(f"wrote {dst} ({dst.stat().st_size} bytes)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path to the optika source tree>")
    main(pathlib.Path(sys.argv[1]))
