"""Optical constants n + i k of a medium, mirroring optika/chemicals.

The reference reads IMD ``.nk`` tables and interpolates them linearly in
wavelength (optika/chemicals/_chemicals.py:101-144).  Here a
:class:`Chemical` holds its table (wavelength in nm, n, k) explicitly;
:meth:`Chemical.from_nk_file` reads the IMD text format (wavelength in
Angstrom, ';' comment lines).  Outside the table the end values are held
(numpy.interp semantics).
"""

from __future__ import annotations

import dataclasses
import pathlib

import numpy as np

__all__ = ["Chemical"]


@dataclasses.dataclass(eq=False)
class Chemical:
    wavelength: np.ndarray  # nm, increasing
    n: np.ndarray
    k: np.ndarray
    name: str = ""

    def __post_init__(self):
        self.wavelength = np.asarray(self.wavelength, dtype=np.float64)
        self.n = np.asarray(self.n, dtype=np.float64)
        self.k = np.asarray(self.k, dtype=np.float64)
        if self.wavelength.ndim != 1 or self.wavelength.size < 1:
            raise ValueError("a chemical table needs at least one wavelength")
        if self.n.shape != self.wavelength.shape or self.k.shape != self.wavelength.shape:
            raise ValueError("n and k must have the shape of wavelength")
        if np.any(np.diff(self.wavelength) <= 0):
            raise ValueError("table wavelengths must be strictly increasing")

    @classmethod
    def from_nk_file(cls, path: str | pathlib.Path, name: str = "") -> "Chemical":
        path = pathlib.Path(path)
        rows = []
        for line in path.read_text().splitlines():
            s = line.strip()
            if not s or s.startswith(";"):
                continue
            rows.append([float(v) for v in s.split()[:3]])
        a = np.asarray(rows, dtype=np.float64)
        return cls(wavelength=a[:, 0] / 10.0, n=a[:, 1], k=a[:, 2], name=name or path.stem)

    def index(self, wavelength_nm) -> np.ndarray:
        """Host-side complex index (float64), for setting up inputs."""
        w = np.asarray(wavelength_nm, dtype=np.float64)
        return np.interp(w, self.wavelength, self.n) + 1j * np.interp(w, self.wavelength, self.k)
