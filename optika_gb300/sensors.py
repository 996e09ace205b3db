"""Imaging sensors, mirroring optika/sensors/_sensors.py.

An :class:`ImagingSensor` is the last surface of a system: flat, vacuum
(the ideal sensor material, optika/sensors/materials/_materials.py:1567),
with the pixel array as its aperture (:84-90).  Binning
(:meth:`ImagingSensor.collect`, :92-171) counts the unvignetted rays and
sums their intensity per pixel on the GPU; images are laid out as
``[num_wavelength, num_pixel_x, num_pixel_y]`` with pixel edges
``linspace(-half_width, +half_width, num + 1)`` (numpy.histogramdd
semantics: the last edge is inclusive, everything outside is dropped).
"""

from __future__ import annotations

import dataclasses

import numpy as np

from . import apertures as _apertures
from . import materials as _materials
from . import sags as _sags
from . import transforms
from .surfaces import AbstractSurface

__all__ = ["ImagingSensor", "IdealSensorMaterial"]


class IdealSensorMaterial(_materials.Vacuum):
    """Unit quantum efficiency; behaves as vacuum in the trace."""


@dataclasses.dataclass(eq=False)
class ImagingSensor(AbstractSurface):
    name: None | str = None
    width_pixel: float | tuple[float, float] = 0.0  # mm
    axis_pixel: tuple[str, str] = ("detector_x", "detector_y")
    num_pixel: tuple[int, int] = (0, 0)
    timedelta_exposure: float = 0.0
    read_noise: float = 0.0
    material: None | _materials.AbstractMaterial = None
    aperture_mechanical: None | _apertures.AbstractAperture = None
    is_field_stop: bool = False
    is_pupil_stop: bool = False
    transformation: None | transforms.AbstractTransformation = None

    def __post_init__(self):
        if self.material is None:
            self.material = IdealSensorMaterial()

    @property
    def sag(self) -> _sags.NoSag:
        return _sags.NoSag()

    @property
    def rulings(self):
        return None

    @property
    def width_pixel_xy(self) -> tuple[float, float]:
        w = self.width_pixel
        if np.ndim(w) == 0:
            return float(w), float(w)
        return float(w[0]), float(w[1])

    @property
    def aperture(self) -> _apertures.RectangularAperture:
        wx, wy = self.width_pixel_xy
        nx, ny = self.num_pixel
        return _apertures.RectangularAperture(half_width=(wx * nx / 2, wy * ny / 2))

    def collect(self, rays, wavelength=None, where=True):
        """Bin rays (in this sensor's local frame) onto the pixel grid:
        ``(image, direction)``, the intensity image and the flux-weighted
        mean cosine of incidence in each pixel (1 where a pixel is empty),
        as optika/sensors/_sensors.py:92-169 returns them for an ideal
        sensor material.  Images are ``[num_w, num_x, num_y]``.

        ``wavelength`` is ``None`` (one bin, all wavelengths) or
        ``(start, stop, num)`` uniform wavelength edges in nm.
        """
        import torch

        from ._api import collect

        _, flux, mom = collect(self, rays, wavelength=wavelength, where=where, cos_moment=True)
        direction = torch.where(flux > 0, mom / flux, torch.ones_like(flux))
        return flux, direction

    def collect_counts(self, rays, wavelength=None, where=True):
        """``(counts, flux)``: the ray counts and the intensity image."""
        from ._api import collect

        return collect(self, rays, wavelength=wavelength, where=where)

    def expose(self, image, direction=1, timedelta=None, noise: bool = True, seed: int = 0,
               photons: bool = True, wavelength=None):
        """Electrons measured from a photon image (optika/sensors/_sensors.py:
        173-252 with the ideal material, optika/sensors/materials/
        _materials.py:1576-1598), on the GPU: ``image x timedelta`` photons
        per pixel, Poisson shot noise and Gaussian read noise of
        ``read_noise`` electrons when ``noise``.  ``timedelta`` defaults to
        ``timedelta_exposure``.  ``photons=False`` means the image is an
        energy flux (J), converted to photons with h c / lambda at the
        centres of the wavelength bin edges ``wavelength`` (nm).  The ideal
        material's quantum efficiency is 1, so ``direction`` (the refracted
        cosine) does not enter."""
        import torch

        from ._api import device, expose

        img = image if isinstance(image, torch.Tensor) else torch.as_tensor(
            np.asarray(image, dtype=np.float32))
        img = img.to(device=device(), dtype=torch.float32)
        if not photons:
            if wavelength is None:
                raise ValueError("an energy image needs the wavelength bin edges")
            w = np.asarray(wavelength, dtype=np.float64)
            centers = (w[:-1] + w[1:]) / 2
            hc = 6.62607015e-34 * 299792458.0 * 1e9  # J nm
            per = torch.as_tensor(centers / hc, dtype=torch.float32, device=img.device)
            img = img * per.reshape((-1,) + (1,) * (img.ndim - 1))
        dt = self.timedelta_exposure if timedelta is None else timedelta
        return expose(img, float(dt), float(self.read_noise), noise, seed)

    def photons_absorbed(self, image, direction=1, timedelta=None):
        """The photon flux absorbed in each pixel from an electron image, the
        deterministic inverse of :meth:`expose` (optika/sensors/_sensors.py:
        254-315): the ideal material yields one electron per photon
        (optika/sensors/materials/_materials.py:1627-1633), so this divides
        by the exposure time.  Elementwise torch arithmetic on the image's
        device."""
        import torch

        img = image if isinstance(image, torch.Tensor) else torch.as_tensor(
            np.asarray(image, dtype=np.float32))
        dt = self.timedelta_exposure if timedelta is None else timedelta
        return img / dt

    def uncertainty(self, image, direction=1):
        """Standard deviation of the noise of an electron image
        (optika/sensors/_sensors.py:317-372): the ideal material's shot
        noise sqrt(electrons) (optika/sensors/materials/_materials.py:
        1635-1644) and the read noise, added in quadrature."""
        import torch

        img = image if isinstance(image, torch.Tensor) else torch.as_tensor(
            np.asarray(image, dtype=np.float32))
        return torch.sqrt(img + float(self.read_noise) ** 2)

    def measure(self, rays, wavelength=None, where=True, timedelta=None, noise: bool = True,
                seed: int = 0):
        """:meth:`collect` then :meth:`expose` (optika/sensors/_sensors.py:
        374-428): electrons per pixel ``[num_w, num_x, num_y]``."""
        image, direction = self.collect(rays, wavelength=wavelength, where=where)
        return self.expose(image, direction=direction, timedelta=timedelta, noise=noise,
                           seed=seed)
