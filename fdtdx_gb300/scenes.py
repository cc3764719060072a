"""Seeded synthetic scenes of the benchmark workloads (user-level code on the public API).

* ``dipole_boxes``      100^3 at 50 nm, 20 random dielectric boxes, z dipole with a 5 fs
                        Gaussian pulse at 1.55 um, Ez plane field detector (the plain CPU case)
* ``coupler``           400x400x200 at 20 nm: two Si strips in SiO2, CW Gaussian plane source
                        on one strip, full-volume phasor of Ex/Ey/Ez, phasor flux at each arm
* ``inverse_design``    200x200x100 at 25 nm: 120x120x9 design region, pulsed plane source,
                        phasor objective plane above the region
* ``strip``             a single Si strip of given width (the batch/serving unit)

Every builder takes a ``scale`` that shrinks the grid for tests (sizes in cells are
scaled, the physical spacing is kept) and a ``steps`` override.
"""

from __future__ import annotations

import math

import numpy as np
import torch

from fdtdx_gb300 import constants
from fdtdx_gb300.config import GradientConfig, Recorder, SimulationConfig, UniformGrid
from fdtdx_gb300.core import GaussianPulseProfile, SingleFrequencyProfile, WaveCharacter
from fdtdx_gb300.initialization import place_objects
from fdtdx_gb300.objects import (
    BoundaryConfig,
    Device,
    FieldDetector,
    GaussianPlaneSource,
    Material,
    PhasorDetector,
    PhasorPoyntingFluxDetector,
    PointDipoleSource,
    SimulationVolume,
    UniformMaterialObject,
    UniformPlaneSource,
    boundary_objects_from_config,
)

WL = 1.55e-6
EPS_SIO2 = 2.1025
EPS_SI = 12.11


def _config(dx: float, steps: int, courant_factor: float = 0.99, gradient: bool = False,
            recorder: Recorder | None = None) -> SimulationConfig:
    dt = courant_factor / math.sqrt(3) * dx / constants.c
    gc = GradientConfig(method="reversible", recorder=recorder or Recorder()) if gradient else None
    return SimulationConfig(time=steps * dt, grid=UniformGrid(dx), courant_factor=courant_factor, gradient_config=gc)


def pulse_5fs() -> GaussianPulseProfile:
    """Gaussian pulse at 1.55 um with 5 fs FWHM: sigma_t = 5 fs / 2.3548, width f = 1/(2 pi sigma_t)."""
    sigma_t = 5e-15 / 2.3548
    return GaussianPulseProfile(
        spectral_width=WaveCharacter(frequency=1.0 / (2 * math.pi * sigma_t)),
        center_wave=WaveCharacter(wavelength=WL),
    )


def dipole_boxes(shape=(100, 100, 100), steps: int = 1000, seed: int = 0, n_boxes: int = 20, pml: int = 10,
                 dx: float = 50e-9, boundary: str = "pml", device=None):
    rng = np.random.default_rng(seed)
    cfg = _config(dx, steps)
    vol = SimulationVolume(shape=shape)
    objs = [vol]
    bc = BoundaryConfig.from_uniform_bound(thickness=pml, boundary_type=boundary)
    objs += list(boundary_objects_from_config(bc, vol).values())
    lo, hi = [pml] * 3, [n - pml for n in shape]
    for b in range(n_boxes):
        st = []
        for a in range(3):
            span = hi[a] - lo[a]
            side = int(rng.integers(3, min(15, max(3, span - 1)) + 1))
            side = min(side, span)
            start = int(rng.integers(lo[a], hi[a] - side + 1))
            st.append((start, start + side))
        eps = float(rng.choice([EPS_SIO2, EPS_SI]))
        objs.append(UniformMaterialObject(name=f"box{b}", grid_slice_tuple=tuple(st),
                                          material=Material(permittivity=eps), placement_order=b))
    c = [n // 2 for n in shape]
    objs.append(PointDipoleSource(name="dipole", grid_slice_tuple=tuple((x, x + 1) for x in c), polarization=2,
                                  wave_character=WaveCharacter(wavelength=WL), temporal_profile=pulse_5fs()))
    objs.append(FieldDetector(name="ez_plane", grid_slice_tuple=((0, shape[0]), (0, shape[1]), (c[2], c[2] + 1)),
                              components=("Ez",)))
    return place_objects(objs, cfg, device=device)


def coupler(shape=(400, 400, 200), steps: int = 8000, scale: float = 1.0, dx: float = 20e-9, pml: int = 10,
            full_phasor: bool = True, boundary: str = "pml", device=None):
    """Two parallel Si strips (500 x 220 nm, 200 nm gap) spanning x in SiO2, CW Gaussian source on strip 1."""
    nx, ny, nz = shape
    s = scale
    w, h, gap = max(2, round(25 * s)), max(2, round(11 * s)), max(1, round(10 * s))
    cfg = _config(dx, steps)
    vol = SimulationVolume(shape=shape, material=Material(permittivity=EPS_SIO2))
    objs = [vol]
    objs += list(boundary_objects_from_config(BoundaryConfig.from_uniform_bound(thickness=pml, boundary_type=boundary),
                                              vol).values())
    yc, zc = ny // 2, nz // 2
    y1 = (yc - gap // 2 - w, yc - gap // 2)
    y2 = (yc + (gap - gap // 2), yc + (gap - gap // 2) + w)
    z = (zc - h // 2, zc - h // 2 + h)
    for name, yy in (("strip1", y1), ("strip2", y2)):
        objs.append(UniformMaterialObject(name=name, grid_slice_tuple=((0, nx), yy, z),
                                          material=Material(permittivity=EPS_SI)))
    xs = max(pml + 2, min(round(50 * s), nx // 4))
    half = max(3, round(30 * s))
    ysc = (y1[0] + y1[1]) // 2
    src_y = (max(pml, ysc - half), min(ny - pml, ysc + half))
    src_z = (max(pml, zc - half), min(nz - pml, zc + half))
    objs.append(GaussianPlaneSource(name="source", grid_slice_tuple=((xs, xs + 1), src_y, src_z), direction="+",
                                    radius=0.6e-6 * s if s < 1 else 0.6e-6, fixed_E_polarization_vector=(0, 1, 0),
                                    wave_character=WaveCharacter(wavelength=WL),
                                    temporal_profile=SingleFrequencyProfile()))
    if full_phasor:
        objs.append(PhasorDetector(name="phasor", grid_slice_tuple=((0, nx), (0, ny), (0, nz)),
                                   wave_characters=(WaveCharacter(wavelength=WL),), components=("Ex", "Ey", "Ez")))
    xd = nx - max(pml + 2, min(round(50 * s), nx // 4))
    pad = max(2, round(5 * s))
    for name, yy in (("flux1", y1), ("flux2", y2)):
        objs.append(PhasorPoyntingFluxDetector(
            name=name, grid_slice_tuple=((xd, xd + 1), (yy[0] - pad, yy[1] + pad), (z[0] - pad, z[1] + pad)),
            direction="+", wave_characters=(WaveCharacter(wavelength=WL),)))
    return place_objects(objs, cfg, device=device)


def inverse_design(shape=(200, 200, 100), steps: int = 3000, seed: int = 0, dx: float = 25e-9, pml: int = 10,
                   design=(120, 120, 9), plane=(40, 40), recorder: Recorder | None = None, device=None):
    nx, ny, nz = shape
    cfg = _config(dx, steps, gradient=True, recorder=recorder)
    vol = SimulationVolume(shape=shape, material=Material(permittivity=EPS_SIO2))
    objs = [vol]
    objs += list(boundary_objects_from_config(BoundaryConfig.from_uniform_bound(thickness=pml), vol).values())
    c = [n // 2 for n in shape]
    dsl = tuple((c[a] - design[a] // 2, c[a] - design[a] // 2 + design[a]) for a in range(3))
    objs.append(Device(name="design", grid_slice_tuple=dsl, permittivity_low=EPS_SIO2, permittivity_high=EPS_SI))
    zs = max(pml + 2, dsl[2][0] - max(3, nz // 5))
    objs.append(UniformPlaneSource(name="source", grid_slice_tuple=((pml, nx - pml), (pml, ny - pml), (zs, zs + 1)),
                                   direction="+", fixed_E_polarization_vector=(1, 0, 0),
                                   wave_character=WaveCharacter(wavelength=WL), temporal_profile=pulse_5fs()))
    zo = min(nz - pml - 2, dsl[2][1] + max(3, nz // 5))
    osl = ((c[0] - plane[0] // 2, c[0] - plane[0] // 2 + plane[0]), (c[1] - plane[1] // 2, c[1] - plane[1] // 2 + plane[1]),
           (zo, zo + 1))
    objs.append(PhasorDetector(name="objective", grid_slice_tuple=osl, wave_characters=(WaveCharacter(wavelength=WL),),
                               components=("Ex", "Ey", "Ez"), scaling_mode="pulse"))
    objects, arrays, params, cfg, info = place_objects(objs, cfg, device=device)
    rng = np.random.default_rng(seed)
    params["design"] = torch.tensor(rng.uniform(0.0, 1.0, size=design), dtype=torch.float32, device=arrays.device)
    return objects, arrays, params, cfg, info


def strip(shape=(128, 128, 96), width_um: float = 0.5, steps: int = 2000, dx: float = 25e-9, pml: int = 10,
          device=None):
    """A single Si strip (220 nm tall) in SiO2 spanning x; pulsed Gaussian source; transmitted phasor flux."""
    nx, ny, nz = shape
    cfg = _config(dx, steps)
    vol = SimulationVolume(shape=shape, material=Material(permittivity=EPS_SIO2))
    objs = [vol]
    objs += list(boundary_objects_from_config(BoundaryConfig.from_uniform_bound(thickness=pml), vol).values())
    w = max(2, round(width_um * 1e-6 / dx))
    h = max(2, round(220e-9 / dx))
    yc, zc = ny // 2, nz // 2
    ys, zs = (yc - w // 2, yc - w // 2 + w), (zc - h // 2, zc - h // 2 + h)
    objs.append(UniformMaterialObject(name="strip", grid_slice_tuple=((0, nx), ys, zs),
                                      material=Material(permittivity=EPS_SI)))
    xs = pml + 2
    half_y, half_z = min(ny // 2 - pml - 1, 2 * w), min(nz // 2 - pml - 1, 4 * h)
    objs.append(GaussianPlaneSource(name="source", grid_slice_tuple=((xs, xs + 1), (yc - half_y, yc + half_y),
                                                                     (zc - half_z, zc + half_z)),
                                    direction="+", radius=min(half_y, half_z) * dx, fixed_E_polarization_vector=(0, 1, 0),
                                    wave_character=WaveCharacter(wavelength=WL), temporal_profile=pulse_5fs()))
    xd = nx - pml - 3
    objs.append(PhasorPoyntingFluxDetector(name="flux", grid_slice_tuple=((xd, xd + 1), (yc - half_y, yc + half_y),
                                                                          (zc - half_z, zc + half_z)),
                                           direction="+", wave_characters=(WaveCharacter(wavelength=WL),),
                                           scaling_mode="pulse"))
    return place_objects(objs, cfg, device=device)


def serving_job(shape=(64, 64, 64), steps: int = 1000, seed: int = 0, anisotropic: bool = False,
                gradient: bool = False, with_recorder: bool = True, n_boxes: int = 20, pml: int = 10,
                dx: float = 50e-9, device=None):
    """A request of the serving stream: random boxes (isotropic eps from {2.1025, 12.11}, or
    per-axis eps uniform in [2, 12]), a pulsed z dipole at the centre and an E phasor plane
    near the +z face whose sum |phasor|^2 is the gradient jobs' objective."""
    rng = np.random.default_rng(seed)
    pml = min(pml, max(2, min(shape) // 4))
    cfg = _config(dx, steps, gradient=gradient and with_recorder)
    vol = SimulationVolume(shape=shape)
    objs = [vol]
    objs += list(boundary_objects_from_config(BoundaryConfig.from_uniform_bound(thickness=pml), vol).values())
    lo, hi = [pml] * 3, [n - pml for n in shape]
    for b in range(n_boxes):
        st = []
        for a in range(3):
            span = hi[a] - lo[a]
            side = min(int(rng.integers(3, min(15, max(3, span - 1)) + 1)), span)
            start = int(rng.integers(lo[a], hi[a] - side + 1))
            st.append((start, start + side))
        if anisotropic:
            eps = tuple(float(x) for x in rng.uniform(2.0, 12.0, size=3))
        else:
            eps = float(rng.choice([EPS_SIO2, EPS_SI]))
        objs.append(UniformMaterialObject(name=f"box{b}", grid_slice_tuple=tuple(st),
                                          material=Material(permittivity=eps), placement_order=b))
    c = [n // 2 for n in shape]
    objs.append(PointDipoleSource(name="dipole", grid_slice_tuple=tuple((x, x + 1) for x in c), polarization=2,
                                  wave_character=WaveCharacter(wavelength=WL), temporal_profile=pulse_5fs()))
    zd = max(c[2] + 1, shape[2] - pml - 2)
    objs.append(PhasorDetector(name="objective", grid_slice_tuple=((lo[0], hi[0]), (lo[1], hi[1]), (zd, zd + 1)),
                               wave_characters=(WaveCharacter(wavelength=WL),), components=("Ex", "Ey", "Ez"),
                               scaling_mode="pulse"))
    return place_objects(objs, cfg, device=device)
