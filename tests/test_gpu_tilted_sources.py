"""Tilted sources on the GB300 path against the oracle (float32: asserted, 1e-4 relative L2;
float64: reported).

A tilted TFSF plane reaches the device as per-cell incident profiles and per-cell Yee time
offsets, a tilted point dipole as one ordinary dipole record per component its orientation
reaches; the kernels are the untilted ones.
"""

import math

import pytest
import torch

import fdtdx_gb300 as fx
from fdtdx_gb300 import scenes
from tests.helpers import compare_states, oracle_run

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _cfg(steps, dx=50e-9):
    dt = 0.99 / math.sqrt(3) * dx / 299792458.0
    return fx.SimulationConfig(time=steps * dt, grid=fx.UniformGrid(dx))


def test_tilted_sources():
    """A tilted Gaussian plane source (per-cell Yee time offsets across the plane) and tilted
    electric and magnetic point dipoles (one source record per injected component) in a
    diagonally anisotropic, magnetic block, against the oracle."""
    cfg = _cfg(120, dx=25e-9)
    vol = fx.SimulationVolume(shape=(36, 32, 30))
    objs = [vol] + list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(6), vol).values())
    objs.append(fx.UniformMaterialObject(name="blk", grid_slice_tuple=((14, 26), (10, 22), (12, 20)),
                                         material=fx.Material(permittivity=(2.0, 3.0, 2.5), permeability=(1.2, 1.0, 1.4))))
    wc = fx.WaveCharacter(wavelength=1.0e-6)
    objs.append(fx.GaussianPlaneSource(name="g", grid_slice_tuple=((7, 29), (7, 25), (9, 10)), direction="+",
                                       radius=7 * 25e-9, fixed_E_polarization_vector=(1, 0, 0), azimuth_angle=25.0,
                                       elevation_angle=-10.0, wave_character=wc))
    objs.append(fx.PointDipoleSource(name="de", grid_slice_tuple=((18, 19), (15, 16), (16, 17)), polarization=2,
                                     azimuth_angle=35.0, elevation_angle=20.0, wave_character=wc,
                                     temporal_profile=scenes.pulse_5fs()))
    objs.append(fx.PointDipoleSource(name="dm", grid_slice_tuple=((22, 23), (12, 13), (14, 15)), polarization=0,
                                     azimuth_angle=-30.0, elevation_angle=15.0, source_type="magnetic",
                                     amplitude=0.7, wave_character=wc))
    R = ((10, 26), (9, 23), (11, 22))
    objs += [
        fx.PhasorDetector(name="ph", grid_slice_tuple=R, wave_characters=(wc,)),
        fx.PoyntingFluxDetector(name="flux", grid_slice_tuple=((8, 28), (8, 24), (22, 23)), direction="+"),
    ]
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg)
    _, out = fx.run_fdtd(arrays, objects, cfg)
    torch.cuda.synchronize()
    _, r32 = oracle_run(objects, arrays, cfg, torch.float32)
    _, r64 = oracle_run(objects, arrays, cfg, torch.float64)
    compare_states("tilted_sources", out, r32, r64, TOL)
