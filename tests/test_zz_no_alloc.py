"""fdtd_detector_sample_noalloc against the plan's detector path (collected last on purpose).

A forward run through fdtd_forward records reducing FIELD, FLUX and ENERGY detectors;
the allocation-free entry point, called twice in a row through the C ABI on the final
fields (and H before the last H update), must reproduce the entry of the last step.
Both run the same kernels, so the tolerance is tight: relative 1e-6.
"""

import ctypes as C
import math

import pytest
import torch

import fdtdx_gb300 as fx
from fdtdx_gb300 import _native as N
from fdtdx_gb300.engine import Scene, detector_tables

pytestmark = pytest.mark.gpu
C0 = 299792458.0


def _scene(steps):
    dx = 40e-9
    dt = 0.99 / math.sqrt(3) * dx / C0
    cfg = fx.SimulationConfig(time=steps * dt, grid=fx.UniformGrid(dx))
    vol = fx.SimulationVolume(shape=(28, 26, 24), material=fx.Material(permittivity=1.5))
    objs = [vol] + list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(5), vol).values())
    objs.append(fx.UniformMaterialObject(name="blk", grid_slice_tuple=((10, 18), (9, 17), (8, 16)),
                                         material=fx.Material(permittivity=(3.0, 4.0, 6.0))))
    objs.append(fx.PointDipoleSource(name="d", grid_slice_tuple=((13, 14), (12, 13), (11, 12)), polarization=1,
                                     wave_character=fx.WaveCharacter(wavelength=1.0e-6)))
    R = ((9, 19), (8, 18), (7, 17))
    objs += [
        fx.FieldDetector(name="f_red", grid_slice_tuple=R, components=("Ex", "Hy", "Hz"), reduce_volume=True),
        fx.PoyntingFluxDetector(name="flux", grid_slice_tuple=((19, 20), (7, 19), (6, 18)), direction="+"),
        fx.PoyntingFluxDetector(name="flux_all", grid_slice_tuple=((11, 16), (10, 15), (9, 14)), direction="-",
                                keep_all_components=True, exact_interpolation=False),
        fx.EnergyDetector(name="energy", grid_slice_tuple=R, reduce_volume=True),
    ]
    return fx.place_objects(objs, cfg, device="cuda")


def test_noalloc_sample_matches_forward_detectors_twice():
    n = 48
    objects, arrays, _, cfg, _ = _scene(n)
    scene = Scene(objects, arrays, cfg)
    scene.forward(arrays, 0, n - 1, graph=False)
    torch.cuda.synchronize()
    H_prev = arrays.fields.H.clone()
    scene.forward(arrays, n - 1, 1, graph=False)
    torch.cuda.synchronize()
    lib = N.load()
    nx, ny, nz = objects.volume.grid_shape
    periodic = (C.c_int32 * 3)(0, 0, 0)
    mu = arrays.inv_permeabilities
    n_mu = mu.shape[0] if isinstance(mu, torch.Tensor) else 0
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for q, det in enumerate(scene.detectors):
        state = next(iter(arrays.detector_states[det.name].values()))
        slot = int(detector_tables(det, cfg)[0][n])
        expected = state[slot].reshape(-1)
        outs = []
        for _ in range(2):
            out = torch.full((expected.numel(),), float("nan"), device="cuda")
            rc = lib.fdtd_detector_sample_noalloc(
                C.byref(scene.desc.detectors[q]), nx, ny, nz, periodic,
                N.ptr(arrays.fields.E), N.ptr(H_prev), N.ptr(arrays.fields.H),
                N.ptr(arrays.inv_permittivities), arrays.inv_permittivities.shape[0],
                N.ptr(mu) if n_mu else None, n_mu, 1.0 if n_mu else float(mu), N.ptr(out), stream)
            assert rc == N.OK, det.name
            torch.cuda.synchronize()
            outs.append(out.cpu())
        exp = expected.cpu()
        assert torch.linalg.vector_norm(exp).item() > 0, det.name
        for out in outs:
            assert torch.allclose(out, exp, rtol=1e-6, atol=1e-6 * exp.abs().max().item()), (det.name, out, exp)
        assert torch.equal(outs[0], outs[1]), det.name


def _periodic_scene(steps):
    """All-periodic grid, an anisotropic magnetic block (n_mu = 3), regions touching the faces."""
    dx = 40e-9
    dt = 0.99 / math.sqrt(3) * dx / C0
    cfg = fx.SimulationConfig(time=steps * dt, grid=fx.UniformGrid(dx))
    n = (20, 18, 16)
    vol = fx.SimulationVolume(shape=n)
    objs = [vol] + list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(1, "periodic"),
                                                        vol).values())
    objs.append(fx.UniformMaterialObject(name="blk", grid_slice_tuple=((0, 20), (4, 14), (3, 12)),
                                         material=fx.Material(permittivity=(3.0, 4.0, 6.0),
                                                              permeability=(1.5, 1.2, 2.0))))
    objs.append(fx.PointDipoleSource(name="d", grid_slice_tuple=((9, 10), (8, 9), (7, 8)), polarization=2,
                                     wave_character=fx.WaveCharacter(wavelength=1.0e-6)))
    objs += [
        fx.PoyntingFluxDetector(name="flux_lo", grid_slice_tuple=((0, 1), (0, 18), (0, 16)), direction="-"),
        # all three components: the x flux through the last x plane is zero here, on the oracle too
        fx.PoyntingFluxDetector(name="flux_hi", grid_slice_tuple=((19, 20), (0, 18), (0, 16)), direction="+",
                                keep_all_components=True),
        fx.EnergyDetector(name="energy_all", grid_slice_tuple=((0, 20), (0, 18), (0, 16)), reduce_volume=True),
        fx.FieldDetector(name="e_only", grid_slice_tuple=((0, 20), (0, 18), (15, 16)), components=("Ex", "Ez"),
                         reduce_volume=True),
    ]
    return fx.place_objects(objs, cfg, device="cuda")


def test_noalloc_periodic_faces_and_magnetic_tensor():
    """Wrap-around co-location on every axis (regions on the faces), n_mu = 3, and an
    E-only exact FIELD sample called without H_prev (it reads no H)."""
    n = 40
    objects, arrays, _, cfg, _ = _periodic_scene(n)
    mu = arrays.inv_permeabilities
    assert isinstance(mu, torch.Tensor) and mu.shape[0] == 3
    scene = Scene(objects, arrays, cfg)
    scene.forward(arrays, 0, n - 1, graph=False)
    torch.cuda.synchronize()
    H_prev = arrays.fields.H.clone()
    scene.forward(arrays, n - 1, 1, graph=False)
    torch.cuda.synchronize()
    lib = N.load()
    nx, ny, nz = objects.volume.grid_shape
    periodic = (C.c_int32 * 3)(1, 1, 1)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for q, det in enumerate(scene.detectors):
        state = next(iter(arrays.detector_states[det.name].values()))
        slot = int(detector_tables(det, cfg)[0][n])
        exp = state[slot].reshape(-1).cpu()
        hp = None if det.name == "e_only" else N.ptr(H_prev)
        outs = []
        for _ in range(2):
            out = torch.full((exp.numel(),), float("nan"), device="cuda")
            rc = lib.fdtd_detector_sample_noalloc(
                C.byref(scene.desc.detectors[q]), nx, ny, nz, periodic, N.ptr(arrays.fields.E), hp,
                N.ptr(arrays.fields.H), N.ptr(arrays.inv_permittivities), arrays.inv_permittivities.shape[0],
                N.ptr(mu), 3, 1.0, N.ptr(out), stream)
            assert rc == N.OK, det.name
            torch.cuda.synchronize()
            outs.append(out.cpu())
        assert exp.abs().max().item() > 0, det.name  # (face fluxes are ~1e-24: a float32 norm underflows)
        for out in outs:
            assert torch.allclose(out, exp, rtol=1e-6, atol=1e-6 * exp.abs().max().item()), (det.name, out, exp)
        assert torch.equal(outs[0], outs[1]), det.name


def test_noalloc_rejects_regions_beyond_the_scratch():
    lib = N.load()
    d = N.DetectorDesc()
    d.kind = N.DET_FIELD
    d.comp_mask = 1
    d.lo[0] = d.lo[1] = d.lo[2] = 0
    d.hi[0] = d.hi[1] = d.hi[2] = 300  # 2.7e7 cells -> 105469 partial sums > 65536
    buf = torch.zeros(8, device="cuda")
    out = torch.zeros(1, device="cuda")
    periodic = (C.c_int32 * 3)(0, 0, 0)
    rc = lib.fdtd_detector_sample_noalloc(C.byref(d), 300, 300, 300, periodic, N.ptr(buf), N.ptr(buf), N.ptr(buf),
                                          N.ptr(buf), 1, None, 0, 1.0, N.ptr(out),
                                          C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == N.EINVAL
    assert (N.NOALLOC_SCRATCH_FLOATS // 1) * 256 < 300**3
