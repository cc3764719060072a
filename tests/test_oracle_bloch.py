"""Bloch boundaries on the oracle (CPU): complex fields with a phase on the wrap halo.

The oracle states the complex path (the checker of the GPU kernels' complex fields).  Pins:

* the phase exp(i k L) of the boundary's axis component, unit magnitude, one at k = 0
  (tests/unit/objects/boundaries/test_bloch.py:109-206), and the ghost layers of the padded
  field: the '+' layer is the wrapped first layer times the phase, the '-' layer the wrapped
  last layer times its conjugate (objects/boundaries/bloch.py:59-94);
* a zero Bloch vector is the periodic boundary: same (real) fields, same phasor
  (tests/simulation/physics/boundaries/test_bloch_zero_vector.py, 1e-4; here bitwise);
* one forward and one backward step restore seeded complex fields at atol 1e-5 in float32,
  with Bloch on every face (k = (1e6, 0, 0)) and with Bloch x, y plus CPML z and interface
  recording (tests/simulation/fdtd/test_time_reversal.py:311-328, 497-520); ten steps each
  way in float64 restore them to rel 1e-9;
* the reference's oblique-incidence check itself: a 30-degree TE plane wave in a 20-cell
  Bloch cell (k_x = k0 sin 30 degrees) crossing a vacuum / eps_r = 4 interface transmits
  T = 0.854 within 5% (tests/simulation/physics/boundaries/test_bloch_oblique.py:1-205; the
  oracle gives 0.851);
* the reversible gradient on complex fields equals autograd through the complex run
  (float64, rel 1e-9), finite and non-zero (test_time_reversal.py:687-800);
* the library builds the complex description of a non-zero Bloch vector and refuses the
  reversible gradient of such a scene before any device work (its forward and reverse steps
  run on the GPU: tests/test_gpu_bloch.py).
"""

import cmath
import math

import pytest
import torch

import fdtdx_gb300 as fx
from oracle import fdtd_oracle as O

C0 = 299792458.0
FACES = ("min_x", "max_x", "min_y", "max_y", "min_z", "max_z")


def _scene(types: dict, kv=(0.0, 0.0, 0.0), shape=(10, 9, 8), dx=50e-9, steps=4, dtype=torch.float32, record=False,
           extra=()):
    cfg = fx.SimulationConfig(time=steps * 0.99 / math.sqrt(3) * dx / C0, grid=fx.UniformGrid(dx),
                              gradient_config=fx.GradientConfig(recorder=fx.Recorder()) if record else None)
    vol = fx.SimulationVolume(shape=shape)
    bc = fx.BoundaryConfig.from_uniform_bound(3, override_types=types, bloch_vector=kv)
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values()) + list(extra)
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    return objects, arrays, cfg, O.OracleScene(objects, arrays, cfg, dtype=dtype)


def _seed_complex(sc, seed=42):
    g = torch.Generator().manual_seed(seed)
    st = sc.init_state()
    real = sc.dtype

    def rnd():
        return torch.complex(torch.randn(st.E.shape, generator=g, dtype=real),
                             torch.randn(st.E.shape, generator=g, dtype=real)) * 1e-3

    st.E, st.H = rnd(), rnd()
    return st


def test_bloch_phase_and_ghost_layers():
    kv = (2.0e6, -1.5e6, 0.0)
    objects, arrays, cfg, sc = _scene({f: "bloch" for f in FACES[:4]}, kv)
    bl = {(b.axis, b.direction): b for b in objects.boundary_objects if isinstance(b, fx.BlochBoundary)}
    for (axis, _d), b in bl.items():
        L = sc.shape[axis] * sc.dx
        ph = b.get_bloch_phase(sc.shape, sc.dx)
        assert abs(ph - cmath.exp(1j * kv[axis] * L)) < 1e-12 and abs(abs(ph) - 1.0) < 1e-12
        assert b.needs_complex_fields
    zero = fx.BlochBoundary(axis=0, direction="+", bloch_vector=(0.0, 3e6, 0.0))
    assert not zero.needs_complex_fields and zero.get_bloch_phase((4, 4, 4), 1e-8) == 1.0
    assert sc.field_dtype == torch.complex64 and len(sc.bloch) == 4
    g = torch.Generator().manual_seed(3)
    F = torch.complex(torch.randn(3, *sc.shape, generator=g), torch.randn(3, *sc.shape, generator=g))
    P = sc.pad(F)
    ph_x, ph_y = (cmath.exp(1j * kv[a] * sc.shape[a] * sc.dx) for a in (0, 1))
    inner = P[:, :, 1:-1, 1:-1]
    assert torch.allclose(inner[:, -1], F[:, 0] * ph_x, atol=1e-6) and torch.allclose(inner[:, 0], F[:, -1] * ph_x.conjugate(),
                                                                                      atol=1e-6)
    inner = P[:, 1:-1, :, 1:-1]
    assert torch.allclose(inner[:, :, -1], F[:, :, 0] * ph_y, atol=1e-6)
    assert torch.allclose(inner[:, :, 0], F[:, :, -1] * ph_y.conjugate(), atol=1e-6)
    assert torch.count_nonzero(P[:, 1:-1, 1:-1, 0]) == 0 and torch.count_nonzero(P[:, 1:-1, 1:-1, -1]) == 0
    # a corner ghost carries both axes' phases
    assert torch.allclose(P[:, -1, -1, 1:-1], F[:, 0, 0] * ph_x * ph_y, atol=1e-6)


def test_zero_vector_is_periodic():
    dx, nz = 50e-9, 80
    wc = fx.WaveCharacter(wavelength=1e-6)

    def extra():
        return (fx.UniformPlaneSource(name="s", grid_slice_tuple=((0, 3), (0, 3), (12, 13)), direction="+",
                                      fixed_E_polarization_vector=(1, 0, 0), wave_character=wc),
                fx.PhasorDetector(name="ph", grid_slice_tuple=((1, 2), (1, 2), (17, 18)), wave_characters=(wc,),
                                  components=("Ex",), reduce_volume=True))

    out = []
    for bt in ("periodic", "bloch"):
        _, _, _, sc = _scene({f: bt for f in FACES[:4]}, shape=(3, 3, nz), dx=dx, steps=600, extra=extra())
        assert sc.field_dtype == torch.float32
        out.append(O.run(sc))
    assert torch.equal(out[0].E, out[1].E) and torch.equal(out[0].det["ph"]["phasor"], out[1].det["ph"]["phasor"])
    assert out[0].det["ph"]["phasor"].abs().max() > 0


@pytest.mark.parametrize("mixed", [False, True])
def test_time_reversal_one_step_complex(mixed):
    types = {f: "bloch" for f in (FACES[:4] if mixed else FACES)}
    kv = (1e6, 1e6, 0.0) if mixed else (1e6, 0.0, 0.0)
    objs = (fx.UniformMaterialObject(name="blk", grid_slice_tuple=((3, 7), (2, 6), (3, 6)),
                                     material=fx.Material(permittivity=4.0)),)
    _, _, _, sc = _scene(types, kv, record=mixed, extra=objs)
    assert sc.field_dtype == torch.complex64 and (len(sc.pmls) == 2) == mixed
    st = _seed_complex(sc)
    E0, H0 = st.E.clone(), st.H.clone()
    fwd = O.forward(sc, st, record_detectors=False, record_boundaries=mixed)
    if mixed:
        assert all(v.is_complex() for v in fwd.rec[0].values())
    bwd = O.backward(sc, fwd)
    assert torch.allclose(bwd.E, E0, atol=1e-5) and torch.allclose(bwd.H, H0, atol=1e-5)
    assert (fwd.E - E0).abs().max() > 1e-5  # the step did move the fields


def test_time_reversal_multistep_complex_fp64():
    objs = (fx.UniformMaterialObject(name="blk", grid_slice_tuple=((3, 7), (2, 6), (3, 6)),
                                     material=fx.Material(permittivity=4.0, electric_conductivity=2e4,
                                                          magnetic_conductivity=3e4)),)
    _, _, _, sc = _scene({f: "bloch" for f in FACES}, (1.3e6, -0.7e6, 2.1e6), steps=10, dtype=torch.float64,
                         extra=objs)
    assert sc.field_dtype == torch.complex128 and len(sc.bloch) == 6
    st = _seed_complex(sc)
    E0, H0 = st.E.clone(), st.H.clone()
    for _ in range(10):
        st = O.forward(sc, st, record_detectors=False)
    for _ in range(10):
        st = O.backward(sc, st)
    assert float((st.E - E0).abs().max() / E0.abs().max()) < 1e-9
    assert float((st.H - H0).abs().max() / H0.abs().max()) < 1e-9


def test_bloch_oblique_fresnel_te():
    wl, dx, nx, nz = 1e-6, 25e-9, 20, 160
    theta = math.radians(30.0)
    k_x = 2 * math.pi / wl * math.sin(theta)
    out = []
    for diel in (False, True):
        cfg = fx.SimulationConfig(time=120e-15, grid=fx.UniformGrid(dx))
        vol = fx.SimulationVolume(shape=(nx, 3, nz))
        bc = fx.BoundaryConfig.from_uniform_bound(10, override_types={"min_x": "bloch", "max_x": "bloch",
                                                                      "min_y": "periodic", "max_y": "periodic"},
                                                  bloch_vector=(k_x, 0.0, 0.0))
        objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
        if diel:
            objs.append(fx.UniformMaterialObject(name="d", grid_slice_tuple=((0, nx), (0, 3), (80, nz)),
                                                 material=fx.Material(permittivity=4.0)))
        objs.append(fx.UniformPlaneSource(name="src", grid_slice_tuple=((0, nx), (0, 3), (14, 15)), direction="+",
                                          fixed_E_polarization_vector=(0, 1, 0), azimuth_angle=30.0,
                                          wave_character=fx.WaveCharacter(wavelength=wl)))
        objs.append(fx.PoyntingFluxDetector(name="flux", grid_slice_tuple=((0, nx), (0, 3), (120, 121)), direction="+",
                                            reduce_volume=True))
        objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
        sc = O.OracleScene(objects, arrays, cfg, torch.float32)
        assert sc.field_dtype == torch.complex64
        st = O.run(sc, sc.T)
        spp = round(wl / (C0 * sc.dt))
        out.append(float(st.det["flux"]["poynting_flux"][:, 0].double()[-10 * spp:].mean()))
    s0, s1 = out
    assert s0 > 0 and s1 > 0
    tt = math.asin(math.sin(theta) / 2.0)
    t_ref = (2.0 * math.cos(tt)) / math.cos(theta) * (2.0 * math.cos(theta) / (math.cos(theta) + 2.0 * math.cos(tt))) ** 2
    assert abs(s1 / s0 - t_ref) / t_ref < 0.05, (s1 / s0, t_ref)


def test_library_bloch_description_and_gradient_refusal():
    """A non-zero Bloch vector gives complex fields (the container's E, H and psi are
    complex64) and a plan description with the axis' phase exp(i k L) on the '+' ghost; the
    inv_permeabilities gradient of such a scene is refused before any device work (the
    inv_permittivities gradient runs on the device)."""
    from fdtdx_gb300.engine import Scene

    kv = (1e6, 0.0, 0.0)
    objects, arrays, cfg, sc = _scene({f: "bloch" for f in FACES[:2]}, kv)
    assert arrays.fields.E.dtype == torch.complex64 and arrays.fields.H.dtype == torch.complex64
    assert all(t.dtype == torch.complex64 for pair in arrays.fields.psi_E.values() for t in pair)
    scene = Scene(objects, arrays, cfg)
    d = scene.desc
    ph = cmath.exp(1j * kv[0] * sc.shape[0] * sc.dx)
    assert scene.complex_fields and d.bloch_axes == 1 and d.periodic[0] == 1
    assert abs(d.bloch_cos[0] - ph.real) < 1e-7 and abs(d.bloch_sin[0] - ph.imag) < 1e-7
    objects, arrays, cfg, _ = _scene({f: "bloch" for f in FACES[:2]}, kv, record=True)
    mu = torch.ones((1, *arrays.inv_permittivities.shape[1:]), requires_grad=True)
    with pytest.raises(NotImplementedError, match="complex"):
        fx.reversible_fdtd(arrays.aset("inv_permeabilities", mu), objects, cfg)


@pytest.mark.parametrize("pml", [False, True])
def test_reversible_gradient_with_complex_fields(pml):
    """The reversible VJP on complex Bloch fields: d sum|E_T|^2 / d inv_eps equals autograd
    through the whole complex run (float64; all-Bloch box: everywhere, Bloch x, y with CPML z:
    away from the absorbing slabs), finite and non-zero (tests/simulation/fdtd/
    test_time_reversal.py:687-800 checks finiteness and non-zero for PML + Bloch)."""
    dx, n, steps = 50e-9, 10, 60
    cfg = fx.SimulationConfig(time=steps * 0.99 / math.sqrt(3) * dx / C0, grid=fx.UniformGrid(dx),
                              gradient_config=fx.GradientConfig(recorder=fx.Recorder()))
    vol = fx.SimulationVolume(shape=(n, n, n + (8 if pml else 0)))
    types = {f: "bloch" for f in FACES}
    if pml:
        types["min_z"] = types["max_z"] = "pml"
    bc = fx.BoundaryConfig.from_uniform_bound(4, override_types=types,
                                              bloch_vector=(1e6, 1.7e6, 0.0 if pml else 0.9e6))
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
    objs.append(fx.UniformMaterialObject(name="slab", grid_slice_tuple=((0, n), (0, n), (3, 7)),
                                         material=fx.Material(permittivity=2.0, electric_conductivity=1e2)))
    objs.append(fx.PointDipoleSource(name="dip", grid_slice_tuple=((5, 6), (5, 6), (5, 6)), polarization=0,
                                     wave_character=fx.WaveCharacter(frequency=C0 / 800e-9)))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    sc = O.OracleScene(objects, arrays, cfg, torch.float64)
    assert sc.field_dtype == torch.complex128
    T = cfg.time_steps_total
    ie = sc.inv_eps.clone().requires_grad_(True)
    st = sc.init_state()
    for _ in range(T):
        st = O.forward(sc, st, inv_eps=ie)
    (g_chk,) = torch.autograd.grad((st.E.abs() ** 2).sum(), [ie])
    final = O.run(sc, T, record_boundaries=True)
    g_rev = O.reversible_gradient(sc, final, {}, cot_E=2 * final.E)
    assert not g_rev.is_complex() and torch.isfinite(g_rev).all()
    sl = (slice(None), slice(None), slice(None), slice(5, -5)) if pml else (slice(None),) * 4
    a, b = g_rev[sl], g_chk[sl]
    assert b.abs().max() > 0 and (a - b).abs().max() / b.abs().max() < 1e-9
