"""Full 3x3 anisotropic materials on the GPU against the oracle.

A 9-component inverse permittivity / permeability or conductivity runs that side's tensor
half-steps (fdtdx/fdtd/update.py:356-492, 751-807, reverse :641-676, :956-995): the curl
(CPML terms included) into a scratch field, then F_i = sum_j A_ij F_j@i + s sum_j B_ij
curl_j@i with the four-point averages of fdtdx/fdtd/misc.py:132-213 for the off-diagonal
terms.  Sources take the tensor branches (dipole contraction, TFSF face rows) and the energy
detector 0.5 E.eps.E + 0.5 H.mu.H.  Tolerance: relative L2 <= 1e-4 against the float32
oracle (float64 reported).
"""

from __future__ import annotations

import math

import pytest
import torch

import fdtdx_gb300 as fx
from fdtdx_gb300.engine import Scene
from oracle import fdtd_oracle as O
from tests.helpers import compare_states, log_result, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-4
C0 = 299792458.0
FACES = ("min_x", "max_x", "min_y", "max_y", "min_z", "max_z")
EPS = (3.0, 0.6, 0.2, 0.6, 2.5, 0.3, 0.2, 0.3, 2.0)
MU = (1.6, -0.2, 0.1, -0.2, 1.3, 0.15, 0.1, 0.15, 1.4)
SIG_E = (2e4, 5e3, 0.0, 5e3, 1e4, 0.0, 0.0, 0.0, 4e3)
SIG_H = (3e9, 0.0, 1e9, 0.0, 2e9, 0.0, 1e9, 0.0, 2.5e9)


def _cfg(steps, dx=50e-9, record=False):
    return fx.SimulationConfig(time=steps * 0.99 / math.sqrt(3) * dx / C0, grid=fx.UniformGrid(dx),
                               gradient_config=fx.GradientConfig(recorder=fx.Recorder()) if record else None)


def _tensor_block(name, sl, lossy=True):
    return fx.UniformMaterialObject(name=name, grid_slice_tuple=sl, material=fx.Material(
        permittivity=EPS, permeability=MU, electric_conductivity=SIG_E if lossy else 0.0,
        magnetic_conductivity=SIG_H if lossy else 0.0))


def _seeded(shape, seed, complex_=False):
    g = torch.Generator().manual_seed(seed)

    def rnd():
        r = torch.randn((3, *shape), generator=g) * 1e-3
        return torch.complex(r, torch.randn((3, *shape), generator=g) * 1e-3) if complex_ else r

    return rnd(), rnd()


CASES = {
    "cpml": ({}, None, dict(kappa_end=1.5)),
    "periodic_pec_pmc": ({"min_x": "periodic", "max_x": "periodic", "min_y": "pec", "max_y": "pmc"}, None, {}),
    "bloch_cpml": ({f: "bloch" for f in FACES[:4]}, (1.1e6, -0.7e6, 0.0), {}),
}


@pytest.mark.parametrize("case", list(CASES))
def test_tensor_seeded_steps_match_oracle(case):
    """Seeded fields, 12 steps, a lossy block with off-diagonal eps, mu, sigma_E and sigma_H
    tensors: CPML on every face (kappa != 1); periodic x with PEC / PMC walls; Bloch x and y
    (complex fields) with CPML z.  E, H and psi."""
    types, kv, kw = CASES[case]
    shape = (14, 12, 16)
    cfg = _cfg(12)
    vol = fx.SimulationVolume(shape=shape)
    bc = fx.BoundaryConfig.from_uniform_bound(4, override_types=types, **({"bloch_vector": kv} if kv else {}), **kw)
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
    objs.append(_tensor_block("blk", ((2, 12), (1, 10), (3, 13))))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cuda")
    assert arrays.inv_permittivities.shape[0] == 9 and arrays.inv_permeabilities.shape[0] == 9
    assert arrays.electric_conductivity.shape[0] == 9 and arrays.magnetic_conductivity.shape[0] == 9
    cplx = kv is not None
    E0, H0 = _seeded(shape, 3, cplx)
    sc32 = O.OracleScene(objects, arrays, cfg, torch.float32)
    sc64 = O.OracleScene(objects, arrays, cfg, torch.float64)
    work = arrays.aset("fields->E", E0.cuda().contiguous()).aset("fields->H", H0.cuda().contiguous())
    scene = Scene(objects, work, cfg)
    assert scene.full_tensor
    scene.forward(work, 0, 12, graph=False)
    scene.status()
    torch.cuda.synchronize()
    refs = []
    for sc in (sc32, sc64):
        st = sc.init_state()
        st.E, st.H = E0.to(sc.field_dtype), H0.to(sc.field_dtype)
        refs.append(O.run(sc, 12, state=st))
    compare_states(f"tensor_seeded_{case}", work, refs[0], refs[1], TOL)
    for p in sc32.pmls:
        for q in range(2):
            assert rel_l2(work.fields.psi_E[p.name][q], refs[0].psi_E[p.name][q]) <= 5 * TOL
            assert rel_l2(work.fields.psi_H[p.name][q], refs[0].psi_H[p.name][q]) <= 5 * TOL
    scene.close()


def test_tensor_sources_and_detectors_through_run_fdtd():
    """run_fdtd (CUDA graph) on a scene whose tensor block holds a tilted electric dipole and a
    magnetic dipole (full-tensor contraction, every component injected), a TFSF plane source in
    the isotropic background (9-component arrays: the face rows of the tensor branch), and
    energy (tensor form), flux, field and phasor detectors over the block."""
    wc = fx.WaveCharacter(wavelength=1.0e-6)
    shape = (28, 22, 20)
    blk = ((12, 22), (5, 17), (5, 15))
    objs = [fx.SimulationVolume(shape=shape)]
    objs += list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(5), objs[0]).values())
    objs += [
        _tensor_block("blk", blk),
        fx.PointDipoleSource(name="de", grid_slice_tuple=((16, 17), (10, 11), (9, 10)), polarization=2,
                             azimuth_angle=30.0, elevation_angle=15.0, wave_character=wc),
        fx.PointDipoleSource(name="dm", grid_slice_tuple=((15, 16), (12, 13), (10, 11)), polarization=0,
                             source_type="magnetic", wave_character=wc),
        fx.UniformPlaneSource(name="pl", grid_slice_tuple=((8, 9), (0, 22), (0, 20)), direction="+",
                              fixed_E_polarization_vector=(0, 1, 1), wave_character=wc),
        fx.EnergyDetector(name="en", grid_slice_tuple=blk, reduce_volume=True),
        fx.EnergyDetector(name="en_vol", grid_slice_tuple=((14, 18), (8, 12), (7, 11))),
        fx.PoyntingFluxDetector(name="fl", grid_slice_tuple=((22, 23), (5, 17), (5, 15)), direction="+"),
        fx.FieldDetector(name="f", grid_slice_tuple=((12, 22), (5, 17), (10, 11)), components=("Ex", "Ey", "Hz")),
        fx.PhasorDetector(name="ph", grid_slice_tuple=blk, wave_characters=(wc,)),
    ]
    objects, arrays, _, cfg, _ = fx.place_objects(objs, _cfg(120), device="cuda")
    assert arrays.inv_permittivities.shape[0] == 9
    _, out = fx.run_fdtd(arrays, objects, cfg)
    torch.cuda.synchronize()
    res = [O.run(O.OracleScene(objects, arrays, cfg, dt)) for dt in (torch.float32, torch.float64)]
    assert res[1].det["en"]["energy"].abs().max() > 0
    compare_states("tensor_sources_detectors", out, res[0], res[1], TOL)


def test_tensor_branch_equals_diagonal_branch_on_the_gpu():
    """A diagonal material given as 9-component arrays (the tensor half-steps) against the same
    material as 3-component arrays (the diagonal kernels), 60 steps with a dipole and CPML:
    both GPU paths agree to float32 rounding."""
    shape = (20, 18, 16)
    objs = [fx.SimulationVolume(shape=shape)]
    objs += list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(4), objs[0]).values())
    objs += [fx.UniformMaterialObject(name="blk", grid_slice_tuple=((5, 15), (4, 14), (4, 12)), material=fx.Material(
                 permittivity=(2.0, 3.0, 4.0), permeability=(1.5, 1.2, 1.8), electric_conductivity=(1e4, 2e4, 0.0))),
             fx.PointDipoleSource(name="d", grid_slice_tuple=((10, 11), (9, 10), (8, 9)), polarization=1,
                                  wave_character=fx.WaveCharacter(wavelength=1.0e-6))]
    objects, arrays, _, cfg, _ = fx.place_objects(objs, _cfg(60), device="cuda")

    def as9(t):
        out = torch.zeros((9, *t.shape[1:]), device=t.device)
        for q in range(3):
            out[4 * q] = t[min(q, t.shape[0] - 1)]
        return out

    _, a3 = fx.run_fdtd(arrays, objects, cfg)
    a9 = arrays.aset("inv_permittivities", as9(arrays.inv_permittivities)).aset(
        "inv_permeabilities", as9(arrays.inv_permeabilities)).aset(
        "electric_conductivity", as9(arrays.electric_conductivity))
    _, b9 = fx.run_fdtd(a9, objects, cfg)
    torch.cuda.synchronize()
    eE, eH = rel_l2(b9.fields.E, a3.fields.E), rel_l2(b9.fields.H, a3.fields.H)
    log_result("tensor_vs_diagonal_branch", rel_l2_E=eE, rel_l2_H=eH)
    assert a3.fields.E.abs().max() > 0 and eE <= 1e-5 and eH <= 1e-5, (eE, eH)


def test_tensor_reverse_restores_with_recording():
    """Forward 40 steps with the CPML interfaces recorded, then 40 reverse steps (tensor reverse
    matrices A = M2^-1 M1, B = c M2^-1 inv): the interior returns to the seeded state, and the
    kernels' reverse agrees with the oracle's.  The tensor block keeps three cells from the
    CPML: a tensor cell's update averages the curl one cell away, so a block reaching into
    the absorbing layers would read curls with frozen psi there, and the reconstruction (the
    reference's as well as this one) would no longer be exact."""
    from fdtdx_gb300.initialization import init_arrays

    shape = (18, 16, 20)
    vol = fx.SimulationVolume(shape=shape)
    objs = [vol] + list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(4), vol).values())
    objs.append(_tensor_block("blk", ((7, 11), (7, 9), (7, 13)), lossy=False))
    objects, _, _, cfg, _ = fx.place_objects(objs, _cfg(40, record=True), device="cuda")
    arrays = init_arrays(objects, cfg, device="cuda")
    E0, H0 = _seeded(shape, 8)
    work = arrays.aset("fields->E", E0.cuda()).aset("fields->H", H0.cuda())
    scene = Scene(objects, work, cfg, record_interfaces=True)
    scene.forward(work, 0, 40)
    scene.reverse(work, 40, 40)
    scene.status()
    torch.cuda.synchronize()
    inner = (slice(None), slice(5, -5), slice(5, -5), slice(5, -5))
    eE = rel_l2(work.fields.E[inner], E0[inner])
    eH = rel_l2(work.fields.H[inner], H0[inner])
    sc = O.OracleScene(objects, arrays, cfg, torch.float64)
    st = sc.init_state()
    st.E, st.H = E0.double(), H0.double()
    st = O.run(sc, 40, record_boundaries=True, state=st)
    for _ in range(40):
        st = O.backward(sc, st)
    eo = rel_l2(work.fields.E[inner], st.E[inner])
    log_result("tensor_reverse_roundtrip", rel_l2_E=eE, rel_l2_H=eH, vs_oracle_reverse=eo)
    assert eE < 1e-3 and eH < 1e-3 and eo < 1e-3
    scene.close()


def test_tensor_gradient_is_refused():
    """The reversible gradient of tensor materials is not built: refused on the host."""
    shape = (10, 10, 10)
    objs = [fx.SimulationVolume(shape=shape), _tensor_block("blk", ((2, 8), (2, 8), (2, 8)), lossy=False)]
    objects, arrays, _, cfg, _ = fx.place_objects(objs, _cfg(8, record=True), device="cuda")
    ie = arrays.inv_permittivities.clone().requires_grad_(True)
    with pytest.raises(NotImplementedError, match="3x3"):
        fx.reversible_fdtd(arrays.aset("inv_permittivities", ie), objects, cfg)
