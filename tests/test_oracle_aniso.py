"""Pins of the oracle's full 3x3 anisotropic branch (CPU, float64).

The reference's own known-answer tests for the averaging stencils and the update matrices
(tests/unit/fdtd/test_fdtd_misc.py:158-395) are replayed on the oracle's restatement, and
the branch is checked to reduce to the diagonal update when the off-diagonal entries are
zero (the reference takes the diagonal branch for (1 | 3)-component arrays and the tensor
branch for 9-component ones; both must agree on a diagonal tensor).  The same holds for the
tensor branches of the sources (dipole contraction, TFSF faces, plane impedance and energy
normalisation) and of the energy detector, and the reference's full-tensor dipole check
(tests/unit/objects/sources/test_dipole.py:178-193) is replayed.  The GB300 library does not
build the tensor branch yet (it refuses 9-component arrays); these pins keep the oracle
ready for it.
"""

import math

import pytest
import torch

import fdtdx_gb300 as fx
from oracle import fdtd_oracle as O

C0 = 299792458.0


def _kat_field():
    """The padded (3, 3, 3, 3) field of the reference's averaging tests."""
    plane = [[[0, 0, 0], [0, 1, 0], [0, 0, 0]], [[0, 2, 0], [3, 4, 5], [0, 6, 0]], [[0, 0, 0], [0, 7, 0], [0, 0, 0]]]
    return torch.tensor([plane, plane, plane], dtype=torch.float64)


def test_avg_E_component_kats():
    f = _kat_field()
    expect = {(0, 1): (4 + 6 + 1 + 0) / 4, (0, 2): (4 + 5 + 1 + 0) / 4, (1, 0): (4 + 7 + 2 + 0) / 4,
              (1, 2): (4 + 5 + 2 + 0) / 4, (2, 0): (4 + 7 + 3 + 0) / 4, (2, 1): (4 + 6 + 3 + 0) / 4,
              (0, 0): (4 + 7 + 1 + 4) / 4, (1, 1): (4 + 6 + 2 + 4) / 4, (2, 2): (4 + 5 + 3 + 4) / 4}
    for (comp, loc), v in expect.items():
        got = O.avg_aniso_E(f, comp, loc)
        assert got.shape == (1, 1, 1) and math.isclose(got.item(), v), (comp, loc, got.item(), v)


def test_avg_H_component_kats():
    f = _kat_field()
    expect = {(0, 1): (4 + 2 + 7 + 0) / 4, (0, 2): (4 + 3 + 7 + 0) / 4, (1, 0): (4 + 1 + 6 + 0) / 4,
              (1, 2): (4 + 3 + 6 + 0) / 4, (2, 0): (4 + 1 + 5 + 0) / 4, (2, 1): (4 + 2 + 5 + 0) / 4,
              (0, 0): (4 + 1 + 7 + 4) / 4, (1, 1): (4 + 2 + 6 + 4) / 4, (2, 2): (4 + 3 + 5 + 4) / 4}
    for (comp, loc), v in expect.items():
        got = O.avg_aniso_H(f, comp, loc)
        assert got.shape == (1, 1, 1) and math.isclose(got.item(), v), (comp, loc, got.item(), v)


def test_update_matrices_kats():
    """misc.py:69-129: without conductivity A = I and B = c inv (forward and reverse); with it A
    differs from I and the forward and reverse A differ."""
    grid = (5, 5, 5)
    inv = torch.arange(3 * 3 * 5 * 5 * 5, dtype=torch.float64).reshape(3, 3, *grid)
    eye = torch.eye(3, dtype=torch.float64)[:, :, None, None, None].expand(3, 3, *grid)
    for rev in (False, True):
        A, B = O.aniso_update_matrices(inv, None, 0.5, 1.0, reverse=rev)
        assert torch.allclose(A, eye, atol=1e-6) and torch.allclose(B, 0.5 * inv, atol=1e-6)
    sigma = 0.5 * eye
    A, B = O.aniso_update_matrices(inv, sigma, 0.5, 1.0)
    Ar, _ = O.aniso_update_matrices(inv, sigma, 0.5, 1.0, reverse=True)
    assert not torch.allclose(A, eye) and A.shape == (3, 3, *grid) and torch.isfinite(A).all() and torch.isfinite(B).all()
    eye3 = torch.eye(3, dtype=torch.float64)[:, :, None, None, None].expand(3, 3, 3, 3, 3)
    Af, _ = O.aniso_update_matrices(eye3, 0.5 * eye3, 0.5, 1.0)
    Ar2, _ = O.aniso_update_matrices(eye3, 0.5 * eye3, 0.5, 1.0, reverse=True)
    assert not torch.allclose(Af, Ar2)


def test_expand_to_3x3():
    a = torch.rand(1, 2, 3, 4, dtype=torch.float64)
    b = torch.rand(3, 2, 3, 4, dtype=torch.float64)
    c = torch.rand(9, 2, 3, 4, dtype=torch.float64)
    ea, eb, ec = O.expand_to_3x3(a), O.expand_to_3x3(b), O.expand_to_3x3(c)
    assert ea.shape == eb.shape == ec.shape == (3, 3, 2, 3, 4)
    assert torch.equal(ea[1, 1], a[0]) and torch.equal(ea[0, 1], torch.zeros(2, 3, 4, dtype=torch.float64))
    assert torch.equal(eb[2, 2], b[2]) and torch.equal(ec[1, 2], c[5])
    es = O.expand_to_3x3(2.0)
    assert es.shape == (3, 3, 1, 1, 1) and es[0, 0].item() == 2.0 and es[0, 1].item() == 0.0


def _diag_scene(periodic: bool):
    dx = 50e-9
    steps = 6
    dt = 0.99 / math.sqrt(3) * dx / C0
    cfg = fx.SimulationConfig(time=steps * dt, grid=fx.UniformGrid(dx))
    vol = fx.SimulationVolume(shape=(14, 12, 10))
    bc = fx.BoundaryConfig.from_uniform_bound(3, "periodic" if periodic else "pml")
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
    objs.append(fx.UniformMaterialObject(
        name="blk", grid_slice_tuple=((3, 11), (2, 9), (2, 8)),
        material=fx.Material(permittivity=(2.0, 3.0, 4.0), permeability=(1.5, 1.2, 1.8),
                             electric_conductivity=(1e4, 2e4, 0.0), magnetic_conductivity=(0.0, 3e9, 1e9))))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    return objects, arrays, cfg


def _as9(x):
    return O.expand_to_3x3(x).reshape(9, *x.shape[1:])


@pytest.mark.parametrize("periodic", [False, True])
def test_tensor_branch_reduces_to_diagonal_branch(periodic):
    """A 9-component tensor holding a diagonal material gives the diagonal branch's update,
    forward and reverse, E and H, with conductivities and CPML (float64, 1e-12)."""
    objects, arrays, cfg = _diag_scene(periodic)
    sc = O.OracleScene(objects, arrays, cfg, torch.float64)
    g = torch.Generator().manual_seed(5)
    shape = sc.inv_eps.shape[1:]
    E = torch.randn((3, *shape), generator=g, dtype=torch.float64)
    H = torch.randn((3, *shape), generator=g, dtype=torch.float64)
    st = sc.init_state()
    psi_E = {k: (torch.randn(a.shape, generator=g, dtype=torch.float64), torch.randn(b.shape, generator=g,
                                                                                     dtype=torch.float64))
             for k, (a, b) in st.psi_E.items()}
    psi_H = {k: (torch.randn(a.shape, generator=g, dtype=torch.float64), torch.randn(b.shape, generator=g,
                                                                                     dtype=torch.float64))
             for k, (a, b) in st.psi_H.items()}
    ie3, im3 = sc.inv_eps, sc.inv_mu
    assert ie3.shape[0] == 3 and im3.shape[0] == 3
    e_diag, pe_diag = O.update_E(sc, 0, E, H, psi_E, ie3)
    e_full, pe_full = O.update_E(sc, 0, E, H, psi_E, _as9(ie3))
    h_diag, ph_diag = O.update_H(sc, 0, E, H, psi_H, im3)
    h_full, ph_full = O.update_H(sc, 0, E, H, psi_H, _as9(im3))
    er_diag = O.update_E_reverse(sc, 0, E, H, psi_E, ie3)
    er_full = O.update_E_reverse(sc, 0, E, H, psi_E, _as9(ie3))
    hr_diag = O.update_H_reverse(sc, 0, E, H, psi_H, im3)
    hr_full = O.update_H_reverse(sc, 0, E, H, psi_H, _as9(im3))
    for a, b in ((e_diag, e_full), (h_diag, h_full), (er_diag, er_full), (hr_diag, hr_full)):
        assert torch.allclose(a, b, rtol=1e-12, atol=1e-12)
    for k in pe_diag:
        for q in range(2):
            assert torch.equal(pe_diag[k][q], pe_full[k][q]) and torch.equal(ph_diag[k][q], ph_full[k][q])


def test_tensor_branch_off_diagonal_coupling_is_stable():
    """A symmetric positive-definite off-diagonal permittivity in a periodic box (no loss): the
    field energy stays bounded over 200 steps from a seeded start (the branch's four-point
    averages couple the components without blowing up at the Courant number 0.99/sqrt(3))."""
    objects, arrays, cfg = _diag_scene(True)
    sc = O.OracleScene(objects, arrays, cfg, torch.float64)
    sc.sigma_E = None
    sc.sigma_H = None
    sc.sources = []
    shape = sc.inv_eps.shape[1:]
    eps = torch.tensor([[3.0, 0.6, 0.2], [0.6, 2.5, 0.3], [0.2, 0.3, 2.0]], dtype=torch.float64)
    inv9 = torch.linalg.inv(eps).reshape(9, 1, 1, 1).expand(9, *shape).clone()
    g = torch.Generator().manual_seed(9)
    E = 1e-3 * torch.randn((3, *shape), generator=g, dtype=torch.float64)
    H = torch.zeros((3, *shape), dtype=torch.float64)
    st = sc.init_state()
    e0 = float((E**2).sum())
    peak = e0
    for t in range(200):
        E, _ = O.update_E(sc, t, E, H, st.psi_E, inv9)
        H, _ = O.update_H(sc, t, E, H, st.psi_H, 1.0)
        peak = max(peak, float((E**2).sum()))
    assert torch.isfinite(E).all() and peak < 100 * e0


def test_full_tensor_dipole_keeps_coupled_components():
    """An x-dipole in a medium whose inverse permittivity has the column (1, 2, 3) injects
    (1, 2, 3) times the same scalar (tests/unit/objects/sources/test_dipole.py:178-193)."""
    dx = 50e-9
    cfg = fx.SimulationConfig(time=20 * 0.99 / math.sqrt(3) * dx / C0, grid=fx.UniformGrid(dx))
    vol = fx.SimulationVolume(shape=(8, 8, 8))
    objs = [vol, fx.PointDipoleSource(name="d", grid_slice_tuple=((4, 5), (4, 5), (4, 5)), polarization=0,
                                      wave_character=fx.WaveCharacter(wavelength=1e-6))]
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    inv = torch.zeros((9, 8, 8, 8))
    inv[0], inv[3], inv[6] = 1.0, 2.0, 3.0
    sc = O.OracleScene(objects, arrays.aset("inv_permittivities", inv), cfg, torch.float32)
    E = O._source_update_E(sc, sc.sources[0], torch.zeros((3, 8, 8, 8)), sc.inv_eps, 10.0, False)
    v = E[:, 4, 4, 4]
    assert v[0] != 0 and torch.allclose(v[1], 2 * v[0], atol=1e-6) and torch.allclose(v[2], 3 * v[0], atol=1e-6)
    rest = E.clone()
    rest[:, 4, 4, 4] = 0
    assert torch.count_nonzero(rest) == 0


def test_tensor_sources_and_detectors_reduce_to_diagonal():
    """Six forward steps of a scene with a tilted electric dipole and a magnetic dipole inside a
    diagonal (eps, mu) block, a TFSF plane in vacuum, and energy / flux / phasor detectors: the
    9-component form of the same tensors gives the diagonal form's fields and detector states
    (the full-tensor source branches dipole.py:15-37, 219-232, tfsf.py:287-299, 384-393, the
    tensor impedance and energy of tfsf.py:144-190 and metrics.py:34-51; float64, 1e-11)."""
    dx = 50e-9
    steps = 6
    cfg = fx.SimulationConfig(time=steps * 0.99 / math.sqrt(3) * dx / C0, grid=fx.UniformGrid(dx))
    vol = fx.SimulationVolume(shape=(16, 12, 10))
    objs = [vol] + list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(3), vol).values())
    blk = ((7, 12), (2, 9), (2, 8))
    objs.append(fx.UniformMaterialObject(name="blk", grid_slice_tuple=blk, material=fx.Material(
        permittivity=(2.0, 3.0, 4.0), permeability=(1.5, 1.2, 1.8), electric_conductivity=(1e4, 2e4, 0.0))))
    wc = fx.WaveCharacter(wavelength=1e-6)
    objs += [
        fx.PointDipoleSource(name="de", grid_slice_tuple=((9, 10), (5, 6), (4, 5)), polarization=2, azimuth_angle=35.0,
                             elevation_angle=20.0, wave_character=wc),
        fx.PointDipoleSource(name="dm", grid_slice_tuple=((8, 9), (4, 5), (5, 6)), polarization=1,
                             source_type="magnetic", wave_character=wc),
        fx.UniformPlaneSource(name="pl", grid_slice_tuple=((4, 5), (3, 9), (3, 7)), direction="+",
                              fixed_E_polarization_vector=(0, 1, 1), wave_character=wc),
        fx.EnergyDetector(name="en", grid_slice_tuple=blk),
        fx.PoyntingFluxDetector(name="fl", grid_slice_tuple=((10, 11), (3, 9), (3, 7)), direction="+"),
        fx.PhasorDetector(name="ph", grid_slice_tuple=blk, wave_characters=(wc,)),
    ]
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    a9 = arrays.aset("inv_permittivities", _as9(arrays.inv_permittivities)).aset(
        "inv_permeabilities", _as9(arrays.inv_permeabilities))
    sc3 = O.OracleScene(objects, arrays, cfg, torch.float64)
    sc9 = O.OracleScene(objects, a9, cfg, torch.float64)
    assert sc9.inv_eps.shape[0] == 9 and sc9.inv_mu.shape[0] == 9
    for s3, s9 in zip(sc3.sources, sc9.sources):
        if s3.kind == "plane":
            for a, b in ((s3.E_inc, s9.E_inc), (s3.H_inc, s9.H_inc), (s3.off_E, s9.off_E), (s3.off_H, s9.off_H)):
                assert torch.allclose(a, b, rtol=1e-12, atol=1e-15)
    st3 = O.run(sc3, steps)
    st9 = O.run(sc9, steps)
    assert st3.E.abs().max() > 0 and st3.H.abs().max() > 0
    assert torch.allclose(st3.E, st9.E, rtol=1e-11, atol=1e-11 * st3.E.abs().max().item())
    assert torch.allclose(st3.H, st9.H, rtol=1e-11, atol=1e-11 * st3.H.abs().max().item())
    for name in ("en", "fl", "ph"):
        for k, v in st3.det[name].items():
            w = st9.det[name][k]
            assert torch.allclose(v, w, rtol=1e-10, atol=1e-10 * v.abs().max().item()), name
    assert st3.det["en"]["energy"].abs().max() > 0


def test_tensor_plane_source_in_anisotropic_medium_is_refused():
    """A plane source inside a genuinely anisotropic tensor medium is refused, as the reference's
    time-offset computation refuses it (fdtdx/core/grid.py:781-861)."""
    dx = 50e-9
    cfg = fx.SimulationConfig(time=4 * 0.99 / math.sqrt(3) * dx / C0, grid=fx.UniformGrid(dx))
    vol = fx.SimulationVolume(shape=(8, 8, 8))
    objs = [vol, fx.UniformPlaneSource(name="pl", grid_slice_tuple=((4, 5), (0, 8), (0, 8)), direction="+",
                                       fixed_E_polarization_vector=(0, 1, 0))]
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    eps = torch.tensor([[3.0, 0.6, 0.2], [0.6, 2.5, 0.3], [0.2, 0.3, 2.0]], dtype=torch.float64)
    inv9 = torch.linalg.inv(eps).reshape(9, 1, 1, 1).expand(9, 8, 8, 8).clone().float()
    with pytest.raises(NotImplementedError):
        O.OracleScene(objects, arrays.aset("inv_permittivities", inv9), cfg, torch.float32)
