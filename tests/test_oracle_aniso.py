"""Pins of the oracle's full 3x3 anisotropic branch (CPU, float64).

The reference's own known-answer tests for the averaging stencils and the update matrices
(tests/unit/fdtd/test_fdtd_misc.py:158-395) are replayed on the oracle's restatement, and
the branch is checked to reduce to the diagonal update when the off-diagonal entries are
zero (the reference takes the diagonal branch for (1 | 3)-component arrays and the tensor
branch for 9-component ones; both must agree on a diagonal tensor).  The GB300 library does
not build this branch yet; these pins keep the oracle ready for it.
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
    sc.sources = []  # the sources' tensor-material handling is not part of this branch's pin
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
