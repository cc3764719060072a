"""The algebra of the split CPML half-steps, pinned on the CPU in float64.

The split kernels (``fdtd_split.cuh``) run the plain Yee update of every cell and add the
slab cells' CPML terms afterwards, one axis at a time:

    forward:  F_new = [(1 - q) F + s c m curl] / (1 + q) + s c m dcurl / (1 + q)
    reverse:  F_old = [(1 + q) F - s c m curl] / (1 - q) - s c m dcurl / (1 - q)

with ``dcurl`` the terms of ax_term (psi advanced in a forward step, frozen in a reverse one).
This test restates that decomposition with the oracle's own building blocks (``curl_E`` /
``curl_H`` without slabs for the plain curl, ``step_cpml`` per slab for the terms) and checks
it against the oracle's fused half-steps on a scene with kappa != 1, electric and magnetic
conductivity and slabs meeting at edges and corners.
"""

import math

import torch

import fdtdx_gb300 as fx
from fdtdx_gb300 import scenes
from oracle import fdtd_oracle as O


def _scene():
    dx = 50e-9
    dt = 0.99 / math.sqrt(3) * dx / 299792458.0
    cfg = fx.SimulationConfig(time=30 * dt, grid=fx.UniformGrid(dx))
    vol = fx.SimulationVolume(shape=(18, 16, 20))
    bc = fx.BoundaryConfig.from_uniform_bound(5, "pml", kappa_end=1.7)
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
    objs.append(fx.UniformMaterialObject(name="blk", grid_slice_tuple=((1, 14), (2, 15), (0, 17)),
                                         material=fx.Material(permittivity=(4.0, 3.0, 5.0), electric_conductivity=2e4,
                                                              permeability=1.3, magnetic_conductivity=3e9)))
    objs.append(fx.PointDipoleSource(name="d", grid_slice_tuple=((9, 10), (8, 9), (10, 11)), polarization=2,
                                     wave_character=fx.WaveCharacter(wavelength=1.55e-6),
                                     temporal_profile=scenes.pulse_5fs()))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg)
    return O.OracleScene(objects, arrays, cfg, torch.float64)


def _slab_terms(sc, F_pad, psi, eside, advance):
    """dcurl of every slab, axis by axis, and the psi each slab stores (the kernels' per-axis
    correction launches)."""
    if eside:  # backward differences of H
        c = (slice(1, -1), slice(1, -1), slice(1, -1))
        d = {(0, 2): F_pad[2][c] - F_pad[2][:-2, 1:-1, 1:-1], (0, 1): F_pad[1][c] - F_pad[1][:-2, 1:-1, 1:-1],
             (1, 0): F_pad[0][c] - F_pad[0][1:-1, :-2, 1:-1], (1, 2): F_pad[2][c] - F_pad[2][1:-1, :-2, 1:-1],
             (2, 1): F_pad[1][c] - F_pad[1][1:-1, 1:-1, :-2], (2, 0): F_pad[0][c] - F_pad[0][1:-1, 1:-1, :-2]}
    else:  # forward differences of E
        c = (slice(1, -1), slice(1, -1), slice(1, -1))
        d = {(0, 2): F_pad[2][2:, 1:-1, 1:-1] - F_pad[2][c], (0, 1): F_pad[1][2:, 1:-1, 1:-1] - F_pad[1][c],
             (1, 0): F_pad[0][1:-1, 2:, 1:-1] - F_pad[0][c], (1, 2): F_pad[2][1:-1, 2:, 1:-1] - F_pad[2][c],
             (2, 1): F_pad[1][1:-1, 1:-1, 2:] - F_pad[1][c], (2, 0): F_pad[0][1:-1, 1:-1, 2:] - F_pad[0][c]}
    dcurls, new_psi = [], {}
    for ax in range(3):
        dc = torch.zeros((3, *sc.shape), dtype=torch.float64)
        for pml in sc.pmls:
            if pml.axis != ax:
                continue
            # d1 of component (ax + 2) % 3, d2 of component (ax + 1) % 3, both along ax
            d1 = d[(ax, (ax + 2) % 3)][pml.grid_slice]
            d2 = d[(ax, (ax + 1) % 3)][pml.grid_slice]
            p1, p2 = psi[pml.name]
            c1, c2, q1, q2 = O.step_cpml(pml, d1, d2, p1, p2, not eside, advance)
            dc[(ax + 1) % 3][pml.grid_slice] -= c1
            dc[(ax + 2) % 3][pml.grid_slice] += c2
            new_psi[pml.name] = (q1, q2)
        dcurls.append(dc)
    return dcurls, new_psi


def _factor(sc, eside, m):
    sig = sc.sigma_E if eside else sc.sigma_H
    if sig is None:
        return 0.0
    return sc.courant * sig * (O.ETA0 if eside else 1 / O.ETA0) * m / 2


def test_split_equals_fused_forward_and_reverse():
    sc = _scene()
    st = O.run(sc, 12)  # fields, psi and the source's history non-trivial
    c = sc.courant
    # ---- forward E half-step (sources left out on both sides: they follow the update)
    m, q = sc.inv_eps, _factor(sc, True, sc.inv_eps)
    H_pad = sc.pad(st.H)
    curl_fused, psi_fused = O.curl_H(H_pad, st.psi_E, sc.pmls, True)
    fused = ((1 - q) * st.E + c * curl_fused * m) / (1 + q)
    curl_plain, _ = O.curl_H(H_pad, {}, [], True)
    split = ((1 - q) * st.E + c * curl_plain * m) / (1 + q)
    dcurls, psi_split = _slab_terms(sc, H_pad, st.psi_E, True, True)
    for dc in dcurls:  # x, y, z launches in turn
        split = split + c * m * dc / (1 + q)
    assert torch.allclose(split, fused, rtol=1e-12, atol=1e-12 * fused.abs().max())
    for k in psi_fused:
        for a, b in zip(psi_split[k], psi_fused[k]):
            assert torch.equal(a, b)
    # ---- forward H half-step on the new E
    E1 = fused
    m, q = sc.inv_mu, _factor(sc, False, sc.inv_mu)
    E_pad = sc.pad(E1)
    curl_fused, psi_fused = O.curl_E(E_pad, st.psi_H, sc.pmls, True)
    fused_H = ((1 - q) * st.H - c * curl_fused * m) / (1 + q)
    curl_plain, _ = O.curl_E(E_pad, {}, [], True)
    split_H = ((1 - q) * st.H - c * curl_plain * m) / (1 + q)
    dcurls, psi_split = _slab_terms(sc, E_pad, st.psi_H, False, True)
    for dc in dcurls:
        split_H = split_H - c * m * dc / (1 + q)
    assert torch.allclose(split_H, fused_H, rtol=1e-12, atol=1e-12 * fused_H.abs().max())
    for k in psi_fused:
        for a, b in zip(psi_split[k], psi_fused[k]):
            assert torch.equal(a, b)
    # ---- reverse E half-step (psi frozen): the oracle's update_E_reverse without sources
    m, q = sc.inv_eps, _factor(sc, True, sc.inv_eps)
    curl_fused, _ = O.curl_H(H_pad, st.psi_E, sc.pmls, False)
    fused_rev = ((1 + q) * E1 - c * curl_fused * m) / (1 - q)
    curl_plain, _ = O.curl_H(H_pad, {}, [], False)
    split_rev = ((1 + q) * E1 - c * curl_plain * m) / (1 - q)
    dcurls, psi_frozen = _slab_terms(sc, H_pad, st.psi_E, True, False)
    for dc in dcurls:
        split_rev = split_rev - c * m * dc / (1 - q)
    assert torch.allclose(split_rev, fused_rev, rtol=1e-12, atol=1e-12 * fused_rev.abs().max())
    for k in psi_frozen:
        for a, b in zip(psi_frozen[k], st.psi_E[k]):
            assert torch.equal(a, b)
    # not vacuous: every axis carried slab terms, and the forward step advanced psi
    assert all(dc.abs().max() > 0 for dc in dcurls)
    assert any(not torch.equal(psi_fused[k][0], st.psi_H[k][0]) for k in psi_fused)
