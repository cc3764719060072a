"""The batched forward path against the per-simulation path and the oracle.

A batch mixes uneven grids (even and odd nz, so both z-vector widths), CPML and
periodic boundaries, dipole and plane sources, fused E-only phasors, H-reading phasors
(the parity twin of H) and reducing detectors.  Each simulation of the batch must match
the same simulation run alone through fdtd_forward (relative L2 <= 1e-5: the batch runs
the register-queue core where the single run may use the TMA core, so summation order
can differ) and the float32 oracle (<= 1e-4).  Graph, direct and autotuned runs agree
with each other exactly.
"""

import math

import pytest
import torch

import fdtdx_gb300 as fx
from fdtdx_gb300 import scenes
from fdtdx_gb300.batch import SimulationBatch
from fdtdx_gb300.engine import Scene
from oracle import fdtd_oracle as O
from tests.helpers import compare_states, log_result, rel_l2

pytestmark = pytest.mark.gpu
STEPS = 60


def _periodic_scene():
    dx = 40e-9
    dt = 0.99 / math.sqrt(3) * dx / 299792458.0
    cfg = fx.SimulationConfig(time=80 * dt, grid=fx.UniformGrid(dx))
    vol = fx.SimulationVolume(shape=(20, 22, 18))
    objs = [vol] + list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(1, "periodic"),
                                                        vol).values())
    objs.append(fx.UniformMaterialObject(name="blk", grid_slice_tuple=((5, 12), (6, 15), (4, 13)),
                                         material=fx.Material(permittivity=3.0)))
    objs.append(fx.PointDipoleSource(name="d", grid_slice_tuple=((10, 11), (11, 12), (9, 10)), polarization=0,
                                     wave_character=fx.WaveCharacter(wavelength=1.0e-6)))
    objs.append(fx.FieldDetector(name="f", grid_slice_tuple=((0, 20), (0, 22), (9, 10)), components=("Ex", "Hz"),
                                 reduce_volume=True))
    return fx.place_objects(objs, cfg, device="cuda")


def _sims():
    out = []
    o, a, _, c, _ = scenes.dipole_boxes(shape=(34, 30, 28), steps=80, n_boxes=5, pml=6, device="cuda")
    out.append((a, o, c))
    o, a, _, c = scenes.strip(shape=(40, 36, 29), steps=80, pml=6, device="cuda")[:4]
    out.append((a, o, c))
    o, a, _, c, _ = scenes.coupler(shape=(48, 44, 24), steps=80, scale=0.3, pml=6, device="cuda")
    out.append((a, o, c))
    o, a, _, c, _ = _periodic_scene()
    out.append((a, o, c))
    return out


def _alone(arrays, objects, config, steps):
    from fdtdx_gb300.fdtd import _materials_detached

    work = _materials_detached(arrays).reset()
    scene = Scene(objects, work, config)
    scene.forward(work, 0, steps, graph=False)
    torch.cuda.synchronize()
    scene.close()
    return work


def _states(arrays):
    out = {"E": arrays.fields.E, "H": arrays.fields.H}
    for dn, st in arrays.detector_states.items():
        for k, v in st.items():
            out[f"{dn}.{k}"] = v
    return out


@pytest.mark.parametrize("graph,autotune", [(False, False), (True, False), (True, True)])
def test_batch_matches_single_runs(graph, autotune):
    sims = _sims()
    batch = SimulationBatch(sims)
    batch.advance(STEPS, t0=[0] * len(sims), graph=graph, autotune=autotune)
    torch.cuda.synchronize()
    for q, (arrays, objects, config) in enumerate(sims):
        ref = _alone(arrays, objects, config, STEPS)
        got = batch.arrays[q]
        errs = {k: rel_l2(v, _states(ref)[k]) for k, v in _states(got).items()}
        log_result(f"batch_vs_single_{q}_g{int(graph)}_a{int(autotune)}", **errs)
        for k, e in errs.items():
            assert e <= 1e-5, (q, k, e)
    if autotune:
        t = batch.tuning()
        assert t["shell_chunk"] in (2, 4, 8) and t["blocks_per_sm"] in (4, 8, 16)
        assert t["mode"] in ("persistent", "branches", "fused")
    else:
        assert batch.launches_per_step() <= 13
    batch.close()


@pytest.mark.parametrize("graph", [False, True])
def test_batch_branch_mode_matches_single_runs(graph):
    """Mode 'branches': every simulation's own launch chain on its own stream; bitwise equal
    to the single runs (the same kernels, TMA cores included)."""
    sims = _sims()
    batch = SimulationBatch(sims)
    batch.set_mode("branches")
    batch.advance(STEPS, t0=[0] * len(sims), graph=graph, autotune=False)
    torch.cuda.synchronize()
    for q, (arrays, objects, config) in enumerate(sims):
        ref = _alone(arrays, objects, config, STEPS)
        for k, v in _states(batch.arrays[q]).items():
            assert torch.equal(v, _states(ref)[k]), (q, k)
    batch.close()


def test_batch_fused_mode_matches_persistent_mode_and_oracle():
    """Mode 'fused': every step of a call in ONE cooperative launch, the phases separated by
    bounded grid barriers.  The same device bodies as the persistent mode, so each simulation
    matches the persistent-mode batch (relative L2 <= 1e-6: detector sums may add in another
    order) and the single runs (<= 1e-5); two calls (an odd first chunk, so the parity twin
    is handed back) against the float32 / float64 oracle (<= 1e-4)."""
    sims = _sims()
    n = len(sims)
    ref = SimulationBatch(sims)
    ref.advance(STEPS, t0=[0] * n, graph=False, autotune=False)
    fused = SimulationBatch(sims)
    fused.set_mode("fused")
    assert fused.mode == "fused" and fused.launches_per_step() == 1
    fused.advance(23, t0=[0] * n, graph=True, autotune=False)
    fused.advance(STEPS - 23, graph=True, autotune=False)
    torch.cuda.synchronize()
    for q, (arrays, objects, config) in enumerate(sims):
        got, want = _states(fused.arrays[q]), _states(ref.arrays[q])
        errs = {k: rel_l2(v, want[k]) for k, v in got.items()}
        log_result(f"batch_fused_vs_persistent_{q}", **errs)
        for k, e in errs.items():
            assert e <= 1e-6, (q, k, e)
        alone = _states(_alone(arrays, objects, config, STEPS))
        for k, v in got.items():
            assert rel_l2(v, alone[k]) <= 1e-5, (q, k)
    for q in range(2):
        arrays, objects, config = sims[q]
        sc32 = O.OracleScene(objects, arrays, config, torch.float32)
        sc64 = O.OracleScene(objects, arrays, config, torch.float64)
        compare_states(f"batch_fused_oracle_{q}", fused.arrays[q], O.run(sc32, STEPS), O.run(sc64, STEPS), 1e-4)
    ref.close()
    fused.close()


def test_batch_fused_mode_barrier_expiry_is_reported_and_the_batch_stays_usable():
    """An injected block that never arrives at the first grid barrier: the other blocks' bounded
    waits run out, the call raises FDTD_ETIMEOUT, and the next call runs normally."""
    from fdtdx_gb300 import _native as N

    sims = _sims()[:2]
    ref = SimulationBatch(sims)
    ref.set_mode("fused")
    ref.advance(20, t0=[0, 0], graph=False, autotune=False)
    torch.cuda.synchronize()
    b = SimulationBatch(sims)
    b.set_mode("fused")
    assert N.load().fdtd_debug_inject(N.INJECT_BARRIER_EXPIRY, 1) == N.OK
    with pytest.raises(N.NativeError) as ei:
        b.advance(10, t0=[0, 0], graph=False, autotune=False)
    assert ei.value.code == N.ETIMEOUT
    for a in b.arrays:  # back to step 0 in place (the batch holds these tensors)
        for v in [a.fields.E, a.fields.H, *[x for pair in (*a.fields.psi_E.values(), *a.fields.psi_H.values())
                                              for x in pair]]:
            v.zero_()
        for st in a.detector_states.values():
            for v in st.values():
                v.zero_()
    b.advance(20, t0=[0, 0], graph=False, autotune=False)
    torch.cuda.synchronize()
    for q in range(2):
        for k, v in _states(b.arrays[q]).items():
            assert torch.allclose(v, _states(ref.arrays[q])[k], rtol=1e-6, atol=0), (q, k)
    ref.close()
    b.close()


def test_batch_against_oracle_and_continuation():
    """Two advance() calls (an odd first chunk, so the H parity twin is handed back) against
    the float32 / float64 oracle."""
    sims = _sims()[:2]
    batch = SimulationBatch(sims)
    batch.advance(23, t0=[0, 0], graph=True, autotune=False)
    batch.advance(STEPS - 23, graph=True, autotune=False)
    torch.cuda.synchronize()
    for q, (arrays, objects, config) in enumerate(sims):
        sc32 = O.OracleScene(objects, arrays, config, torch.float32)
        sc64 = O.OracleScene(objects, arrays, config, torch.float64)
        r32, r64 = O.run(sc32, STEPS), O.run(sc64, STEPS)
        compare_states(f"batch_oracle_{q}", batch.arrays[q], r32, r64, 1e-4)
    batch.close()
