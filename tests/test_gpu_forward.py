"""Forward-path parity of the GB300 kernels against the oracle (float32: asserted; float64: reported).

Tolerance: relative L2 <= 1e-4 on fields and detector states
against the float32 restatement of the reference after the full run.
"""

import math

import pytest
import torch

import fdtdx_gb300 as fx
from fdtdx_gb300 import scenes
from fdtdx_gb300.engine import Scene
from oracle import fdtd_oracle as O
from tests.helpers import compare_states, log_result, oracle_run, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _cfg(steps, dx=50e-9, record=False):
    dt = 0.99 / math.sqrt(3) * dx / 299792458.0
    gc = fx.GradientConfig(recorder=fx.Recorder()) if record else None
    return fx.SimulationConfig(time=steps * dt, grid=fx.UniformGrid(dx), gradient_config=gc)


def test_dipole_boxes_small():
    objects, arrays, _, cfg, _ = scenes.dipole_boxes(shape=(34, 30, 28), steps=160, n_boxes=6, pml=6)
    _, out = fx.run_fdtd(arrays, objects, cfg)
    torch.cuda.synchronize()
    _, r32 = oracle_run(objects, arrays, cfg, torch.float32)
    _, r64 = oracle_run(objects, arrays, cfg, torch.float64)
    compare_states("dipole_boxes_small", out, r32, r64, TOL)


def _seeded(arrays, objects, seed=1):
    g = torch.Generator(device="cpu").manual_seed(seed)
    E = torch.randn(arrays.fields.E.shape, generator=g) * 1e-3
    H = torch.randn(arrays.fields.H.shape, generator=g) * 1e-3
    return E, H


@pytest.mark.parametrize("boundary", ["periodic", "pec", "pmc", "pml"])
def test_boundaries_seeded_steps(boundary):
    """Seeded random fields, 12 steps, every boundary type (halo wrap, wall zeroing, CPML)."""
    cfg = _cfg(12)
    vol = fx.SimulationVolume(shape=(20, 18, 22))
    bc = fx.BoundaryConfig.from_uniform_bound(4 if boundary == "pml" else 1, boundary)
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
    objs.append(fx.UniformMaterialObject(name="blk", grid_slice_tuple=((5, 12), (6, 13), (4, 15)),
                                         material=fx.Material(permittivity=3.0)))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg)
    E, H = _seeded(arrays, objects)
    sc64 = O.OracleScene(objects, arrays, cfg, torch.float64)
    sc32 = O.OracleScene(objects, arrays, cfg, torch.float32)
    E = O._walls(sc64, E.double(), sc64.pec).float()
    H = O._walls(sc64, H.double(), sc64.pmc).float()
    arrays = arrays.aset("fields->E", E.cuda().contiguous()).aset("fields->H", H.cuda().contiguous())
    scene = Scene(objects, arrays, cfg)
    scene.forward(arrays, 0, 12, graph=False)
    torch.cuda.synchronize()
    refs = []
    for sc in (sc32, sc64):
        st = sc.init_state()
        st.E, st.H = E.to(sc.dtype), H.to(sc.dtype)
        refs.append(O.run(sc, 12, state=st))
    compare_states(f"boundary_{boundary}", arrays, refs[0], refs[1], TOL)
    for p in sc32.pmls:
        for q in range(2):
            assert rel_l2(arrays.fields.psi_E[p.name][q], refs[0].psi_E[p.name][q]) <= 5 * TOL
            assert rel_l2(arrays.fields.psi_H[p.name][q], refs[0].psi_H[p.name][q]) <= 5 * TOL


def test_materials_conductive_anisotropic_magnetic():
    """Diagonal anisotropic eps and mu, electric and magnetic conductivity, kappa != 1 CPML."""
    cfg = _cfg(60)
    vol = fx.SimulationVolume(shape=(24, 26, 22))
    bc = fx.BoundaryConfig.from_uniform_bound(5, "pml", kappa_end=2.0)
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
    objs.append(fx.UniformMaterialObject(
        name="aniso", grid_slice_tuple=((6, 14), (7, 18), (6, 16)),
        material=fx.Material(permittivity=(2.0, 5.0, 9.0), permeability=(1.5, 1.0, 2.0),
                             electric_conductivity=(3e4, 1e4, 0.0), magnetic_conductivity=(2e9, 0.0, 5e9))))
    objs.append(fx.PointDipoleSource(name="d", grid_slice_tuple=((12, 13), (12, 13), (11, 12)), polarization=0,
                                     wave_character=fx.WaveCharacter(wavelength=1.55e-6),
                                     temporal_profile=scenes.pulse_5fs()))
    objs.append(fx.PointDipoleSource(name="m", grid_slice_tuple=((9, 10), (14, 15), (9, 10)), polarization=1,
                                     source_type="magnetic", wave_character=fx.WaveCharacter(wavelength=1.55e-6),
                                     temporal_profile=scenes.pulse_5fs()))
    objs.append(fx.EnergyDetector(name="energy", grid_slice_tuple=((4, 20), (4, 22), (4, 18)), reduce_volume=True))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg)
    assert arrays.inv_permittivities.shape[0] == 3 and isinstance(arrays.inv_permeabilities, torch.Tensor)
    _, out = fx.run_fdtd(arrays, objects, cfg)
    torch.cuda.synchronize()
    _, r32 = oracle_run(objects, arrays, cfg, torch.float32)
    _, r64 = oracle_run(objects, arrays, cfg, torch.float64)
    compare_states("materials", out, r32, r64, TOL)


def test_plane_sources_and_all_detectors():
    """CW Gaussian plane source (TFSF), pulsed uniform plane source going '-', every detector kind."""
    cfg = _cfg(140, dx=25e-9)
    vol = fx.SimulationVolume(shape=(40, 36, 32), material=fx.Material(permittivity=2.1025))
    objs = [vol] + list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(6), vol).values())
    objs.append(fx.UniformMaterialObject(name="wg", grid_slice_tuple=((0, 40), (14, 22), (13, 19)),
                                         material=fx.Material(permittivity=12.11)))
    wc = fx.WaveCharacter(wavelength=1.55e-6)
    objs.append(fx.GaussianPlaneSource(name="g", grid_slice_tuple=((9, 10), (8, 28), (8, 24)), direction="+",
                                       radius=8 * 25e-9, fixed_E_polarization_vector=(0, 1, 0), wave_character=wc))
    objs.append(fx.UniformPlaneSource(name="u", grid_slice_tuple=((8, 32), (8, 28), (24, 25)), direction="-",
                                      fixed_E_polarization_vector=(1, 0, 0), wave_character=wc,
                                      temporal_profile=scenes.pulse_5fs(), static_amplitude_factor=0.5,
                                      switch=fx.OnOffSwitch(start_time=20 * cfg.time_step_duration)))
    R = ((12, 30), (10, 26), (10, 22))
    objs += [
        fx.PhasorDetector(name="ph_all", grid_slice_tuple=R, wave_characters=(wc, fx.WaveCharacter(wavelength=1.3e-6))),
        fx.PhasorDetector(name="ph_red", grid_slice_tuple=R, wave_characters=(wc,), components=("Ey", "Hz"),
                          reduce_volume=True, scaling_mode="pulse", switch=fx.OnOffSwitch(interval=2)),
        fx.FieldDetector(name="f_plane", grid_slice_tuple=((0, 40), (0, 36), (16, 17)), components=("Ex", "Hy")),
        fx.FieldDetector(name="f_red", grid_slice_tuple=R, reduce_volume=True),
        fx.FieldDetector(name="f_raw", grid_slice_tuple=((20, 24), (20, 24), (0, 4)), exact_interpolation=False),
        fx.PoyntingFluxDetector(name="flux", grid_slice_tuple=((30, 31), (10, 26), (10, 22)), direction="+"),
        fx.PoyntingFluxDetector(name="flux_all", grid_slice_tuple=((12, 13), (10, 26), (10, 22)), direction="-",
                                keep_all_components=True, reduce_volume=False),
        fx.EnergyDetector(name="en", grid_slice_tuple=R),
        fx.PhasorPoyntingFluxDetector(name="pflux", grid_slice_tuple=((30, 31), (10, 26), (10, 22)), direction="+",
                                      wave_characters=(wc,)),
    ]
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg)
    _, out = fx.run_fdtd(arrays, objects, cfg)
    torch.cuda.synchronize()
    _, r32 = oracle_run(objects, arrays, cfg, torch.float32)
    _, r64 = oracle_run(objects, arrays, cfg, torch.float64)
    compare_states("plane_sources_detectors", out, r32, r64, TOL)
    pf = objects["pflux"]
    g = pf.compute_poynting_flux(out.detector_states["pflux"], cfg.grid.spacing)
    r = pf.compute_poynting_flux({"phasor": r32.det["pflux"]["phasor"]}, cfg.grid.spacing)
    assert rel_l2(g, r) <= TOL


def test_graph_and_direct_paths_agree():
    objects, arrays, _, cfg, _ = scenes.coupler(shape=(60, 60, 40), steps=100, scale=0.2, pml=6)
    a = arrays.reset()
    b = arrays.reset()
    s = Scene(objects, a, cfg)
    s.forward(a, 0, 100, graph=True)
    s.forward(b, 0, 100, graph=False)
    torch.cuda.synchronize()
    assert torch.equal(a.fields.E, b.fields.E) and torch.equal(a.fields.H, b.fields.H)
    for k in a.detector_states:
        for kk in a.detector_states[k]:
            assert torch.equal(a.detector_states[k][kk], b.detector_states[k][kk])


def test_chunked_run_equals_single_run():
    """Stopping and resuming at arbitrary step boundaries (plan tables indexed by absolute time)."""
    objects, arrays, _, cfg, _ = scenes.dipole_boxes(shape=(24, 24, 24), steps=50, n_boxes=4, pml=5)
    a, b = arrays.reset(), arrays.reset()
    s = Scene(objects, a, cfg)
    s.forward(a, 0, 50)
    for t0, n in ((0, 7), (7, 20), (27, 23)):
        s.forward(b, t0, n)
    torch.cuda.synchronize()
    assert torch.equal(a.fields.E, b.fields.E)
    assert torch.equal(a.detector_states["ez_plane"]["fields"], b.detector_states["ez_plane"]["fields"])


def test_reverse_reconstructs_with_recording():
    """Forward N steps recording the PML interfaces, reverse N steps: the interior returns to the
    initial state (fdtdx/fdtd/backward.py semantics; tests/simulation/fdtd/test_time_reversal.py)."""
    objects, _, _, cfg, _ = scenes.dipole_boxes(shape=(30, 28, 26), steps=80, n_boxes=4, pml=5)
    cfg = fx.SimulationConfig(time=cfg.time, grid=cfg.grid, gradient_config=fx.GradientConfig(recorder=fx.Recorder()))
    from fdtdx_gb300.initialization import init_arrays

    arrays = init_arrays(objects, cfg)
    a = arrays.reset()
    E0, H0 = _seeded(a, objects, seed=3)
    a = a.aset("fields->E", E0.cuda()).aset("fields->H", H0.cuda())
    s = Scene(objects, a, cfg, record_interfaces=True)
    s.forward(a, 0, 80)
    s.reverse(a, 80, 80)
    torch.cuda.synchronize()
    inner = (slice(None), slice(6, -6), slice(6, -6), slice(6, -6))
    eE = rel_l2(a.fields.E[inner], E0[inner])
    eH = rel_l2(a.fields.H[inner], H0[inner])
    log_result("reverse_roundtrip", rel_l2_E=eE, rel_l2_H=eH)
    assert eE < 1e-3 and eH < 1e-3
    # the oracle's reverse from the same final state agrees with the kernel's reverse
    sc = O.OracleScene(objects, a, cfg, torch.float64)
    st = sc.init_state()
    st.E, st.H = E0.double(), H0.double()
    st = O.run(sc, 80, record_boundaries=True, state=st)
    for _ in range(80):
        st = O.backward(sc, st)
    assert rel_l2(a.fields.E[inner], st.E[inner]) < 1e-3


@pytest.mark.parametrize("shape,steps", [((100, 100, 100), 1000)])
def test_dipole_boxes_full_size(shape, steps):
    """The 100^3, 1000-step dipole-in-boxes workload, full size, against the float32 oracle."""
    objects, arrays, _, cfg, _ = scenes.dipole_boxes(shape=shape, steps=steps)
    _, out = fx.run_fdtd(arrays, objects, cfg)
    torch.cuda.synchronize()
    torch.set_num_threads(max(1, torch.get_num_threads()))
    _, r32 = oracle_run(objects, arrays, cfg, torch.float32)
    _, r64 = oracle_run(objects, arrays, cfg, torch.float64)
    compare_states("dipole_boxes_100_1000", out, r32, r64, TOL)


@pytest.mark.parametrize("nz", [24, 21])
def test_vec_and_chunk_variants_agree(nz):
    """Every (vec, chunk) launch shape of the update kernels gives bit-identical results."""
    from fdtdx_gb300 import _native as NATIVE

    objects, arrays, _, cfg, _ = scenes.coupler(shape=(36, 32, nz), steps=40, scale=0.15, pml=5)
    ref = None
    vecs = [v for v in (1, 2, 4) if nz % v == 0]
    for vec in vecs:
        for chunk in (1, 5, 36):
            a = arrays.reset()
            s = Scene(objects, a, cfg)
            NATIVE.check(NATIVE.load().fdtd_plan_tune(s.plan, chunk, vec), s.plan, "tune")
            s.forward(a, 0, 40)
            torch.cuda.synchronize()
            got = [a.fields.E.clone(), a.fields.H.clone()] + [v.clone() for st in a.detector_states.values()
                                                               for v in st.values()]
            s.close()
            if ref is None:
                ref = got
            else:
                for x, y in zip(got, ref):
                    assert torch.equal(x, y), (vec, chunk)


def test_shell_tiling_variants_agree():
    """CPML shell launch shapes (fdtd_plan_tune_shell): x chunks and one or two z cells per
    thread give bit-identical results (same per-cell arithmetic through the per-axis slab
    table); four z cells per thread take the generic six-slab form, whose CPML terms are
    summed in slab order instead of axis order (agreement to rounding)."""
    objects, arrays, _, cfg, _ = scenes.coupler(shape=(36, 32, 40), steps=40, scale=0.15, pml=5)
    outs = {}
    for chunk, vec in ((4, 1), (1, 1), (9, 2), (3, 4)):
        a = arrays.reset()
        s = Scene(objects, a, cfg)
        s.tune_shell(chunk, vec)
        s.forward(a, 0, 40)
        torch.cuda.synchronize()
        outs[(chunk, vec)] = [a.fields.E.clone(), a.fields.H.clone()] + [
            v.clone() for st in a.detector_states.values() for v in st.values()]
        s.close()
    ref = outs[(4, 1)]
    for key in ((1, 1), (9, 2)):
        for x, y in zip(outs[key], ref):
            assert torch.equal(x, y), key
    for x, y in zip(outs[(3, 4)], ref):
        assert rel_l2(x, y) < 1e-6


@pytest.mark.parametrize("tile", [(0, 0, 0, 0), (16, 8, 2, 3), (24, 4, 3, 7), (64, 8, 6, 0)])
def test_tma_kernels_match_register_kernels(tile):
    """The TMA-pipelined half-steps agree with the register-queue half-steps (every tile shape,
    partial tiles in y and z, chunked x, CPML, conductivity, fused detectors): the TMA core with
    the register-queue shell (slab mode 0, rounding-close) and the split form (mode 3: the plain
    TMA kernels over the whole grid, then the slab corrections; a rounding apart per step, which
    psi integrates: measured 1.2e-6 after 50 steps)."""
    tz, ty, ns, chunk = tile
    cfg = _cfg(50)
    vol = fx.SimulationVolume(shape=(30, 27, 44))
    objs = [vol] + list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(5), vol).values())
    objs.append(fx.UniformMaterialObject(name="blk", grid_slice_tuple=((8, 20), (6, 20), (10, 30)),
                                         material=fx.Material(permittivity=(4.0, 3.0, 5.0), electric_conductivity=1e4,
                                                              magnetic_conductivity=1e9, permeability=1.5)))
    objs.append(fx.PointDipoleSource(name="d", grid_slice_tuple=((15, 16), (13, 14), (22, 23)), polarization=1,
                                     wave_character=fx.WaveCharacter(wavelength=1.55e-6),
                                     temporal_profile=scenes.pulse_5fs()))
    objs.append(fx.PhasorDetector(name="ph", grid_slice_tuple=((0, 30), (3, 25), (0, 44)),
                                  wave_characters=(fx.WaveCharacter(wavelength=1.55e-6),), components=("Ex", "Ey", "Ez")))
    objs.append(fx.FieldDetector(name="ez", grid_slice_tuple=((0, 30), (0, 27), (20, 21)), components=("Ez", "Ey")))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg)
    outs = {}
    for run in ("register", 0, 3, 4, 5):
        a = arrays.reset()
        s = Scene(objects, a, cfg)
        if run == "register":
            s.tune_tma(False)
        else:
            s.tune_tma(True, tz, ty, ns, chunk)
            s.tune_shell_tma(run)
            assert s.uses_tma and s.shell_tma == run
        s.forward(a, 0, 50)
        s.status()
        torch.cuda.synchronize()
        outs[run] = a
        s.close()
    ref = outs["register"]
    for run, tol, tol_psi in ((0, 1e-6, 1e-6), (3, 2e-6, 5e-6), (4, 2e-6, 5e-6), (5, 2e-6, 5e-6)):
        got = outs[run]
        for k in ("E", "H"):
            assert rel_l2(getattr(got.fields, k), getattr(ref.fields, k)) < tol, (run, k)
        for dn in ("ph", "ez"):
            for kk, v in got.detector_states[dn].items():
                assert rel_l2(v, ref.detector_states[dn][kk]) < tol, (run, dn)
        for n in got.fields.psi_E:
            for q in range(2):
                assert rel_l2(got.fields.psi_E[n][q], ref.fields.psi_E[n][q]) < tol_psi, (run, n)
                assert rel_l2(got.fields.psi_H[n][q], ref.fields.psi_H[n][q]) < tol_psi, (run, n)


def test_plans_of_different_tile_memory_coexist():
    """A plan built after another must not break it: the TMA kernels' shared-memory limit is a
    process-wide function attribute (an anisotropic plan stages three material planes, an
    isotropic one fewer)."""
    o1, a1, _, c1, _ = scenes.serving_job(shape=(40, 36, 32), steps=30, seed=1, anisotropic=True, device="cuda")
    o2, a2, _, c2, _ = scenes.serving_job(shape=(40, 36, 32), steps=30, seed=2, anisotropic=False, device="cuda")
    s1 = Scene(o1, a1.reset(), c1)
    w1 = a1.reset()
    s1.plan  # build the large-tile plan first
    s2 = Scene(o2, a2.reset(), c2)
    w2 = a2.reset()
    s2.plan
    s1.forward(w1, 0, 30)
    s2.forward(w2, 0, 30)
    torch.cuda.synchronize()
    assert torch.isfinite(w1.fields.E).all() and torch.isfinite(w2.fields.E).all()
    assert s1.uses_tma


@pytest.mark.parametrize("mode,tz,chunk", [(1, 0, 0), (2, 0, 0), (2, 20, 3), (3, 0, 0), (3, 20, 5), (4, 0, 0), (4, 20, 3), (5, 0, 0)])
def test_shell_tma_matches_register_shell(mode, tz, chunk):
    """The CPML slab cells on the TMA kernels with in-tile slab terms (mode 1: the x and y
    slabs, the core widened over them; mode 2: the whole grid in one launch), or split (mode 3:
    the plain TMA kernels over the whole grid, then the slab cells' CPML corrections per axis;
    mode 4: the same with the z slabs' terms inside the tiles; mode 5: mode 4 for E, 3 for H)
    against the register-queue shell kernel: forward steps with kappa != 1, a conductor and a
    dipole inside the slabs and a fused full-volume phasor, then time-reversed steps with the
    recorded interfaces (psi frozen)."""
    cfg = _cfg(60, record=True)
    vol = fx.SimulationVolume(shape=(30, 27, 44))
    bc = fx.BoundaryConfig.from_uniform_bound(6, "pml", kappa_end=1.8)
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
    objs.append(fx.UniformMaterialObject(name="blk", grid_slice_tuple=((3, 22), (2, 20), (2, 40)),
                                         material=fx.Material(permittivity=(4.0, 3.0, 5.0), electric_conductivity=1e4)))
    objs.append(fx.PointDipoleSource(name="d", grid_slice_tuple=((15, 16), (13, 14), (5, 6)), polarization=1,
                                     wave_character=fx.WaveCharacter(wavelength=1.55e-6),
                                     temporal_profile=scenes.pulse_5fs()))
    objs.append(fx.PointDipoleSource(name="d2", grid_slice_tuple=((2, 3), (3, 4), (20, 21)), polarization=2,
                                     wave_character=fx.WaveCharacter(wavelength=1.55e-6),
                                     temporal_profile=scenes.pulse_5fs()))
    objs.append(fx.PhasorDetector(name="ph", grid_slice_tuple=((0, 30), (0, 27), (0, 44)),
                                  wave_characters=(fx.WaveCharacter(wavelength=1.55e-6),), components=("Ex", "Ey", "Ez")))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg)
    assert arrays.recording_state is not None
    outs = []
    for m in (mode, 0):
        a = arrays.reset()
        s = Scene(objects, a, cfg, record_interfaces=True)
        s.tune_shell_tma(m, tz if m >= 2 else 0, chunk if m else 0)
        assert s.uses_tma and s.shell_tma == m
        s.forward(a, 0, 60)
        s.status()
        torch.cuda.synchronize()
        fwd = [a.fields.E.clone(), a.fields.H.clone(), a.detector_states["ph"]["phasor"].clone()]
        fwd += [t.clone() for n in a.fields.psi_E for t in (*a.fields.psi_E[n], *a.fields.psi_H[n])]
        s.reverse(a, 60, 30)
        s.status()
        torch.cuda.synchronize()
        outs.append((fwd, [a.fields.E.clone(), a.fields.H.clone()]))
        s.close()
    # modes 1 and 2 add the slab terms in the shell kernel's order (bitwise-close); modes 3-5
    # add them after the plain update, a rounding apart per step: after 60 steps E, H and the
    # phasor within 4e-7 and psi within 1e-6, except the psi of the two slabs holding the
    # second dipole (1.4e-5 / 7.6e-6: their small norm is dominated by the source cell's
    # neighbourhood); the 30 reverse steps (split too) amplify the difference inside the CPML,
    # where a reverse step is no exact time reversal
    n3 = 3  # E, H, phasor
    tol_f, tol_p, tol_r = (2e-6, 5e-5, 1e-4) if mode >= 3 else (1e-6, 1e-6, 1e-6)
    for q, (x, y) in enumerate(zip(outs[0][0], outs[1][0])):
        assert rel_l2(x, y) < (tol_f if q < n3 else tol_p), q
    for x, y in zip(outs[0][1], outs[1][1]):
        assert rel_l2(x, y) < tol_r


def test_split_halfsteps_with_conductor_faces_against_oracle():
    """The split CPML half-steps (slab modes 3 and 5) on a scene whose min-z and max-x faces are
    PEC and whose min-y face is PMC, CPML on the others (the corrections skip the components
    a conductor face zeroes), with a lossy anisotropic block reaching into the slabs: against
    the register-queue shell (mode 0) and the float32 / float64 oracle, forward steps and
    time-reversed steps."""
    cfg = _cfg(50, record=True)
    vol = fx.SimulationVolume(shape=(30, 27, 44))
    bc = fx.BoundaryConfig.from_uniform_bound(6, "pml", override_types={"min_z": "pec", "max_x": "pec", "min_y": "pmc"})
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
    objs.append(fx.UniformMaterialObject(name="blk", grid_slice_tuple=((2, 25), (1, 22), (0, 40)),
                                         material=fx.Material(permittivity=(4.0, 3.0, 5.0), electric_conductivity=1e4)))
    objs.append(fx.PointDipoleSource(name="d", grid_slice_tuple=((15, 16), (13, 14), (30, 31)), polarization=0,
                                     wave_character=fx.WaveCharacter(wavelength=1.55e-6),
                                     temporal_profile=scenes.pulse_5fs()))
    objs.append(fx.PhasorDetector(name="ph", grid_slice_tuple=((0, 30), (0, 27), (0, 44)),
                                  wave_characters=(fx.WaveCharacter(wavelength=1.55e-6),), components=("Ex", "Ey", "Ez")))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg)
    outs = {}
    for m in (0, 3, 5):
        a = arrays.reset()
        s = Scene(objects, a, cfg, record_interfaces=True)
        s.tune_shell_tma(m)
        assert s.uses_tma and s.shell_tma == m
        s.forward(a, 0, 50)
        s.status()
        torch.cuda.synchronize()
        outs[m] = ([a.fields.E.clone(), a.fields.H.clone(), a.detector_states["ph"]["phasor"].clone()], None)
        if m == 5:
            _, r32 = oracle_run(objects, arrays, cfg, torch.float32, 50)
            _, r64 = oracle_run(objects, arrays, cfg, torch.float64, 50)
            compare_states("split_conductor_faces", a, r32, r64, 1e-4)
        s.reverse(a, 50, 25)
        s.status()
        torch.cuda.synchronize()
        outs[m] = (outs[m][0], [a.fields.E.clone(), a.fields.H.clone()])
        s.close()
    for m in (3, 5):
        for q, (x, y) in enumerate(zip(outs[m][0], outs[0][0])):
            assert rel_l2(x, y) < 2e-6, (m, q)
        for x, y in zip(outs[m][1], outs[0][1]):
            assert rel_l2(x, y) < 1e-4, m
