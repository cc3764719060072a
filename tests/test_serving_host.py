"""Host logic of the serving loop (no GPU): admission by footprint and slots, bounded
backfill, forward chunks that never pass a job's end, phase changes, memory release."""

from fdtdx_gb300.serving import Job, Scheduler, latency_stats


def _job(i, fp, steps=100, kind="forward", arrival=0.0):
    j = Job(build=None, kind=kind, arrival=arrival)
    j.id, j.footprint, j.steps, j.n_cells = i, fp, steps, 1000
    return j


def test_admission_respects_budget_and_slots():
    s = Scheduler(budget_bytes=100, max_slots=2)
    for i, fp in enumerate([40, 40, 10]):
        s.arrive(_job(i, fp))
    got = s.admit(0.0)
    assert [j.id for j in got] == [0, 1] and s.used == 80  # slot limit stops job 2
    s.complete(got[0], 1.0)
    assert s.used == 40
    got = s.admit(1.0)
    assert [j.id for j in got] == [2] and s.used == 50


def test_backfill_is_bounded():
    s = Scheduler(budget_bytes=100, max_slots=8, max_bypass=1)
    s.arrive(_job(9, 50))
    assert [j.id for j in s.admit(0.0)] == [9]
    big = _job(0, 90)
    s.arrive(big)
    s.arrive(_job(1, 10))
    assert [j.id for j in s.admit(0.0)] == [1]  # big does not fit (50 + 10 + 90): job 1 passes it once
    s.arrive(_job(2, 10))
    assert [j.id for j in s.admit(0.0)] == []  # big was passed max_bypass times: it is reserved
    assert big.phase == "queued"
    for j in list(s.active):
        s.complete(j, 1.0)
    assert [j.id for j in s.admit(1.0)] == [0, 2]


def test_forward_chunk_and_phases():
    s = Scheduler(budget_bytes=10**6, max_slots=8)
    a, b = _job(0, 10, steps=30), _job(1, 10, steps=75, kind="gradient")
    s.arrive(a)
    s.arrive(b)
    s.admit(0.0)
    assert s.forward_chunk(50) == 30  # never past a's end
    for j in s.forward_jobs():
        s.advanced(j, 30)
    assert s.forward_finished(a) and not s.forward_finished(b)
    s.complete(a, 2.0)
    assert s.forward_chunk(100) == 45
    s.advanced(b, 45)
    s.start_adjoint(b)
    assert b.phase == "adjoint" and b.t_adj == 76 and s.forward_jobs() == [] and s.adjoint_jobs() == [b]
    s.complete(b, 3.0)
    assert s.idle() and s.used == 0


def test_job_larger_than_budget_is_refused():
    s = Scheduler(budget_bytes=10)
    try:
        s.arrive(_job(0, 11))
    except ValueError:
        return
    raise AssertionError("oversized job accepted")


def test_latency_percentiles():
    jobs = []
    for i, lat in enumerate([1.0, 2.0, 3.0, 4.0, 100.0]):
        j = _job(i, 1, arrival=0.0)
        j.t_done = lat
        jobs.append(j)
    st = latency_stats(jobs)
    assert st["p50_s"] == 3.0 and st["p99_s"] == 100.0 and abs(st["mean_s"] - 22.0) < 1e-12


def test_footprint_counts_gradient_buffers():
    """fdtd_footprint_bytes (host only): a gradient job needs more than its forward run, and a
    magnetic-array scene's gradient footprint covers the permeability array and its gradient
    (4 n_mu bytes per cell each) beyond the same scene with a scalar permeability."""
    import ctypes as C

    import fdtdx_gb300 as fx
    from fdtdx_gb300 import _native as N
    from fdtdx_gb300.build import build
    from fdtdx_gb300.engine import Scene

    build()  # no-op when the library is up to date

    def scene(permeability):
        cfg = fx.SimulationConfig(time=20 * 5e-17, grid=fx.UniformGrid(50e-9),
                                  gradient_config=fx.GradientConfig(recorder=fx.Recorder()))
        vol = fx.SimulationVolume(shape=(24, 20, 16))
        objs = [vol] + list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(4), vol).values())
        objs.append(fx.UniformMaterialObject(name="blk", grid_slice_tuple=((6, 12), (6, 12), (6, 10)),
                                             material=fx.Material(permittivity=3.0, permeability=permeability)))
        return fx.place_objects(objs, cfg, device="cpu")

    lib = N.load()
    sizes = {}
    for mu in (1.0, (1.5, 1.2, 2.0)):
        objects, arrays, _, cfg, _ = scene(mu)
        for rec in (False, True):
            s = Scene(objects, arrays, cfg, record_interfaces=rec)
            sizes[(mu, rec)] = lib.fdtd_footprint_bytes(C.byref(s.desc))
    n = 24 * 20 * 16
    for mu in (1.0, (1.5, 1.2, 2.0)):
        assert sizes[(mu, True)] > sizes[(mu, False)] > 0
    assert sizes[((1.5, 1.2, 2.0), True)] - sizes[(1.0, True)] >= 2 * 4 * 3 * n


def test_withdraw_and_release_phases():
    """A queued job is withdrawn without touching the budget; an active one leaves as
    "cancelled" or "failed" and frees its footprint."""
    s = Scheduler(budget_bytes=100, max_slots=8)
    a, b, c = _job(0, 60), _job(1, 30), _job(2, 50)
    for j in (a, b, c):
        s.arrive(j)
    assert [j.id for j in s.admit(0.0)] == [0, 1]
    assert s.withdraw(c, 0.5) and c.phase == "cancelled" and s.used == 90
    assert not s.withdraw(c, 0.6)  # no longer queued
    s.complete(a, 1.0, "cancelled")
    s.complete(b, 1.0, "failed")
    assert s.used == 0 and s.idle()
    assert [j.phase for j in s.done] == ["cancelled", "cancelled", "failed"]
