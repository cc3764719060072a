"""``run_fdtd``'s dispatch on the gradient configuration (CPU), replaying the reference's wrapper
tests (tests/unit/fdtd/test_wrapper.py:25-250) with the two drivers replaced by recorders:
no gradient config and ``"checkpointed"`` go to ``checkpointed_fdtd``, ``"reversible"`` to
``reversible_fdtd``; an unknown or missing method raises; a custom stopping condition with a
gradient config raises ``NotImplementedError``; ``show_progress`` (default True) and
``progress_callback`` are forwarded.
"""

import types

import pytest

import fdtdx_gb300 as fx
import fdtdx_gb300.adjoint as adjoint_mod
import fdtdx_gb300.fdtd as fdtd_mod


@pytest.fixture
def calls(monkeypatch):
    seen = []

    def checkpointed(arrays, objects, config, key=None, stopping_condition=None, show_progress=True,
                     progress_callback=None):
        seen.append(("checkpointed", stopping_condition, show_progress, progress_callback))
        return 0, arrays

    def reversible(arrays, objects, config, key=None, show_progress=True, progress_callback=None):
        seen.append(("reversible", None, show_progress, progress_callback))
        return 0, arrays

    monkeypatch.setattr(fdtd_mod, "checkpointed_fdtd", checkpointed)
    monkeypatch.setattr(adjoint_mod, "reversible_fdtd", reversible)
    return seen


def _config(gc):
    return types.SimpleNamespace(gradient_config=gc)


def _gc(method):
    return types.SimpleNamespace(method=method)


def test_dispatch(calls):
    fx.run_fdtd("arrays", "objects", _config(None))
    fx.run_fdtd("arrays", "objects", _config(_gc("reversible")))
    fx.run_fdtd("arrays", "objects", _config(_gc("checkpointed")))
    assert [c[0] for c in calls] == ["checkpointed", "reversible", "checkpointed"]
    for bad in ("bogus", None):
        with pytest.raises(Exception, match="Unknown gradient computation method"):
            fx.run_fdtd("arrays", "objects", _config(_gc(bad)))


def test_stopping_condition_with_gradient_config_raises(calls):
    with pytest.raises(NotImplementedError):
        fx.run_fdtd("arrays", "objects", _config(_gc("reversible")), stopping_condition=object())
    fx.run_fdtd("arrays", "objects", _config(_gc("reversible")), stopping_condition=None)
    cond = object()
    fx.run_fdtd("arrays", "objects", _config(None), stopping_condition=cond)
    assert calls[-1][0] == "checkpointed" and calls[-1][1] is cond


def test_progress_arguments_are_forwarded(calls):
    def cb(step, total):
        return None

    for gc in (None, _gc("reversible"), _gc("checkpointed")):
        fx.run_fdtd("arrays", "objects", _config(gc), show_progress=False, progress_callback=cb)
        assert calls[-1][2] is False and calls[-1][3] is cb
        fx.run_fdtd("arrays", "objects", _config(gc))
        assert calls[-1][2] is True and calls[-1][3] is None


def test_real_gradient_config_validation():
    with pytest.raises(Exception, match="Need Recorder"):
        fx.GradientConfig(method="reversible")
    with pytest.raises(Exception, match="Need Checkpoint Number"):
        fx.GradientConfig(method="checkpointed")
