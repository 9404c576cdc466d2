"""Host logic of the shell fit's gradient (fdmnes_gb300/fit.py), on a fake
solver: the one-sided difference where the grid structure changes within h,
and the FP64 re-run of a step whose mixed batch has no adjoint."""
import numpy as np
import pytest


class _FakeSolver:
    """theta is the 'structure'; the adjoint dot product at theta' is theta'^2,
    so the central difference is 2 theta and the one-sided ones 2 theta -+ h."""
    refuse_above = None      # update_grid_values refuses structures above this
    refuse_far = None        # ... or farther than this from the handle's own
    mixed_vjp_fails = False
    calls = []

    def __init__(self, st):
        self.st = st
        self.cur = st
        self.prec = None

    def set_radial(self):
        pass

    def set_tolerance(self, *a):
        pass

    def spectrum(self, items, precision):
        self.prec = precision
        _FakeSolver.calls.append(precision)
        return [np.array([[self.st]])], {}

    def vjp(self, g):
        from fdmnes_gb300.solver import FdmError
        if self.prec == "mixed" and _FakeSolver.mixed_vjp_fails:
            raise FdmError(2, "vjp of a mixed batch with an energy re-solved in FP64")

    def update_grid_values(self, st):
        from fdmnes_gb300.solver import FdmError
        if ((_FakeSolver.refuse_above is not None and st > _FakeSolver.refuse_above) or
                (_FakeSolver.refuse_far is not None and abs(st - self.st) > _FakeSolver.refuse_far)):
            raise FdmError(1, "the grid's integer structure changed")
        self.cur = st

    def adjoint_dot(self, items):
        return np.array([self.cur ** 2])

    def close(self):
        pass


@pytest.fixture
def fake(monkeypatch):
    from fdmnes_gb300 import fit, xanes
    monkeypatch.setattr(fit, "FdmSolver", _FakeSolver)
    monkeypatch.setattr(xanes, "spectrum_inputs", lambda st, E, functions=False: [st])
    monkeypatch.setattr(xanes, "absorption", lambda t: float(t[0][0]))
    monkeypatch.setattr(xanes, "absorption_cotangent", lambda t, g: g)
    _FakeSolver.refuse_above = None
    _FakeSolver.refuse_far = None
    _FakeSolver.mixed_vjp_fails = False
    _FakeSolver.calls = []
    return fit


def test_central_difference_when_the_structure_holds(fake):
    L, g = fake.loss_grad(lambda th: th, 0.3, [1.0], np.array([0.0]), h=1e-4)
    assert L == pytest.approx(0.09)
    assert g == pytest.approx(0.6, abs=1e-9)


def test_one_sided_difference_where_the_structure_changes(fake):
    _FakeSolver.refuse_above = 0.30005       # theta + h changes the structure
    _, g = fake.loss_grad(lambda th: th, 0.3, [1.0], np.array([0.0]), h=1e-4)
    assert g == pytest.approx(2 * 0.3 - 1e-4, abs=1e-9)


def test_structure_changing_on_both_sides_is_an_error(fake):
    from fdmnes_gb300.solver import FdmError
    _FakeSolver.refuse_far = 0.5e-4          # theta +- h both change the structure
    with pytest.raises(FdmError, match="both sides"):
        fake.loss_grad(lambda th: th, 0.3, [1.0], np.array([0.0]), h=1e-4)


def test_step_without_mixed_adjoint_runs_in_fp64(fake):
    _FakeSolver.mixed_vjp_fails = True
    L, g = fake.loss_grad(lambda th: th, 0.3, [1.0], np.array([0.0]), h=1e-4, precision="mixed")
    assert _FakeSolver.calls == ["mixed", "fp64"]
    assert g == pytest.approx(0.6, abs=1e-9)
