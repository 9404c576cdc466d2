"""Adjoint (vector-Jacobian product) of the batched FP64 spectrum.

L = sum_E w_E sigma(E), sigma = -Im Tr Taull(L=1).  fdmgpu_batch_vjp returns
dL/dVr at every grid point; it is checked against central finite differences
of the same FP64 GPU spectrum, Vr(i) +- h with h = 1e-4 Ry, on the small Cu
cluster.  Bar: relative difference <= 1e-5.  The FD quotient's own rounding
error is about 1e-13 |L| / h, i.e. ~6e-6 absolute for |L| ~ 6e3 at h = 1e-4
Ry, against derivatives of 2..7; measured differences are 1e-7..3e-6.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H = 1e-4
TOL = 1e-5


@pytest.fixture(scope="module")
def setup():
    from fdmnes_gb300 import build, cluster as CL, xanes
    from fdmnes_gb300.solver import FdmSolver
    build.build()
    st = CL.small_cu_structure()
    sv = FdmSolver(st)
    items = []
    for E in (3.0, 12.0, 27.0):
        ei = CL.energy_inputs(st, E)
        items.append((ei, CL.newind(st, ei.nlmsa, ei.nlmso)))
    w = np.array([1.0, -0.7, 0.4])

    def loss():
        T, _ = sv.spectrum(items, "fp64")
        return sum(wk * xanes.absorption(t) for wk, t in zip(w, T)), T

    yield st, sv, items, w, loss
    sv.close()


def test_vjp_matches_central_differences(setup):
    from fdmnes_gb300 import xanes
    st, sv, items, w, loss = setup
    L0, T = loss()
    grad, ms = sv.vjp([xanes.absorption_cotangent(t, wk) for t, wk in zip(T, w)])
    g = st.grid
    inter = np.nonzero(g.numia[:g.npoint] == 0)[0]
    atoms = np.nonzero(g.numia[:g.npoint] > 0)[0]
    assert np.all(grad[atoms, 0] == 0.0)
    gmax = np.abs(grad[inter, 0]).max()
    assert gmax > 0
    order = np.argsort(-np.abs(grad[inter, 0]))
    picks = [inter[order[k]] for k in (0, 3, 10, 40)]
    for i in picks:
        v0 = st.Vr[i, 0]
        st.Vr[i, 0] = v0 + H
        Lp, _ = loss()
        st.Vr[i, 0] = v0 - H
        Lm, _ = loss()
        st.Vr[i, 0] = v0
        fd = (Lp - Lm) / (2 * H)
        assert abs(grad[i, 0] - fd) <= TOL * abs(fd) + 1e-3 * TOL * gmax, (i, grad[i, 0], fd)


def test_vjp_is_linear_in_the_cotangent(setup):
    from fdmnes_gb300 import xanes
    st, sv, items, w, loss = setup
    _, T = loss()
    g1, _ = sv.vjp([xanes.absorption_cotangent(t, 1.0) for t in T])
    g2, _ = sv.vjp([xanes.absorption_cotangent(t, wk) for t, wk in zip(T, w)])
    parts = []
    for k in range(len(T)):
        gk = [xanes.absorption_cotangent(t, 1.0 if j == k else 0.0) for j, t in enumerate(T)]
        parts.append(sv.vjp(gk)[0])
    assert np.allclose(sum(parts), g1, rtol=1e-12, atol=1e-12 * np.abs(g1).max())
    assert np.allclose(sum(wk * p for wk, p in zip(w, parts)), g2, rtol=1e-12, atol=1e-12 * np.abs(g2).max())


def test_vjp_needs_fp64_factors(setup):
    from fdmnes_gb300 import xanes
    from fdmnes_gb300.solver import FdmError
    st, sv, items, w, loss = setup
    T, _ = sv.spectrum(items, "mixed")
    with pytest.raises(FdmError):
        sv.vjp([xanes.absorption_cotangent(t) for t in T])
