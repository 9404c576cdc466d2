"""Dipole absorption, its Cartesian tensor and the Lorentzian convolution on
the device (fdmgpu_batch_xanes) against the host restatement in
fdmnes_gb300/xanes.py (tens_ab's E1E1 K-edge channel, source/tensor.f90:1218-1264;
the convolution of source/convolution.f90:1612-1680).  Both are FP64 on the
same Taull; the bar is 1e-13 relative (max |diff| / max |ref|): summation
order and the device's atan differ from numpy's in the last bits."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch():
    from fdmnes_gb300 import build, cluster as CL, xanes
    build.build()
    from fdmnes_gb300.solver import FdmSolver
    st = CL.small_cu_structure()
    E = np.linspace(-5.0, 35.0, 21)
    items = xanes.spectrum_inputs(st, E)
    sv = FdmSolver(st)
    T, _ = sv.spectrum(items, "fp64")
    yield sv, E, T
    sv.close()


def test_sigma_tensor_and_convolution_match_host(batch):
    from fdmnes_gb300 import xanes
    sv, E, T = batch
    sig, conv, ten = sv.xanes(E, 0.78, tensor=True)
    ref = np.array([xanes.absorption(t) for t in T])
    assert rel(sig, ref) < 1e-13
    assert rel(ten, np.array([xanes.dipole_tensor(t) for t in T])) < 1e-13
    assert np.allclose(np.trace(ten, axis1=1, axis2=2), sig, rtol=1e-13, atol=0)
    assert rel(conv, xanes.lorentzian_convolve(E, ref, 0.78)) < 1e-13


def test_energy_dependent_widths_and_weights(batch):
    from fdmnes_gb300 import xanes
    sv, E, T = batch
    width = 0.2 + 0.05 * (E - E[0])                 # broadening growing with energy
    w = 1.0 + 0.01 * np.arange(len(E))              # |radial integral|^2 per energy
    ref = np.array([wk * xanes.absorption(t) for wk, t in zip(w, T)])
    for per_input in (False, True):
        sig, conv = sv.xanes(E, width, width_per_input=per_input, weight=w)
        assert rel(sig, ref) < 1e-13
        assert rel(conv, xanes.lorentzian_convolve(E, ref, width, width_per_input=per_input)) < 1e-13


def test_rejects_unordered_energies(batch):
    from fdmnes_gb300.solver import FdmError
    sv, E, T = batch
    with pytest.raises(FdmError):
        sv.xanes(E[::-1], 0.78)
