"""Spectrum-level helpers around the batched FDM solve.

* ``spectrum_inputs`` builds the per-energy inputs of one spectrum (the
  caller-side work of the reference's energy loop, source/fdm.f90:3493-3820,
  restricted to what ``mat`` consumes).
* ``absorption`` is the dipole K-edge absorption used to state errors: the
  p-projected absorber density -Im Tr Taull(L=1) (the reference multiplies
  Taull by radial integrals in tenseur_car, source/tensor.f90:15; those
  integrals do not change with the solver and are left out here).
* ``lorentzian_convolve`` restates the reference's convolution of a spectrum
  sampled on an energy grid by a Lorentzian of half width ``half_width``:
  each sample stands for the bin between the mid-points to its neighbours and
  the Lorentzian is integrated exactly over every bin,
  out(E_i) = -(1/pi) sum_j [atan((e1_j - E_i)/b) - atan((e2_j - E_i)/b)] x_j
  (source/convolution.f90:1612-1680).
"""
from __future__ import annotations

import math
from typing import List, Sequence, Tuple

import numpy as np

from . import cluster as CL


def spectrum_inputs(st: CL.Structure, energies: Sequence[float], functions: bool = True,
                    ispin: int = 1) -> List[Tuple[CL.EnergyInputs, CL.RowIndex]]:
    """Per-energy inputs and row numbering of a spectrum.  functions=False
    leaves phiato / Bessel / Neumann to the device (FdmSolver.set_radial)."""
    out = []
    rows = {}  # newind depends on the energy only through the l cut-offs: a few distinct numberings per spectrum
    for E in energies:
        ei = CL.energy_inputs(st, float(E), ispin=ispin, functions=functions)
        key = (tuple(int(x) for x in ei.nlmsa), int(ei.nlmso))
        if key not in rows:
            rows[key] = CL.newind(st, ei.nlmsa, ei.nlmso)
        out.append((ei, rows[key]))
    return out


def absorption(taull: np.ndarray) -> float:
    """-Im of the trace of the L = 1 block of Taull (harmonics 1..3, 0-based)."""
    return float(-np.imag(np.trace(taull[1:4, 1:4])))


def absorption_so(taull4: np.ndarray) -> float:
    """Spin-orbit counterpart of ``absorption``: -Im of the trace of the L = 1
    block summed over both spins, for Taull shaped (nlm, 2, nlm, 2) as
    ``FdmSolver.taull_c`` returns it."""
    return float(-np.imag(sum(np.trace(taull4[1:4, s, 1:4, s]) for s in range(taull4.shape[1]))))


def absorption_cotangent(taull: np.ndarray, g_sigma: float = 1.0) -> np.ndarray:
    """dL/d(Im Taull) for L = g_sigma * absorption(taull): -g_sigma on the L = 1 diagonal."""
    g = np.zeros(taull.shape, dtype=np.float64)
    for a in (1, 2, 3):
        g[a, a] = -g_sigma
    return g


def dipole_tensor(taull: np.ndarray, weight: float = 1.0) -> np.ndarray:
    """S(a, b) = -Im w (T(a,b) + T(b,a)) / 2 over the Cartesian components
    a, b = x, y, z of the L = 1 real harmonics (0-based harmonic 3, 1, 2)."""
    idx = [3, 1, 2]
    T = taull[np.ix_(idx, idx)]
    return -weight * 0.5 * np.imag(T + T.T)


def lorentzian_convolve(energies: np.ndarray, x: np.ndarray, half_width, width_per_input: bool = False) -> np.ndarray:
    """half_width: a number, or one width per energy (of the output energy,
    or of the input bin when width_per_input, the reference's Gamma_var)."""
    E = np.asarray(energies, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    n = len(E)
    if n < 2:
        return x.copy()
    bw = np.broadcast_to(np.asarray(half_width, dtype=np.float64), (n,))
    bw = np.where(bw >= 0.0, np.maximum(bw, 1e-8), bw)
    e1 = np.empty(n)
    e2 = np.empty(n)
    e1[0] = 1.5 * E[0] - 0.5 * E[1]
    e1[1:] = 0.5 * (E[1:] + E[:-1])
    e2[:-1] = 0.5 * (E[1:] + E[:-1])
    e2[-1] = 1.5 * E[-1] - 0.5 * E[-2]
    out = np.empty(n)
    for i in range(n):
        b = bw if width_per_input else bw[i]
        lor = np.arctan((e1 - E[i]) / b) - np.arctan((e2 - E[i]) / b)
        out[i] = -np.sum(lor * x) / math.pi
    return out


def convolved_relative_error(energies, taull_test, taull_ref, half_width: float = 0.78) -> float:
    """max_E |conv(sigma_test) - conv(sigma_ref)| / max_E |conv(sigma_ref)|."""
    a = np.array([absorption(t) for t in taull_test])
    r = np.array([absorption(t) for t in taull_ref])
    ca = lorentzian_convolve(energies, a, half_width)
    cr = lorentzian_convolve(energies, r, half_width)
    return float(np.abs(ca - cr).max() / max(np.abs(cr).max(), 1e-300))
