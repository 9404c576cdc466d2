"""Gradients of a spectrum loss through the adjoint of the batched solve.

L = sum_E w_E sigma(E) with sigma the dipole absorption -Im Tr Taull(L=1)
(``xanes.absorption``).  Two parameter families:

* the grid potential Vr: ``FdmSolver.vjp`` (exact reverse mode on the device);
* a shell distance (the radius of one coordination shell around the
  absorber): dL/dtheta = Lambda^T (dB/dtheta - dA/dtheta X), with
  Lambda, X of the forward solve and the derivative of the assembled matrix
  taken by central differences of the assembly only
  (``fdmgpu_batch_adjoint_dot`` at theta +- h).  The structure (grid
  membership, row numbering) must not change within +- h.

``precision`` selects the forward batch: "fp64" (FP64 factors and solves) or
"mixed" (FP32 factors with double-float refinement; the adjoint then runs on
the same factors, refined to the handle's tolerance).
"""
from __future__ import annotations

from typing import Callable, Sequence, Tuple

import numpy as np

from . import cluster as CL
from . import xanes


def spectrum_loss(sv, items, weights, precision: str = "fp64") -> Tuple[float, list]:
    T, _ = sv.spectrum(items, precision)
    return float(sum(w * xanes.absorption(t) for w, t in zip(weights, T))), T


def loss_and_gradients(sv, build_structure: Callable[[float], CL.Structure], theta: float,
                       energies: Sequence[float], weights: Sequence[float], h: float = 1e-4,
                       precision: str = "fp64"):
    """L(theta), dL/dVr and dL/dtheta.

    build_structure(theta) returns the Structure at parameter theta; sv must hold
    the structure at theta (its grid values).  h is the assembly step (same unit
    as theta).  Returns (L, T list, grad_vr, dL/dtheta, device ms of the vjp).
    """
    st0 = sv.st
    gen = getattr(sv, "radial_args", None) is not None   # inputs generated on the device
    items = xanes.spectrum_inputs(st0, energies, functions=not gen)
    L, T = spectrum_loss(sv, items, weights, precision)
    grad_vr, ms = sv.vjp([xanes.absorption_cotangent(t, w) for t, w in zip(T, weights)])
    dots = []
    for sgn in (1.0, -1.0):
        st_s = build_structure(theta + sgn * h)
        sv.update_grid_values(st_s)
        if gen:
            sv.set_radial()
        dots.append(sv.adjoint_dot(xanes.spectrum_inputs(st_s, energies, functions=not gen)).sum())
    sv.update_grid_values(st0)
    if gen:
        sv.set_radial()
    return L, T, grad_vr, (dots[0] - dots[1]) / (2.0 * h), ms


def cu_shell_structure(delta_ang: float, **kw) -> CL.Structure:
    """Cu cluster of the benchmark with the first shell (2.553 A) moved by delta_ang."""
    adimp = kw.pop("adimp_ang", 0.25)
    rsort = kw.pop("rsort_ang", 3.0)
    rcl = kw.pop("r_cluster_ang", 2.6)
    e_max = kw.pop("e_max_ev", 35.0)
    cl = CL.move_shell(CL.cu_cluster(rcl), 3.61 / np.sqrt(2.0), delta_ang)
    return CL.build_structure(cl, adimp, rsort, e_max, **kw)
