"""Gradient fit of a shell distance to a target spectrum through the adjoint.

The role of the reference's fitting loop (source/minim.f90), restricted to one
structural parameter: theta moves the first coordination shell of the
absorber radially.  Loss L(theta) = sum_E (sigma_E(theta) - target_E)^2 with
sigma the dipole absorption -Im Tr Taull(L=1).  Each step runs the batched
spectrum (FP64, or mixed precision with ``--precision mixed``), one
vector-Jacobian product (cotangent 2 (sigma - target))
and the two adjoint dot products that give dL/dtheta
(``gradients``); the step length follows Barzilai-Borwein.  The grid's
membership (which points lie inside atoms) can change between steps, so the
handle is rebuilt for every theta.

Usage:  python -m fdmnes_gb300.fit [--energies N] [--steps K] [--offset A] [--precision P]
"""
from __future__ import annotations

import argparse
import json
import time
from typing import Callable, List, Sequence

import numpy as np

from . import cluster as CL
from . import xanes
from .solver import FdmError, FdmSolver


def sigma_spectrum(st: CL.Structure, energies: Sequence[float]) -> np.ndarray:
    sv = FdmSolver(st)
    sv.set_radial()
    T, _ = sv.spectrum(xanes.spectrum_inputs(st, energies, functions=False), "fp64")
    sv.close()
    return np.array([xanes.absorption(t) for t in T])


def loss_grad(build: Callable[[float], CL.Structure], theta: float, energies: Sequence[float],
              target: np.ndarray, h: float = 1e-4, precision: str = "fp64"):
    """L(theta) and dL/dtheta through the adjoint of the batch of ``precision``."""
    st = build(theta)
    sv = FdmSolver(st)
    sv.set_radial()   # phiato / Bessel / Neumann of every energy generated on the device
    if precision == "mixed":
        sv.set_tolerance(1e-8, 1e-6)
    items = xanes.spectrum_inputs(st, energies, functions=False)
    T, _ = sv.spectrum(items, precision)
    sig = np.array([xanes.absorption(t) for t in T])
    r = sig - target
    try:
        sv.vjp([xanes.absorption_cotangent(t, 2.0 * rk) for t, rk in zip(T, r)])
    except FdmError:
        # a mixed batch with an energy the mixed path could not refine (left
        # unconverged or re-solved in FP64) has no mixed adjoint: this step
        # runs in FP64
        T, _ = sv.spectrum(items, "fp64")
        sig = np.array([xanes.absorption(t) for t in T])
        r = sig - target
        sv.vjp([xanes.absorption_cotangent(t, 2.0 * rk) for t, rk in zip(T, r)])
    # central difference of the adjoint dot product; where a grid point
    # changes membership between theta and theta +- h (the integer structure
    # differs, so the handle's values cannot be swapped), that side is theta
    # itself and the difference one-sided
    dots, steps = [], []
    for sgn in (1.0, -1.0):
        st_s = build(theta + sgn * h)
        try:
            sv.update_grid_values(st_s)
            dt = sgn * h
        except FdmError:
            st_s = st
            sv.update_grid_values(st_s)
            dt = 0.0
        sv.set_radial()
        dots.append(sv.adjoint_dot(xanes.spectrum_inputs(st_s, energies, functions=False)).sum())
        steps.append(dt)
    sv.close()
    if steps[0] == steps[1]:
        raise FdmError(1, "the grid structure changes on both sides of theta within h")
    return float((r ** 2).sum()), (dots[0] - dots[1]) / (steps[0] - steps[1])


def fit(build: Callable[[float], CL.Structure], energies: Sequence[float], target: np.ndarray,
        theta0: float = 0.0, steps: int = 20, step0: float = 1e-3, precision: str = "fp64") -> List[dict]:
    """Barzilai-Borwein gradient descent on theta; returns the per-step history."""
    hist = []
    theta, alpha = theta0, None
    prev = None
    for k in range(steps):
        t0 = time.time()
        L, g = loss_grad(build, theta, energies, target, precision=precision)
        hist.append({"step": k, "theta": theta, "loss": L, "grad": g, "s": time.time() - t0})
        if prev is not None:
            dth, dg = theta - prev[0], g - prev[1]
            alpha = abs(dth / dg) if dg != 0 else alpha
        if alpha is None:
            alpha = step0 / max(abs(g), 1e-300)
        prev = (theta, g)
        theta = theta - alpha * g
    return hist


def main():
    from . import build as B
    from .gradients import cu_shell_structure
    ap = argparse.ArgumentParser()
    ap.add_argument("--energies", type=int, default=41)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--offset", type=float, default=0.03, help="shell displacement of the target (A)")
    ap.add_argument("--precision", choices=("fp64", "mixed"), default="fp64")
    args = ap.parse_args()
    B.build()
    energies = CL.energy_grid(-5.0, 35.0, 40.0 / (args.energies - 1))
    target = sigma_spectrum(cu_shell_structure(args.offset), energies)
    hist = fit(cu_shell_structure, energies, target, 0.0, args.steps, precision=args.precision)
    for hrow in hist:
        print(json.dumps(hrow), flush=True)


if __name__ == "__main__":
    main()
