"""CPU emulation of the mixed path's FP32 factor numerics (test infrastructure).

Reproduces the refinement behaviour of the GPU's FP32 factor on full Cu
matrices assembled by the oracle, and the variants that were weighed against
it: the reversed row order, power-of-two row-then-column equilibration,
64-row tile-local partial pivoting and FP32 storage of the band, with each
step's operations either in FP32 arithmetic or with FP64 accumulation of the
FP32 operands (rounded to FP32 after, as double-float sums would be).  The
refinement uses an FP64 residual and reports how many corrections reach
max|dx|/max|x| <= 1e-8 and the median contraction per step.

It also locates the element growth: per diagonal tile, the smallest ratio of
the chosen pivot to the largest entry of its column below, and the largest
multiplier below the tile.

Run from the repository root (about a minute per energy and variant):
    python oracle/factor_emulation.py --energies 22 26 34
    python oracle/factor_emulation.py --energies 22 --growth
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np
import scipy.linalg as sl

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from fdmnes_gb300 import abi, cluster as CL  # noqa: E402

TS = 64
VARIANTS = {
    "fp32": (False, False),               # FP32 arithmetic throughout
    "wide-trailing-atom": ("atom", False),
    "wide-panel-atom": (False, "atom"),
    "wide-atom": ("atom", "atom"),
    "wide-everywhere": (True, True),
}


def equilibrated_system(st, energy):
    """Reversed-order, power-of-two equilibrated matrix and RHS of one energy,
    and the tile rows that hold atom-harmonic rows."""
    ga = abi.GridArgs(st)
    ei = CL.energy_inputs(st, energy)
    ri = CL.newind(st, ei.nlmsa, ei.nlmso)
    A, B = oracle.assemble_dense(ga, abi.EnergyArgs(st, ei, ri))
    n = A.shape[0]
    Ar = A[::-1, ::-1].copy()
    Br = B.T[::-1].copy()
    r = 2.0 ** -np.round(np.log2(np.abs(Ar).max(1)))
    As = Ar * r[:, None]
    c = 2.0 ** -np.round(np.log2(np.abs(As).max(0)))
    As = As * c[None, :]
    atom_rows = (ri.newinv < 0)[::-1]
    atom_tiles = {t for t in range((n + TS - 1) // TS) if atom_rows[t * TS:(t + 1) * TS].any()}
    return As, Br * r[:, None], atom_tiles


def factor(As, atom_tiles, wide_trailing, wide_panel):
    """Blocked LU with tile-local pivoting and FP32 storage; returns (LU, perm)."""
    n = As.shape[0]
    M = As.astype(np.float32).copy()
    perm = np.arange(n)
    for k0 in range(0, n, TS):
        k1 = min(n, k0 + TS)
        atom = (k0 // TS) in atom_tiles
        wt = atom if wide_trailing == "atom" else bool(wide_trailing)
        wp = atom if wide_panel == "atom" else bool(wide_panel)
        for k in range(k0, k1):
            p = k + int(np.argmax(np.abs(M[k:k1, k])))
            if p != k:
                M[[k, p], :] = M[[p, k], :]
                perm[[k, p]] = perm[[p, k]]
            if wp:
                col = (M[k + 1:, k].astype(np.float64) / np.float64(M[k, k])).astype(np.float32)
                M[k + 1:, k] = col
                M[k + 1:, k + 1:k1] = (M[k + 1:, k + 1:k1].astype(np.float64) -
                                       np.outer(col.astype(np.float64), M[k, k + 1:k1].astype(np.float64))
                                       ).astype(np.float32)
            else:
                M[k + 1:, k] /= M[k, k]
                M[k + 1:, k + 1:k1] -= np.outer(M[k + 1:, k], M[k, k + 1:k1])
        if k1 < n:
            L = np.tril(M[k0:k1, k0:k1], -1) + np.eye(k1 - k0, dtype=np.float32)
            if wp:
                M[k0:k1, k1:] = sl.solve_triangular(L.astype(np.float64), M[k0:k1, k1:].astype(np.float64),
                                                    lower=True, unit_diagonal=True).astype(np.float32)
            else:
                M[k0:k1, k1:] = sl.solve_triangular(L, M[k0:k1, k1:], lower=True, unit_diagonal=True)
            if wt:
                M[k1:, k1:] = (M[k1:, k1:].astype(np.float64) -
                               M[k1:, k0:k1].astype(np.float64) @ M[k0:k1, k1:].astype(np.float64)
                               ).astype(np.float32)
            else:
                M[k1:, k1:] -= M[k1:, k0:k1] @ M[k0:k1, k1:]
    return M, perm


def refine(As, Bs, M, perm, maxit=60):
    """Classical refinement with the FP32 factors and an FP64 residual."""
    X = np.zeros_like(Bs)
    hist = []
    for _ in range(maxit):
        R = (Bs - As @ X)[perm].astype(np.float32)
        y = sl.solve_triangular(M, R, lower=True, unit_diagonal=True)
        D = sl.solve_triangular(M, y, lower=False).astype(np.float64)
        X += D
        hist.append(np.abs(D).max() / np.abs(X).max())
        if not np.isfinite(hist[-1]) or hist[-1] < 1e-10:
            break
    return hist


def growth(As, atom_tiles):
    """Per tile: min |pivot| / max |column below| and max multiplier below the tile."""
    n = As.shape[0]
    M = As.copy()
    out = []
    for k0 in range(0, n, TS):
        k1 = min(n, k0 + TS)
        minpiv, maxl = np.inf, 0.0
        for k in range(k0, k1):
            p = k + int(np.argmax(np.abs(M[k:k1, k])))
            if p != k:
                M[[k, p], :] = M[[p, k], :]
            minpiv = min(minpiv, abs(M[k, k]) / np.abs(M[k:, k]).max())
            M[k + 1:, k] /= M[k, k]
            M[k + 1:, k + 1:k1] -= np.outer(M[k + 1:, k], M[k, k + 1:k1])
            M[k + 1:k1, k1:] -= np.outer(M[k + 1:k1, k], M[k, k1:])
            if k1 < n:
                maxl = max(maxl, np.abs(M[k1:, k]).max())
        if k1 < n:
            M[k1:, k1:] -= M[k1:, k0:k1] @ M[k0:k1, k1:]
        out.append((k0 // TS, (k0 // TS) in atom_tiles, minpiv, maxl))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--energies", type=float, nargs="+", default=[22.0, 26.0, 34.0])
    ap.add_argument("--variants", nargs="+", default=["fp32", "wide-trailing-atom", "wide-atom"],
                    choices=sorted(VARIANTS))
    ap.add_argument("--growth", action="store_true", help="report the element growth per tile instead")
    args = ap.parse_args()
    oracle.build()
    st = CL.cu_structure()
    for E in args.energies:
        As, Bs, atom_tiles = equilibrated_system(st, E)
        if args.growth:
            rows = sorted(growth(As, atom_tiles), key=lambda t: -t[3])[:8]
            for t, atom, mp, ml in rows:
                print(f"E={E:5.1f} tile {t:3d} atom rows={atom!s:5s} min |pivot|/best below={mp:.1e} "
                      f"max multiplier below={ml:.1e}", flush=True)
            continue
        for name in args.variants:
            wt, wp = VARIANTS[name]
            M, perm = factor(As, atom_tiles, wt, wp)
            h = refine(As, Bs, M, perm)
            k8 = next((i + 1 for i, v in enumerate(h) if v < 1e-8), None)
            ratio = np.median([h[i + 1] / h[i] for i in range(len(h) - 1)])
            print(f"E={E:5.1f} {name:20s} steps to 1e-8: {k8}  median contraction {ratio:.2f}", flush=True)


if __name__ == "__main__":
    main()
