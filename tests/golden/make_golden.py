"""Generate the committed golden fixtures of the test suite.

* golden_problem.npz - the complete mat_solve arguments of a small FDM problem
  (fcc Cu absorber, FDM radius 1.4 A, grid step 0.25 A, C1) at two energies,
  with the oracle's solution smr and Taull.  The GPU parity tests load these
  arrays, so both machines solve bit-identical inputs.
* golden_complex.npz - the complex (Cal_comp) mat_solve arguments of a small
  spin-orbit problem (fcc Pt absorber, FDM radius 1.2 A, nspino = 2, complex
  harmonics, relativistic terms) at 6 eV with the oracle's solution
  smr + i smi and its Taull (nlm, 2, nlm, 2).
* kat_special.npz   - known-answer values of the special functions used by the
  inputs: spherical Bessel/Neumann functions from scipy (times sqrt(k/pi), as
  source/sphere.f90:7356 normalises them) and real spherical harmonics from
  scipy's complex Y_lm with the reference's real-harmonics convention
  (source/general.f90:11696-11725).

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from fdmnes_gb300 import abi, cluster as CL, complex_path as CP  # noqa: E402
import oracle  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
ENERGIES = (-5.0, 15.0)


def golden_structure():
    return CL.build_structure(CL.cu_cluster(0.5), 0.25, 1.4, 15.0)


def make_problem():
    st = golden_structure()
    gd = abi.grid_dict(st)
    ga = abi.GridArgs(gd)
    out = {"g_" + k: np.asarray(v) for k, v in gd.items()}
    out["energies"] = np.array(ENERGIES)
    for k, E in enumerate(ENERGIES):
        ei = CL.energy_inputs(st, E)
        ri = CL.newind(st, ei.nlmsa, ei.nlmso)
        ed = abi.energy_dict(st, ei, ri)
        ea = abi.EnergyArgs(ed)
        X, _ = oracle.mat_solve(ga, ea)
        T = oracle.taull(ga, ea, X)
        out.update({f"e{k}_" + n: np.asarray(v) for n, v in ed.items()})
        out[f"e{k}_smr"] = X
        out[f"e{k}_taull"] = T
        A, B = oracle.assemble_dense(ga, ea)
        out[f"e{k}_dense_solution"] = np.linalg.solve(A, B.T).T
    np.savez_compressed(os.path.join(OUT, "golden_problem.npz"), **out)


def make_complex():
    st = CL.build_structure(CL.pt_cluster(0.5), 0.25, 1.2, 15.0, nspin=2)
    gd = CP.grid_dict(st, True)
    ga = abi.GridArgs(gd)
    ed = CP.energy_dict(st, 6.0, spinorbit=True)
    ea = abi.EnergyArgs(ed)
    X, _ = oracle.mat_solve_c(ga, ea)
    T = oracle.taull_c(ga, ea, X)
    out = {"g_" + k: np.asarray(v) for k, v in gd.items()}
    out.update({"e_" + k: np.asarray(v) for k, v in ed.items()})
    out["smr"], out["smi"], out["taull"] = X.real.copy(), X.imag.copy(), T
    np.savez_compressed(os.path.join(OUT, "golden_complex.npz"), **out)


def make_special():
    from scipy import special
    z = np.array([0.3, 1.0, 2.5, 7.0, 13.0])
    lmax = 10
    fnorm = 0.7
    jn = np.array([[fnorm * special.spherical_jn(l, zz) for l in range(lmax + 1)] for zz in z])
    yn = np.array([[fnorm * special.spherical_yn(l, zz) for l in range(lmax + 1)] for zz in z])
    rng = np.random.default_rng(1)
    v = rng.standard_normal((3, 12))
    v[:, 0] = [0.0, 0.0, 1.3]
    v[:, 1] = [0.4, -0.2, 0.0]
    lmax_y = 6
    r = np.sqrt((v ** 2).sum(0))
    theta = np.arccos(np.clip(v[2] / r, -1, 1))
    phi = np.arctan2(v[1], v[0])
    ylm = []
    for L in range(lmax_y + 1):
        for m in range(-L, L + 1):
            yc = special.sph_harm_y(L, abs(m), theta, phi)   # complex Y_L^{|m|}
            if m < 0:
                ylm.append((-1) ** m * np.sqrt(2) * yc.imag)
            elif m == 0:
                ylm.append(yc.real)
            else:
                ylm.append((-1) ** m * np.sqrt(2) * yc.real)
    np.savez_compressed(os.path.join(OUT, "kat_special.npz"), z=z, fnorm=fnorm, jn=jn, yn=yn, v=v,
                        ylm=np.array(ylm), lmax_y=lmax_y)


if __name__ == "__main__":
    oracle.build()
    make_problem()
    make_complex()
    make_special()
    print("written", sorted(f for f in os.listdir(OUT) if f.endswith(".npz")))
