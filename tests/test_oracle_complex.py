"""Known-answer tests that pin the complex (Cal_comp) branch of the oracle.

The reference ships no tests or outputs and cannot be compiled here, so the
complex restatement (oracle/oracle_complex.cpp) is pinned by relations that
the reference's equations must satisfy:

K1  the Gaussian profile solve equals a dense LU solve of the same assembled
    complex matrix (with and without spin-orbit);
K2  the complex machinery on real inputs (Cal_comp with the real basis and
    real harmonics) gives a zero imaginary part and the real branch's solution;
K3  the outgoing-wave (Hankel) basis gives the same Taull as the real basis
    renormalised by (I + iS)^-1 (source/mat.f90:312-343) - two different
    matrices, one physical answer;
K4  spin-orbit with the coupling switched off (gradvr = 0, no relativistic
    terms, spin-diagonal atomic solutions) decouples into two copies of the
    complex-harmonic problem, bit for bit;
K5  complex harmonics give Taull_c = U Taull_r U^H, U the unitary map of Yc
    (source/mat.f90:1733-1754) from the real harmonics;
K7  FDM_comp's irregular cluster solution (both atomic solutions, the
    boundary points split in halves, no outer-sphere rows): the Gaussian
    profile solve equals a dense LU solve of the same assembled matrix, and
    Tau_RI is the product of the two solutions' amplitudes;
K8  a transparent absorber (flat potential at the interstitial level, the
    free-space j_l and n_l as atomic solutions) at a complex energy: the
    regular solution is the incoming wave (atom amplitude sqrt(k/pi), no
    outgoing wave; with the spin-orbit assembly in each spin channel) up to
    the fourth-order stencil's error, and the exact
    irregular field sqrt(k/pi) (-i j_l + n_l) Y satisfies the irregular
    system's grid rows to the same order.  The irregular atom rows follow the
    reference's rule (each amplitude block projected on the half of the
    boundary points of its own atomic solution, source/mat.f90:1582-1605), so
    the two rows of one harmonic share their amplitude entries.
"""
import numpy as np
import pytest

import oracle
from fdmnes_gb300 import abi, cluster as CL, complex_path as CP

E = 12.0


@pytest.fixture(scope="module")
def cu():
    st = CL.small_cu_structure()
    ga = abi.GridArgs(st)
    ei = CL.energy_inputs(st, E)
    ri = CL.newind(st, ei.nlmsa, ei.nlmso)
    ea = abi.EnergyArgs(st, ei, ri)
    X, _ = oracle.mat_solve(ga, ea)
    return st, ga, ea, X


@pytest.fixture(scope="module")
def pt():
    return CP.pt_so_structure()


def _dense_rel(ga, ea):
    X, _ = oracle.mat_solve_c(ga, ea)
    A, B = oracle.assemble_dense_c(ga, ea)
    Xd = np.linalg.solve(A, B.T).T
    return np.abs(X - Xd).max() / np.abs(Xd).max()


def test_k1_dense_lu_complex_harmonics(pt):
    ga = abi.GridArgs(CP.grid_dict(pt, False))
    ea = abi.EnergyArgs(CP.energy_dict(pt, E, spinorbit=False, ylm_comp=True))
    assert _dense_rel(ga, ea) < 1e-12


def test_k1_dense_lu_spin_orbit(pt):
    """Spin-orbit with the relativistic and gradient terms and a model coupling
    (nligne 1826, 200 right-hand sides); measured 2.5e-11."""
    ga = abi.GridArgs(CP.grid_dict(pt, True))
    ea = abi.EnergyArgs(CP.energy_dict(pt, E, spinorbit=True))
    assert _dense_rel(ga, ea) < 1e-9


def test_k2_complex_machinery_on_real_inputs(cu):
    st, ga, ea, Xr = cu
    d = dict(ea.d)
    d.update(Cal_comp=1)
    Xc, _ = oracle.mat_solve_c(ga, abi.EnergyArgs(d))
    assert np.abs(Xc.imag).max() == 0.0
    # the outer rows associate poidso*Y*Y differently in the two branches
    assert np.abs(Xc.real - Xr).max() <= 1e-12 * np.abs(Xr).max()


def test_k3_outgoing_basis_equals_renormalised_real_basis(cu):
    st, ga, ea, Xr = cu
    Tr = oracle.taull(ga, ea, Xr)
    ea3 = abi.EnergyArgs(CP.energy_dict(st, E, spinorbit=False, ylm_comp=False))
    X3, _ = oracle.mat_solve_c(ga, ea3)
    T3 = oracle.taull_c(ga, ea3, X3, symmetrise=True)[:, 0, :, 0]
    assert np.abs(T3 - Tr).max() <= 1e-11 * np.abs(Tr).max()


def test_k4_spin_orbit_without_coupling_decouples(pt):
    g = pt.grid
    ga1 = abi.GridArgs(CP.grid_dict(pt, False))
    ea1 = abi.EnergyArgs(CP.energy_dict(pt, E, spinorbit=False, ylm_comp=True))
    X1, _ = oracle.mat_solve_c(ga1, ea1)
    T1 = oracle.taull_c(ga1, ea1, X1, symmetrise=False)[:, 0, :, 0]
    ga2 = abi.GridArgs(CP.grid_dict(pt, True))
    ea2 = abi.EnergyArgs(CP.energy_dict(pt, E, spinorbit=True, relativistic=False, so_coupling=0.0,
                                        gradvr=np.zeros((g.npoint, 3, 2), order="F")))
    X2, _ = oracle.mat_solve_c(ga2, ea2)
    T2 = oracle.taull_c(ga2, ea2, X2, symmetrise=False)
    assert np.array_equal(T2[:, 0, :, 0], T1)
    assert np.array_equal(T2[:, 1, :, 1], T1)
    assert np.abs(T2[:, 0, :, 1]).max() == 0.0 and np.abs(T2[:, 1, :, 0]).max() == 0.0
    # the dipole cross-section of the two decoupled spins is twice the spinless one
    from fdmnes_gb300 import xanes
    assert abs(xanes.absorption_so(T2) - 2.0 * xanes.absorption(T1)) <= 1e-14 * abs(xanes.absorption(T1))


def test_k5_complex_harmonics_are_a_unitary_change_of_basis(cu):
    st, ga, _, _ = cu
    ear = abi.EnergyArgs(CP.energy_dict(st, E, spinorbit=False, ylm_comp=False))
    eac = abi.EnergyArgs(CP.energy_dict(st, E, spinorbit=False, ylm_comp=True))
    Tr = oracle.taull_c(ga, ear, oracle.mat_solve_c(ga, ear)[0], symmetrise=False)[:, 0, :, 0]
    Tc = oracle.taull_c(ga, eac, oracle.mat_solve_c(ga, eac)[0], symmetrise=False)[:, 0, :, 0]
    n = Tc.shape[0]
    lmax = int(round(np.sqrt(n))) - 1
    U = np.zeros((n, n), complex)
    for L in range(lmax + 1):
        for m in range(-L, L + 1):
            e1 = np.zeros(n)
            e2 = np.zeros(n)
            e1[L * L + L + m] = 1.0
            e2[L * L + L - m] = 1.0
            U[L * L + L + m] = CP.yc(m, e1, e2)
    assert np.allclose(U @ U.conj().T, np.eye(n), atol=1e-15)
    assert np.abs(Tc - U @ Tr @ U.conj().T).max() <= 1e-12 * np.abs(Tc).max()


def test_newind_spin_orbit_matches_oracle(pt):
    """Row numbering with interleaved spin rows (nspino = 2): the package's
    newind and the oracle's agree, and both spin rows of a point share its
    span and its point (source/mat.f90:1841-1844,1883)."""
    ga = abi.GridArgs(CP.grid_dict(pt, True))
    ei = CL.energy_inputs(pt, E)
    nlmsa = (2 * (ei.lmaxa + 1) ** 2).astype(np.int32)
    nlmso = 2 * (ei.lmaxso + 1) ** 2
    ri = CL.newind(pt, nlmsa, nlmso, 2)
    g = pt.grid
    new, newinv, ianew, lb1, lb2 = oracle.newind(ga, g.xyz[3], pt.distai, nlmsa, nlmso, ri.nligne, g.npoint,
                                                 pt.natome)
    assert np.array_equal(new, ri.new) and np.array_equal(newinv, ri.newinv)
    assert np.array_equal(ianew, ri.ianew)
    assert np.array_equal(lb1, ri.lb1) and np.array_equal(lb2, ri.lb2)
    inter = np.nonzero(ri.new[1:])[0] + 1
    rows = ri.new[inter]
    assert np.array_equal(ri.newinv[rows - 1], inter) and np.array_equal(ri.newinv[rows - 2], inter)
    assert np.array_equal(ri.lb1[rows - 2], ri.lb1[rows - 1])
    assert np.array_equal(ri.lb2[rows - 2], ri.lb2[rows - 1])


def test_newind_irregular_matches_oracle():
    """The irregular numbering (both atomic solutions, no outer-sphere rows):
    the host's newind and the oracle's independent restatement agree, on the
    13-atom Cu cluster (nspino = 1) and on a two-spin-block Pt cluster with
    spin-orbit tables (nspino = 2)."""
    from fdmnes_gb300 import cluster as CL
    cases = []
    cu = CL.build_structure(CL.cu_cluster(2.6), 0.3, 3.0, 35.0)
    cases.append((cu, abi.GridArgs(cu), 1))
    ptc = CL.build_structure(CL.pt_cluster(2.8), 0.3, 3.0, 35.0, nspin=2)
    cases.append((ptc, abi.GridArgs(CP.grid_dict(ptc, True)), 2))
    for st, ga, nspino in cases:
        ei = CL.energy_inputs(st, E)
        nlmsa = (nspino * (ei.lmaxa + 1) ** 2).astype(np.int32)
        nlmso = nspino * (ei.lmaxso + 1) ** 2
        ri = CL.newind(st, nlmsa, nlmso, nspino, irregular=True)
        g = st.grid
        new, newinv, ianew, lb1, lb2 = oracle.newind(ga, g.xyz[3], st.distai, nlmsa, nlmso, ri.nligne, g.npoint,
                                                     st.natome, irregular=True)
        assert st.natome > 1
        assert np.array_equal(new, ri.new) and np.array_equal(newinv, ri.newinv)
        assert np.array_equal(ianew, ri.ianew)
        assert np.array_equal(lb1, ri.lb1) and np.array_equal(lb2, ri.lb2)


def test_gradpot_is_exact_on_linear_potentials(pt):
    """gradvr (source/potential.f90:5436-5477) on V = a.r + b returns a at every
    point whose 12 neighbours lie inside the grid, axis k of neighbour pair iv
    being 1 + ((iv - 1) / 2) mod 3 as the spin-orbit terms of calcMatRow assume;
    the second spin block carries its own potential."""
    import dataclasses
    g = pt.grid
    xyz = g.xyz[:3, :g.npoint]
    a = np.array([0.3, -0.7, 1.1])
    V = (a[:, None] * xyz).sum(0) + 0.5
    st = dataclasses.replace(pt, Vr=np.asfortranarray(np.stack([V, 2.0 * V], 1)))
    gv = CP.gradpot(st, g.cgrad, g.ivois)
    nb = g.ivois[:g.npoint, :12]
    inner = np.all((nb >= 1) & (nb <= g.npoint), axis=1)
    assert inner.sum() > 100
    assert np.abs(gv[inner, :, 0] - a).max() < 1e-13
    assert np.abs(gv[inner, :, 1] - 2.0 * a).max() < 1e-13


def test_oracle_reproduces_the_complex_golden_fixture(golden_complex):
    """The committed spin-orbit fixture (tests/golden/make_golden.py) is
    reproduced by the oracle on its stored inputs: the oracle's complex branch
    has not drifted since the fixture was written."""
    g, e, X0, T0 = golden_complex
    ga, ea = abi.GridArgs(g), abi.EnergyArgs(e)
    X, _ = oracle.mat_solve_c(ga, ea)
    assert np.abs(X - X0).max() <= 1e-12 * np.abs(X0).max()
    T = oracle.taull_c(ga, ea, X)
    assert np.abs(T - T0).max() <= 1e-12 * np.abs(T0).max()


def test_k4_thirteen_atoms():
    """K4 on a 13-atom Pt cluster (coarse 0.45 A grid, FDM radius 3.0 A): with
    the spin-orbit coupling off, every atom's interleaved spin rows and the
    spin-doubled outer rows reproduce the complex-harmonic problem bit for bit
    on both spins (nligne 2722 with spin-orbit)."""
    st = CL.build_structure(CL.pt_cluster(2.8), 0.45, 3.0, 15.0, nspin=2)
    assert st.natome == 13
    g = st.grid
    ga1 = abi.GridArgs(CP.grid_dict(st, False))
    ea1 = abi.EnergyArgs(CP.energy_dict(st, 8.0, spinorbit=False, ylm_comp=True))
    T1 = oracle.taull_c(ga1, ea1, oracle.mat_solve_c(ga1, ea1)[0], symmetrise=False)[:, 0, :, 0]
    ga2 = abi.GridArgs(CP.grid_dict(st, True))
    ea2 = abi.EnergyArgs(CP.energy_dict(st, 8.0, spinorbit=True, relativistic=False, so_coupling=0.0,
                                        gradvr=np.zeros((g.npoint, 3, 2), order="F")))
    T2 = oracle.taull_c(ga2, ea2, oracle.mat_solve_c(ga2, ea2)[0], symmetrise=False)
    assert np.array_equal(T2[:, 0, :, 0], T1) and np.array_equal(T2[:, 1, :, 1], T1)


def test_cbessneu_matches_scipy_for_complex_arguments():
    """cbessneu (source/sphere.f90:7226-7254), the complex-energy outer
    functions of phiso, against scipy's spherical_jn / spherical_yn of complex
    argument times the complex sqrt(k / pi), for the orders the upward
    recursion resolves (l up to about |z| + 3: beyond, j_l falls below the
    recursion's cancellation, in the reference's algorithm as here); the
    package's numpy restatement gives the oracle's values."""
    from scipy import special
    k = np.sqrt(1.9 + 0.05j)
    f = np.sqrt(k / np.pi)
    for z, lmax in ((0.8 + 0.02j, 3), (3.7 + 0.21j, 7), (9.0 + 0.4j, 12)):
        b, n = oracle.cbessneu(f, z, lmax)
        bj = f * np.array([special.spherical_jn(L, z) for L in range(lmax + 1)])
        by = f * np.array([special.spherical_yn(L, z) for L in range(lmax + 1)])
        assert np.all(np.abs(b - bj) <= 1e-11 * np.abs(bj)), z
        assert np.all(np.abs(n - by) <= 1e-12 * np.abs(by)), z
        bp, np_ = CP.cbessneu(f, np.array([z]), lmax)
        assert np.allclose(bp[0], b, rtol=1e-10, atol=0) and np.allclose(np_[0], n, rtol=1e-10, atol=0)


@pytest.mark.parametrize("spinorbit", [False, True])
def test_k6_complex_energy_is_continuous_at_real_energies(pt, spinorbit):
    """K6: the complex-energy regular system (E_comp: complex-argument
    Hankel functions, -i Eimag on the grid diagonal) tends to the real-energy
    system as Eimag -> 0 (5.6e-13 at Eimag = 1e-12 Ry), departs linearly (the
    same slope at 1e-8 and 1e-6 Ry), and its profile solve matches a dense LU
    at a finite broadening."""
    ga = abi.GridArgs(CP.grid_dict(pt, spinorbit))
    X0, _ = oracle.mat_solve_c(ga, abi.EnergyArgs(CP.energy_dict(pt, E, spinorbit=spinorbit)))
    diff = {}
    for eim in (1e-12, 1e-8, 1e-6):
        X, _ = oracle.mat_solve_c(ga, abi.EnergyArgs(CP.energy_dict(pt, E, spinorbit=spinorbit, eimag_ry=eim)))
        diff[eim] = np.abs(X - X0).max() / np.abs(X0).max()
    assert diff[1e-12] < 1e-10
    assert abs(diff[1e-8] / 1e-8 - diff[1e-6] / 1e-6) <= 0.05 * diff[1e-6] / 1e-6
    ea = abi.EnergyArgs(CP.energy_dict(pt, E, spinorbit=spinorbit, eimag_ry=0.037))
    assert _dense_rel(ga, ea) < (1e-9 if spinorbit else 1e-12)


EIMAG_RY = 0.5 / 13.605693122994


@pytest.mark.parametrize("spinorbit", [False, True])
def test_k7_dense_lu_irregular_solution(pt, spinorbit):
    """Irregular solution at 12 eV + 0.5 eV i (nligne 838 / 1676); measured
    1.8e-12 and 2.9e-12."""
    ga = abi.GridArgs(CP.grid_dict(pt, spinorbit))
    ea = abi.EnergyArgs(CP.energy_dict(pt, E, spinorbit=spinorbit, eimag_ry=EIMAG_RY, irregular=True))
    assert ea.d["nligneso"] == ea.nligne
    assert _dense_rel(ga, ea) < 1e-9


def test_newind_irregular_numbering(pt):
    """newind with the irregular solution (source/mat.f90:1761-1921): no
    outer-sphere rows, 2 nlmsa amplitude rows per atom, the grid rows in the
    regular numbering's order, a profile that brackets the diagonal."""
    from fdmnes_gb300 import cluster as CL
    for nspino in (1, 2):
        ei = CL.energy_inputs(pt, E)
        nlmsa = (nspino * (ei.lmaxa + 1) ** 2).astype(np.int32)
        nlmso = nspino * (ei.lmaxso + 1) ** 2
        reg = CL.newind(pt, nlmsa, nlmso, nspino)
        irr = CL.newind(pt, nlmsa, nlmso, nspino, irregular=True)
        assert irr.nligne == reg.nligne - nlmso + int(nlmsa.sum())
        assert irr.nligneso == irr.nligne
        assert not np.any(irr.newinv == 0)
        for ia in range(pt.natome):
            assert np.count_nonzero(irr.newinv == -(ia + 1)) == 2 * nlmsa[ia]
        assert np.array_equal(reg.newinv[reg.newinv > 0], irr.newinv[irr.newinv > 0])
        rows = np.arange(1, irr.nligne + 1)
        assert np.all(irr.lb1 <= rows) and np.all(rows <= irr.lb2) and np.all(irr.lb2 <= irr.nligne)
        assert np.all(np.diff(irr.lb1) >= 0)


def test_k7_tau_ri_is_the_amplitude_product(pt):
    """Tau_RI(Lm1, Lm2, i_RI) = sum_f Ampl(f, Lm1) Ampl_I(f, (i_RI - 1) nlmsa + Lm2)
    (source/mat.f90:219-292), restated here with numpy on the oracle's solutions."""
    from fdmnes_gb300 import cluster as CL
    ga = abi.GridArgs(CP.grid_dict(pt, False))
    er = abi.EnergyArgs(CP.energy_dict(pt, E, spinorbit=False, eimag_ry=EIMAG_RY, fdm_comp=True))
    ei = abi.EnergyArgs(CP.energy_dict(pt, E, spinorbit=False, eimag_ry=EIMAG_RY, irregular=True))
    Xr, _ = oracle.mat_solve_c(ga, er)
    Xi, _ = oracle.mat_solve_c(ga, ei)
    T = oracle.tau_ri(ga, er, Xr, ei, Xi)
    nl = int(er.d["nlmsa"][0])
    a0, b0 = int(er.d["ianew"][0]), int(ei.d["ianew"][0])
    lato, mato = ga.d["lato"][:nl, 0], ga.d["mato"][:nl, 0]
    idx = lato * lato + lato + mato
    ref = np.zeros_like(T)
    for iri in range(2):
        P = Xr[:, a0:a0 + nl].T @ Xi[:, b0 + iri * nl:b0 + (iri + 1) * nl]
        ref[np.ix_(idx, [0], idx, [0], [iri])] = P[:, None, :, None, None]
    assert np.abs(T - ref).max() <= 1e-12 * np.abs(ref).max()
    assert np.abs(T[..., 1]).max() > 0


def test_irregular_solution_needs_complex_energies(pt):
    with pytest.raises(ValueError):
        CP.energy_dict(pt, E, spinorbit=False, irregular=True)
    ga = abi.GridArgs(CP.grid_dict(pt, False))
    d = CP.energy_dict(pt, E, spinorbit=False, eimag_ry=EIMAG_RY, irregular=True)
    d.update(Test_reg=1)     # the reference's test keyword: not restated
    with pytest.raises(RuntimeError):
        oracle.mat_solve_c(ga, abi.EnergyArgs(d))


def _transparent_pt(adimp, irregular, E=12.0):
    """Pt absorber alone, flat potential at the interstitial level of each spin
    block, complex energy (0.5 eV), phiato = free-space j_l (regular) and n_l
    (irregular) times the complex harmonics."""
    st = CP.pt_so_structure(adimp_ang=adimp)
    g = st.grid
    for isp in range(st.nspin):
        st.Vr[:, isp] = st.V0bd + st.spin_shift(isp + 1)
    ga = abi.GridArgs(CP.grid_dict(st, False))
    d = CP.energy_dict(st, E, spinorbit=False, eimag_ry=EIMAG_RY, fdm_comp=True, irregular=irregular)
    from fdmnes_gb300 import cluster as CL
    k = np.sqrt(complex(CL.energy_inputs(st, E).ecinetic_out, EIMAG_RY))
    nl = int(d["nlmsa"][0])
    lmaxa = int(round(np.sqrt(nl))) - 1
    nb = int(g.nbord[0])
    bs, nm = CP.cbessneu(1.0, k * st.rrel[:nb, 0], lmaxa)
    phi = np.zeros_like(d["phiato"])
    for L in range(lmaxa + 1):
        for m in range(-L, L + 1):
            lm = L * L + L + m
            y = CP.yc(m, st.Ylmato[:nb, lm, 0], st.Ylmato[:nb, lm - 2 * m, 0])
            for iri, f in enumerate((bs[:, L], nm[:, L])):
                v = f * y
                phi[:nb, lm, :, 0, iri, 0, 0] = v.real[:, None]
                phi[:nb, lm, :, 0, iri, 0, 1] = v.imag[:, None]
    d["phiato"] = np.asfortranarray(phi)
    return st, ga, abi.EnergyArgs(d), d, np.sqrt(k / np.pi), k


def test_k8_transparent_absorber_regular_solution():
    """Measured: amplitude error 1.4e-3 / 3.0e-4 and outgoing amplitudes
    1.1e-3 / 2.4e-4 at h = 0.3 / 0.2 A (L <= 3 waves)."""
    errs = []
    for h, bar in ((0.3, 3e-3), (0.2, 6e-4)):
        st, ga, ea, d, fn, _ = _transparent_pt(h, irregular=False)
        X, _ = oracle.mat_solve_c(ga, ea)
        sel = np.nonzero(np.floor(np.sqrt(np.arange(d["nlmso"]))) <= 3)[0]
        a0, nl = int(d["ianew"][0]), int(d["nlmsa"][0])
        amp = np.abs(X[sel][:, a0:a0 + nl][:, sel] - fn * np.eye(len(sel))).max() / abs(fn)
        out = np.abs(X[sel][:, d["nligneso"]:][:, sel]).max()
        assert amp < bar and out < bar, (h, amp, out)
        errs.append(amp)
    assert errs[1] < errs[0] / 3


def test_k8_irregular_grid_rows_hold_the_free_space_field():
    """Residual of the irregular system's grid rows at the exact field
    (normwise per row); measured for L <= 1: 3.3e-5 at h = 0.3 A, 2.7e-6 at 0.2 A."""
    from fdmnes_gb300 import cluster as CL
    res_h = []
    for h in (0.3, 0.2):
        st, ga, ea, d, fn, k = _transparent_pt(h, irregular=True)
        A, B = oracle.assemble_dense_c(ga, ea)
        newinv = np.asarray(d["newinv"])
        rows = np.nonzero(newinv > 0)[0]
        xyz = st.grid.xyz[:3, newinv[rows] - 1]
        bs, nm = CP.cbessneu(fn, k * np.sqrt((xyz ** 2).sum(0)), 1)
        Y = CL.real_ylm(1, xyz)
        a0, nl = int(d["ianew"][0]), int(d["nlmsa"][0])
        worst = 0.0
        for L, m in ((0, 0), (1, -1), (1, 1)):
            lm = L * L + L + m
            x = np.zeros(A.shape[0], dtype=complex)
            x[rows] = (-1j * bs[:, L] + nm[:, L]) * CP.yc(m, Y[lm], Y[lm - 2 * m])
            x[a0 + lm] = -1j * fn
            x[a0 + nl + lm] = fn
            r = (A @ x - B[lm])[rows]
            worst = max(worst, np.abs(r).max() / (np.abs(A[rows]).sum(1).max() * np.abs(x).max()))
        res_h.append(worst)
    assert res_h[0] < 1e-4 and res_h[1] < 1e-5 and res_h[1] < res_h[0] / 5, res_h


def test_k8_irregular_atom_rows_follow_the_reference_rule():
    """The rows of the regular and the irregular amplitudes of one harmonic
    carry the same amplitude entries (both blocks projected on their own
    atomic solution's half of the boundary points) and grid entries on
    disjoint halves of the boundary points."""
    st, ga, ea, d, fn, k = _transparent_pt(0.3, irregular=True)
    A, _ = oracle.assemble_dense_c(ga, ea)
    a0, nl = int(d["ianew"][0]), int(d["nlmsa"][0])
    amp = slice(a0, a0 + 2 * nl)
    grid = np.asarray(d["newinv"]) > 0
    for lm in range(nl):
        r1, r2 = A[a0 + lm], A[a0 + nl + lm]
        assert np.array_equal(r1[amp], r2[amp])
        assert not np.any((r1[grid] != 0) & (r2[grid] != 0))
        assert np.any(r1[grid] != 0) and np.any(r2[grid] != 0)


def test_k8_transparent_absorber_spin_orbit():
    """Spin-orbit assembly (interleaved spin rows, lmrep tables, relativistic
    diagonal) on a flat potential, where gradvr and with it every spin-orbit
    coupling term vanishes, with spin-diagonal free-space j_l boundary
    functions: the atom amplitude of harmonic (L, m, s) is sqrt(k/pi) for the
    outer wave (L, m, s) and nothing scatters, in both spin channels.
    Measured 1.5e-3 / 7.7e-4 (amplitudes), 1.1e-3 / 5.9e-4 (outgoing) at
    h = 0.3 / 0.25 A."""
    from fdmnes_gb300 import cluster as CL
    errs = []
    for h, bar in ((0.3, 3e-3), (0.25, 1.5e-3)):
        st = CP.pt_so_structure(adimp_ang=h)
        g = st.grid
        st.Vr[:, :] = st.V0bd
        st.spin_split = 0.0
        ga = abi.GridArgs(CP.grid_dict(st, True))
        d = CP.energy_dict(st, E, spinorbit=True)
        assert np.abs(d["gradvr"]).max() < 1e-12
        k = np.sqrt(CL.energy_inputs(st, E).ecinetic_out)
        fn = np.sqrt(k / np.pi)
        nl = int(d["nlmsa"][0])
        lmaxa = int(round(np.sqrt(nl // 2))) - 1
        nb = int(g.nbord[0])
        bs, _ = CP.cbessneu(1.0, k * st.rrel[:nb, 0], lmaxa)
        phi = np.zeros_like(d["phiato"])
        for L in range(lmaxa + 1):
            for m in range(-L, L + 1):
                lm = L * L + L + m
                v = bs[:, L].real * CP.yc(m, st.Ylmato[:nb, lm, 0], st.Ylmato[:nb, lm - 2 * m, 0])
                for sp in range(2):
                    phi[:nb, lm, sp, sp, 0, 0, 0] = v.real
                    phi[:nb, lm, sp, sp, 0, 0, 1] = v.imag
        d["phiato"] = np.asfortranarray(phi)
        X, _ = oracle.mat_solve_c(ga, abi.EnergyArgs(d))
        nlmso = int(d["nlmso"])
        lso, mso, iso = (ga.d[k_][:nlmso] for k_ in ("lso", "mso", "iso"))
        lato, mato, iato = (ga.d[k_][:nl, 0] for k_ in ("lato", "mato", "iato"))
        sel = np.nonzero(lso <= 3)[0]
        expect = np.zeros((nlmso, nl), dtype=complex)
        for f in sel:
            q = np.nonzero((lato == lso[f]) & (mato == mso[f]) & (iato == iso[f]))[0]
            expect[f, q] = fn
        a0 = int(d["ianew"][0])
        amp = np.abs(X[sel][:, a0:a0 + nl] - expect[sel]).max() / abs(fn)
        out = np.abs(X[sel][:, d["nligneso"]:][:, sel]).max()
        assert amp < bar and out < bar, (h, amp, out)
        errs.append(amp)
    assert errs[1] < errs[0] / 1.6


@pytest.mark.parametrize("eimag", [0.0, 0.04])
def test_singular_radial_solution_free_space(eimag):
    """The singular radial solver (source/sphere.f90:2591-2812) on a flat
    potential is sqrt(k/pi) (n_l - i j_l) everywhere inside its starting
    radius, at real and complex energies (measured 3e-4..8e-4, the radial
    mesh's error)."""
    from fdmnes_gb300 import cluster as CL
    r = CL.radial_mesh(78, 3.0)
    i0 = int(np.searchsorted(r, 2.6))
    k = np.sqrt(complex(1.3, eimag))
    sel = (r > 0.4) & (r < 2.5)
    for L in range(4):
        R = CP.sch_radial_singular(r, np.zeros_like(r), 1.3, eimag, k, L, i0)
        bs, nm = CP.cbessneu(np.sqrt(k / np.pi), k * r[sel], L)
        exact = nm[:, L] - 1j * bs[:, L]
        assert np.abs(R[sel] - exact).max() < 2e-3 * np.abs(exact).max(), L


@pytest.mark.parametrize("spinorbit", [False, True])
def test_k7_dense_lu_irregular_solution_singular_inputs(pt, spinorbit):
    """The irregular system with the singular radial solver's atomic
    solutions: Gaussian profile solve vs dense LU (measured 7.4e-12 / 2.2e-11)."""
    ga = abi.GridArgs(CP.grid_dict(pt, spinorbit))
    ea = abi.EnergyArgs(CP.energy_dict(pt, E, spinorbit=spinorbit, eimag_ry=EIMAG_RY, irregular=True,
                                       irregular_radial="singular"))
    assert _dense_rel(ga, ea) < 1e-9
