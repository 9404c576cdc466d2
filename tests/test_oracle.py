"""CPU tests of the oracle restatement and of the input builders.

The reference ships no tests or golden outputs and cannot be compiled here
(Fortran), so the oracle is pinned by known-answer tests: exact stencil
coefficients, closed-form/scipy special functions, a dense LU solve of the
same assembled matrix, the free-space answer of the whole system (a
transparent absorber scatters nothing), and committed golden outputs
(tests/golden).
"""
import numpy as np
import pytest

from conftest import rel
from fdmnes_gb300 import abi, cluster as CL, xanes


def test_stencil_coefficients_and_exactness():
    st = CL.small_cu_structure()
    g = st.grid
    h = g.adimp
    # source/general.f90:9758-9790: clapl = (4/3 h^2) {1, -1/16}, clapl(0) = -7.5/h^2
    assert np.allclose(g.clapl[1:7], 4.0 / 3.0 / h ** 2, rtol=0, atol=1e-12)
    assert np.allclose(g.clapl[7:13], -1.0 / 12.0 / h ** 2, rtol=0, atol=1e-12)
    assert abs(g.clapl[0] + 7.5 / h ** 2) < 1e-12
    # 4th-order Laplacian: exact on polynomials up to degree 5
    offs = [(-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1),
            (-2, 0, 0), (2, 0, 0), (0, -2, 0), (0, 2, 0), (0, 0, -2), (0, 0, 2)]
    rng = np.random.default_rng(0)
    x0 = rng.standard_normal(3)
    for _ in range(5):
        c = rng.standard_normal(6)
        f = lambda p: c[0] * p[0] ** 5 + c[1] * p[1] ** 4 * p[0] + c[2] * p[2] ** 3 + c[3] * p[0] * p[1] * p[2] ** 2 \
            + c[4] * p[1] ** 2 + c[5]
        lap = (c[0] * 20 * x0[0] ** 3 + c[1] * 12 * x0[1] ** 2 * x0[0] + c[2] * 6 * x0[2]
               + c[3] * 2 * x0[0] * x0[1] + c[4] * 2)
        s = g.clapl[0] * f(x0) + sum(g.clapl[iv + 1] * f(x0 + h * np.array(o)) for iv, o in enumerate(offs))
        assert abs(s - lap) < 1e-8 * max(1.0, abs(lap))


def test_bessel_known_answers(oracle_lib):
    d = np.load(CL.__file__.replace("fdmnes_gb300/cluster.py", "tests/golden/kat_special.npz"))
    z, fnorm, jn, yn = d["z"], float(d["fnorm"]), d["jn"], d["yn"]
    lmax = jn.shape[1] - 1
    bs, nm = CL.cbessneur(fnorm, z, lmax)
    for i, zz in enumerate(z):
        lstable = int(max(1, zz))  # upward recursion of j_l is stable for l <~ z
        assert np.allclose(bs[i, :lstable + 1], jn[i, :lstable + 1], rtol=1e-9, atol=0)
        assert np.allclose(nm[i], yn[i], rtol=1e-10, atol=0)
        b2, n2 = oracle_lib.cbessneur(fnorm, zz, lmax)
        assert np.allclose(b2, bs[i], rtol=1e-13, atol=1e-300)
        assert np.allclose(n2, nm[i], rtol=1e-13, atol=1e-300)
    # closed forms of l = 0, 1
    zz = 2.3
    b, n = CL.cbessneur(1.0, np.array([zz]), 1)
    assert abs(b[0, 0] - np.sin(zz) / zz) < 1e-15
    assert abs(n[0, 1] - (-np.cos(zz) / zz ** 2 - np.sin(zz) / zz)) < 1e-15


def test_real_harmonics_known_answers():
    d = np.load(CL.__file__.replace("fdmnes_gb300/cluster.py", "tests/golden/kat_special.npz"))
    y = CL.real_ylm(int(d["lmax_y"]), d["v"])
    assert np.abs(y - d["ylm"]).max() < 1e-12


def test_exchange_sort_matches_reference_rule():
    rng = np.random.default_rng(3)
    key = rng.integers(0, 6, size=60)
    # brute-force restatement of source/general.f90:9529-9543 on integer keys
    a = list(key)
    idx = list(range(len(a)))
    for i in range(len(a)):
        for j in range(i + 1, len(a)):
            if a[i] <= a[j]:
                continue
            a[i], a[j] = a[j], a[i]
            idx[i], idx[j] = idx[j], idx[i]
    assert list(CL._exchange_sort(key)) == idx


def test_grid_sizes_of_cu_cluster():
    st = CL.cu_structure()
    g = st.grid
    assert st.natome == 13
    assert g.npoint == 7153 and g.npr == 4472
    assert g.nbordf[0] > 0 and g.nsortf > 0


def test_radial_solution_free_space():
    # V = 0: the regular solution is proportional to r j_l(k r)
    from scipy.special import spherical_jn
    r = CL.radial_mesh(29, 4.0)
    for L in range(4):
        ec = 1.3
        R = CL.sch_radial(r, np.zeros_like(r), ec, ec, L, 0.0)
        sel = (r > 0.5) & (r < 2.0)
        ratio = R[sel] / spherical_jn(L, np.sqrt(ec) * r[sel])
        assert np.std(ratio) / abs(np.mean(ratio)) < 2e-3


def test_transparent_absorber_does_not_scatter(oracle_lib):
    """Whole-system known answer: with the potential flat at the interstitial
    level and the free-space j_l(k r) Y as the atom's boundary functions,
    nothing scatters: the real-basis scattering amplitudes (the outer rows of
    the solution) of the L <= 3 waves vanish up to the fourth-order stencil's
    error and fall with the grid step (measured 1.1e-3, 2.4e-4 at h = 0.3,
    0.2 A).  Pins the signs and normalisations of the grid, atom and outer
    rows and of the Bessel / Neumann functions together."""
    import dataclasses
    from scipy.special import spherical_jn
    worst = []
    for h in (0.3, 0.2):
        st = CL.build_structure(CL.cu_cluster(0.5), h, 1.6, 35.0)
        g = st.grid
        st.Vr[:, :] = st.V0bd
        ei = CL.energy_inputs(st, 12.0)
        k = np.sqrt(ei.ecinetic_out)
        phi = np.zeros_like(ei.phiato)
        nb = int(g.nbord[0])
        for L in range(int(ei.lmaxa[0]) + 1):
            jl = spherical_jn(L, k * st.rrel[:nb, 0])
            for m in range(-L, L + 1):
                lm = L * L + L + m
                phi[:nb, lm, 0, 0, 0, 0, 0] = jl * st.Ylmato[:nb, lm, 0]
        ei = dataclasses.replace(ei, phiato=phi)
        ri = CL.newind(st, ei.nlmsa, ei.nlmso)
        X, _ = oracle_lib.mat_solve(abi.GridArgs(st), abi.EnergyArgs(st, ei, ri))
        sel = np.nonzero(np.floor(np.sqrt(np.arange(ei.nlmso))) <= 3)[0]
        worst.append(np.abs(X[sel][:, ri.nligneso:][:, sel]).max())
    assert worst[0] < 2e-3 and worst[1] < 5e-4 and worst[1] < worst[0] / 3, worst


def test_transparent_cluster_scattering_falls_with_the_atoms_l_cutoff(oracle_lib):
    """The 13-atom Cu cluster made transparent (flat potential, free-space j_l
    about each atom as its boundary functions): the incoming wave about the
    absorber, seen from a neighbour 2.55 A away, needs many harmonics, so the
    residual scattering is that of the atoms' l cut-off and falls fast as the
    cut-off grows (measured max |S| of the L <= 3 waves 0.127 at lmax 4,
    0.037 at lmax 5, h = 0.3 A).  Pins the multi-atom couplings (amplitude
    blocks, boundary points of every atom) physically."""
    import dataclasses
    from scipy.special import spherical_jn
    st = CL.build_structure(CL.cu_cluster(2.6), 0.3, 3.0, 300.0)
    g = st.grid
    st.Vr[:, :] = st.V0bd
    ei0 = CL.energy_inputs(st, 12.0)
    k = np.sqrt(ei0.ecinetic_out)
    smax = []
    for lmx in (4, 5):
        lmaxa = np.minimum(st.lmaxat_max[st.cluster.itype], lmx).astype(np.int32)
        assert lmaxa.min() == lmx
        nlmsa = ((lmaxa + 1) ** 2).astype(np.int32)
        phi = np.zeros((g.nbtm, int(nlmsa.max()), 1, 1, 1, st.natome, 1), order="F")
        for ia in range(st.natome):
            nb = int(g.nbord[ia])
            for L in range(lmx + 1):
                jl = spherical_jn(L, k * st.rrel[:nb, ia])
                for m in range(-L, L + 1):
                    lm = L * L + L + m
                    phi[:nb, lm, 0, 0, 0, ia, 0] = jl * st.Ylmato[:nb, lm, ia]
        ei = dataclasses.replace(ei0, phiato=phi, lmaxa=lmaxa, nlmsa=nlmsa, nlmagm=int(nlmsa.max()))
        ri = CL.newind(st, ei.nlmsa, ei.nlmso)
        X, _ = oracle_lib.mat_solve(abi.GridArgs(st), abi.EnergyArgs(st, ei, ri))
        sel = np.nonzero(np.floor(np.sqrt(np.arange(ei.nlmso))) <= 3)[0]
        smax.append(np.abs(X[sel][:, ri.nligneso:][:, sel]).max())
    assert smax[0] < 0.2 and smax[1] < smax[0] / 2.5, smax


def test_single_atom_scattering_is_reciprocal_and_unitary(oracle_lib):
    """A real potential at real energies: the T-matrix T = K (I + iK)^-1 built
    from the real-basis scattering amplitudes K of the absorber alone (the
    Taull renormalisation of source/mat.f90:312-343) is symmetric
    (reciprocity) and bounded by 1 (unitarity), up to the discretisation
    (measured asymmetry 8e-5..1.6e-3, |T| 0.91..1.00 at h = 0.25 A)."""
    st = CL.build_structure(CL.cu_cluster(0.5), 0.25, 1.6, 35.0)
    for E in (6.0, 12.0, 25.0):
        ei = CL.energy_inputs(st, E)
        ri = CL.newind(st, ei.nlmsa, ei.nlmso)
        X, _ = oracle_lib.mat_solve(abi.GridArgs(st), abi.EnergyArgs(st, ei, ri))
        K = X[:, ri.nligneso:].T
        T = K @ np.linalg.inv(np.eye(K.shape[0]) + 1j * K)
        sel = np.nonzero(np.floor(np.sqrt(np.arange(K.shape[0]))) <= 3)[0]
        Ts = T[np.ix_(sel, sel)]
        assert np.abs(Ts - Ts.T).max() < 3e-3 * np.abs(Ts).max(), E
        assert np.abs(Ts).max() < 1.001, E


def test_radial_solution_free_space_complex_energy():
    # V = 0 at E + i Eimag: the regular solution is proportional to r j_l(k r),
    # k = sqrt(E + i Eimag) complex (source/sphere.f90:471,548,631-633)
    from fdmnes_gb300 import complex_path as CP
    r = CL.radial_mesh(29, 4.0)
    k = np.sqrt(complex(1.3, 0.04))
    sel = (r > 0.5) & (r < 2.0)
    for L in range(4):
        R = CL.sch_radial(r, np.zeros_like(r), 1.3, 1.3, L, 0.0, 0.04)
        bs, _ = CP.cbessneu(1.0, k * r[sel], L)
        ratio = R[sel] / bs[:, L]
        assert np.std(ratio) / abs(np.mean(ratio)) < 1e-3


def test_newind_matches_oracle(oracle_lib):
    st = CL.small_cu_structure()
    ga = abi.GridArgs(st)
    for E in (-5.0, 20.0):
        ei = CL.energy_inputs(st, E)
        ri = CL.newind(st, ei.nlmsa, ei.nlmso)
        new, newinv, ianew, lb1, lb2 = oracle_lib.newind(ga, st.grid.xyz[3], st.distai, ei.nlmsa, ei.nlmso,
                                                        ri.nligne, st.grid.npoint, st.natome)
        assert (new == ri.new).all() and (newinv == ri.newinv).all() and (ianew == ri.ianew).all()
        assert (lb1 == ri.lb1).all() and (lb2 == ri.lb2).all()


def test_golden_oracle_reproduces(oracle_lib, golden):
    grid, energies = golden
    ga = abi.GridArgs(grid)
    for e in energies:
        ea = abi.EnergyArgs(e)
        X, _ = oracle_lib.mat_solve(ga, ea)
        assert np.array_equal(X, e["smr"])
        T = oracle_lib.taull(ga, ea, X)
        assert rel(T, e["taull"]) < 1e-13


def test_gaussian_solver_against_dense_lu(oracle_lib, golden):
    """Known-answer test: the restated no-pivot profile solver equals a dense
    LAPACK solve of the same assembled matrix (tiny, well-conditioned case)."""
    grid, energies = golden
    for e in energies:
        assert rel(e["smr"], e["dense_solution"]) < 1e-10
    ga = abi.GridArgs(grid)
    ea = abi.EnergyArgs(energies[0])
    A, B = oracle_lib.assemble_dense(ga, ea)
    X = np.linalg.solve(A, B.T).T
    assert rel(X, energies[0]["smr"]) < 1e-10


def test_invcomp_against_numpy(oracle_lib):
    rng = np.random.default_rng(5)
    a = rng.standard_normal((40, 40)) + 1j * rng.standard_normal((40, 40))
    assert rel(oracle_lib.invcomp(a), np.linalg.inv(a)) < 1e-11


def test_lorentzian_convolution():
    E = np.linspace(-5, 35, 401)
    out = xanes.lorentzian_convolve(E, np.ones_like(E), 0.8)
    mid = (E > 5) & (E < 25)
    assert np.allclose(out[mid], 1.0, atol=0.05)
    # a single bin is spread as the Lorentzian integral over that bin
    x = np.zeros_like(E)
    x[200] = 1.0
    out = xanes.lorentzian_convolve(E, x, 0.8)
    assert abs(out.sum() * 0.1 / 0.1 - 1.0) < 0.1 and np.argmax(out) == 200
