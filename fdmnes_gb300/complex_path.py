"""Inputs of the complex (Cal_comp) FDM solve: complex harmonics, spin-orbit.

The reference computes in complex arithmetic when the harmonics are complex
(``Ylm_comp``), the energy is complex (``E_comp``) or the basis is not the real
one (``Basereel`` false), ``source/mat.f90:96-104``; spin-orbit forces complex
harmonics (``source/lecture.f90:5401``) and the relativistic terms
(``source/lecture.f90:4923``).  This module builds the ``mat_solve`` arguments
of that case on top of a :class:`cluster.Structure`:

* spin-orbit harmonic tables in ``lmrep``'s order (L, m, spin), C1,
  ``source/general.f90:11227-11330``: every atom and outer harmonic appears
  once per spin, ``nlmsa = 2 (lmax+1)^2``, ``nlmso = 2 (lmaxso+1)^2``;
* ``gradpot``: the centred gradient of Vr on the grid that the relativistic and
  spin-orbit terms of the grid rows use, ``source/potential.f90:5436-5477``;
* complex ``phiato`` (``nphiato7 = 2``): the radial solutions of
  :func:`cluster.boundary_radial` times the complex harmonics of ``Yc``
  (``source/mat.f90:1733-1754``).  With spin-orbit, the solution of atom
  harmonic (L, m, s) has its spin-s component on harmonic m and a model
  coupling on the other spin at m -+ 1 (the m_j = m + 1/2 pairing of
  ``calcMatRow``'s ``m = mato + ispo - isol``, ``source/mat.f90:1289``), of
  relative size ``so_coupling * sqrt((L -+ m)(L +- m + 1)) / (L + 1)``.  The
  reference's coupled radial solver (``Sch_radial`` with spin-orbit,
  ``source/sphere.f90:413``) is upstream of the solve and not restated: these
  are model inputs with the reference's structure.

Energies are real (``E_comp`` false, ``Eimag`` = 0) unless ``eimag_ry`` is
given: the reference's default FDM path zeroes the broadening before the solve
(``source/lecture.f90:5410``).  With ``eimag_ry`` > 0 the outer functions are
the complex-argument j_l, n_l of ``cbessneu`` at k = sqrt(Ecinetic + i Eimag)
(``phiso``, ``source/mat.f90:778-785,978-990``) and the grid diagonal carries
-i Eimag (``E_comp``); ``phiato`` stays the real-energy model unless
``complex_radial`` asks for the radial solutions at the complex energy.  This is the
regular solution; with ``fdm_comp`` phiato also carries an irregular atomic
solution (a free-space model, or the singular radial solver's restatement),
and ``irregular`` builds the arguments of the irregular
cluster solution of the reference's ``FDM_comp`` mode, whose amplitudes and the
regular ones form Tau_RI (``source/mat.f90:219-292``).
"""
from __future__ import annotations

import dataclasses
from typing import Optional

import numpy as np

from . import cluster as CL


def yc(m: int, y1: np.ndarray, y2: np.ndarray) -> np.ndarray:
    """Complex harmonic of order m from the real ones of orders m (y1) and -m (y2)."""
    if m == 0:
        return y1.astype(np.complex128)
    s = 1.0 / np.sqrt(2.0)
    if m < 0:
        return (y2 - 1j * y1) * s
    return (y1 + 1j * y2) * ((-1) ** m) * s


def cbessneu(fnorm: complex, z: np.ndarray, lmax: int):
    """fnorm * j_l(z), fnorm * n_l(z) for complex z by upward recursion
    (source/sphere.f90:7226-7254); z: (n,) -> two (n, lmax + 1) arrays."""
    z = np.asarray(z, dtype=np.complex128)
    bs = np.zeros((len(z), lmax + 1), dtype=np.complex128)
    nm = np.zeros_like(bs)
    nm[:, 0] = -fnorm * np.cos(z) / z
    bs[:, 0] = fnorm * np.sin(z) / z
    if lmax >= 1:
        nm[:, 1] = nm[:, 0] / z - bs[:, 0]
        bs[:, 1] = bs[:, 0] / z + nm[:, 0]
    for L in range(2, lmax + 1):
        nm[:, L] = (2 * L - 1) * nm[:, L - 1] / z - nm[:, L - 2]
        bs[:, L] = (2 * L - 1) * bs[:, L - 1] / z - bs[:, L - 2]
    return bs, nm


def gradpot(st: CL.Structure, cgrad: np.ndarray, ivois: np.ndarray, iord: int = 4) -> np.ndarray:
    """gradvr (npoint, 3, nspin), Fortran order: sum over the axis neighbours of
    cgrad(iv) Vr(j), a neighbour outside the grid counting as the point itself
    (source/potential.f90:5452-5477, cubic grid)."""
    npoint = st.grid.npoint
    nspin = st.Vr.shape[1]
    out = np.zeros((npoint, 3, nspin), order="F")
    pts = np.arange(1, npoint + 1)
    for isp in range(nspin):
        iv = 0
        for _io in range(iord // 2):
            for k in range(3):
                for _s in range(2):
                    iv += 1
                    j = ivois[:npoint, iv - 1].astype(np.int64)
                    j = np.where((j == 0) | (j > npoint), pts, j)
                    out[:, k, isp] += cgrad[iv - 1] * st.Vr[j - 1, isp]
    return out


@dataclasses.dataclass
class SOTables:
    lato: np.ndarray   # (nlmsam, natome)
    mato: np.ndarray
    iato: np.ndarray
    lso: np.ndarray    # (nso1,)
    mso: np.ndarray
    iso: np.ndarray


def so_tables(st: CL.Structure) -> SOTables:
    """lmrep for C1 with nspino = 2: entries (L, m, spin) in that nesting."""
    natome = st.natome
    nlmsam = 2 * st.nlmmax
    lato = np.full((nlmsam, natome), 10000, dtype=np.int32, order="F")
    mato = np.zeros((nlmsam, natome), dtype=np.int32, order="F")
    iato = np.zeros((nlmsam, natome), dtype=np.int32, order="F")
    for ia in range(natome):
        lmax = int(st.lmaxat_max[st.cluster.itype[ia]])
        k = 0
        for L in range(lmax + 1):
            for m in range(-L, L + 1):
                for s in (1, 2):
                    lato[k, ia], mato[k, ia], iato[k, ia] = L, m, s
                    k += 1
    n = 2 * st.nlmomax
    lso = np.zeros(n, dtype=np.int32)
    mso = np.zeros(n, dtype=np.int32)
    iso = np.zeros(n, dtype=np.int32)
    k = 0
    for L in range(st.lmaxso_max + 1):
        for m in range(-L, L + 1):
            for s in (1, 2):
                lso[k], mso[k], iso[k] = L, m, s
                k += 1
    return SOTables(lato, mato, iato, lso, mso, iso)


def grid_dict(st: CL.Structure, spinorbit: bool) -> dict:
    """Energy-independent arguments; with spin-orbit nspino = 2 and its tables."""
    from . import abi
    d = abi.grid_dict(st)
    if spinorbit:
        if st.nspin != 2:
            raise ValueError("spin-orbit needs a structure with nspin = 2")
        t = so_tables(st)
        d.update(nspino=2, nlmsam=t.lato.shape[0], nso1=t.lso.shape[0], lato=t.lato, mato=t.mato, iato=t.iato,
                 lso=t.lso, mso=t.mso, iso=t.iso, Kar=np.ones((64, 2), order="F"), Kari=np.zeros((64, 2), order="F"))
    return d


def _so_weight(L: int, m: int, isol: int, ispo: int, so_coupling: float) -> float:
    if ispo == isol:
        return 1.0
    if isol == 1:      # spin 1 at m, spin 2 at m + 1
        return so_coupling * np.sqrt(max((L - m) * (L + m + 1), 0)) / (L + 1)
    return so_coupling * np.sqrt(max((L + m) * (L - m + 1), 0)) / (L + 1)


def irregular_boundary_radial(st: CL.Structure, enervide: float, lmaxa: np.ndarray) -> dict:
    """Model irregular atomic solutions at every atom's boundary points, keyed
    like :func:`cluster.boundary_radial`: the free-space singular solution
    -sqrt(k / pi) n_l(k r) at the kinetic energy of the spin block, r the
    distance of the boundary point to its atom.  The reference's singular
    radial solver (``Sch_radial_solsing``, ``source/sphere.f90:2591``) is
    upstream of the solve; this is a model input with its structure."""
    g = st.grid
    out = {}
    for isp in range(1, st.nspin + 1):
        k = np.sqrt(enervide - (st.V0bd + st.spin_shift(isp)))
        fn = np.sqrt(k / np.pi)
        for ia in range(st.natome):
            nb = int(g.nbord[ia])
            _, nm = cbessneu(fn, k * st.rrel[:nb, ia], int(lmaxa[ia]))
            for L in range(int(lmaxa[ia]) + 1):
                out[(isp, ia, L)] = -nm[:, L].real
    return out


def sch_radial_singular(r: np.ndarray, V: np.ndarray, enervide: float, eimag: float, k: complex, L: int,
                        i0: int) -> np.ndarray:
    """Singular radial solution R_L(r) = us_L(r) / r on mesh r, complex
    (source/sphere.f90:2591-2812 with Classic_irreg, scalar potential, no
    spin-orbit, no Hubbard term): us = -i r h_L(k r), h_L = sqrt(k/pi)
    (j_L + i n_L), from mesh index i0 outward, then the three-point recursion
    of the regular solver (:324-396) run inward, with -i Eimag on the diagonal
    for complex energies (:2752)."""
    nr = len(r)
    rp = np.empty(nr)
    rm = np.empty(nr)
    rp[:-1] = r[1:]
    rp[-1] = r[-1] ** 2 / r[-2]
    rm[1:] = r[:-1]
    rm[0] = r[0] ** 2 / r[1]
    dr = 0.5 * (rp - rm)
    claplm = 1.0 / ((r - rm) * dr)
    claplp = 1.0 / ((rp - r) * dr)
    g0 = (claplm + claplp) + (V - enervide)
    gm = -claplm
    gp = -claplp
    f2 = 1.0 / r ** 2
    us = np.zeros(nr, dtype=np.complex128)
    bs, nm = cbessneu(np.sqrt(k / np.pi), k * r[i0:], L)
    us[i0:] = -1j * r[i0:] * (bs[:, L] + 1j * nm[:, L])
    L2 = L * (L + 1)
    for ir in range(i0, 0, -1):
        td = g0[ir] + L2 * f2[ir]
        v = td * us[ir] + gp[ir] * us[ir + 1]
        if eimag != 0.0:
            v = v - 1j * eimag * us[ir]
        us[ir - 1] = -v / gm[ir]
    return us / r


def singular_boundary_radial(st: CL.Structure, enervide: float, lmaxa: np.ndarray, eimag: float = 0.0) -> dict:
    """Irregular atomic solutions at every atom's boundary points from the
    singular radial solver (:func:`sch_radial_singular`, started at the atom
    type's radius rmtg, or at the end of its radial mesh if that is shorter)
    and the quadratic interpolation of cal_phiato (source/sphere.f90:3186-3370),
    keyed like :func:`cluster.boundary_radial`."""
    cl, g = st.cluster, st.grid
    out = {}
    cache = {}
    for isp in range(1, st.nspin + 1):
        dvs = st.spin_shift(isp)
        k = np.sqrt(complex(enervide - (st.V0bd + dvs), eimag))
        for ia in range(cl.natome):
            ipr = int(cl.itype[ia])
            r = st.radial_r[ipr]
            i0 = min(int(np.searchsorted(r, cl.rmtg[ipr])), len(r) - 2)
            nb = int(g.nbord[ia])
            rr = st.rrel[:nb, ia]
            idx = np.clip(np.searchsorted(r, rr, side="right"), 2, len(r) - 1)
            for L in range(int(lmaxa[ia]) + 1):
                key = (isp, ipr, L)
                if key not in cache:
                    cache[key] = sch_radial_singular(r, st.radial_V[ipr] + dvs, enervide, eimag, k, L, i0)
                u = cache[key]
                out[(isp, ia, L)] = CL.f_interp2(rr, r[idx - 2], r[idx - 1], r[idx], u[idx - 2], u[idx - 1], u[idx])
    return out


def energy_dict(st: CL.Structure, energy_ev: float, spinorbit: bool, ylm_comp: bool = True,
                relativistic: Optional[bool] = None, so_coupling: float = 0.1, basereel: bool = False,
                gradvr: Optional[np.ndarray] = None, e_fermi_ev: float = -5.0, eimag_ry: float = 0.0,
                fdm_comp: bool = False, irregular: bool = False, irregular_radial: str = "free",
                complex_radial: bool = False) -> dict:
    """Per-energy arguments of one complex mat_solve call.

    spinorbit: nspino = 2 (needs nspin = 2), with the relativistic terms unless
    ``relativistic`` says otherwise.  ylm_comp: complex harmonics (forced with
    spin-orbit in the reference).  basereel: real outer basis (the reference
    never combines it with complex harmonics; kept for the reduction tests).
    fdm_comp: the reference's FDM_comp mode (``source/fdm.f90:1734-1738``):
    phiato carries the regular and the irregular atomic solutions (n_RI = 2);
    irregular (implies fdm_comp, needs eimag_ry > 0): the irregular cluster
    solution with both atomic solutions (Test_reg = 0, n_ato_RI = 2,
    ``source/mat.f90:138-147``) instead of the regular one.
    irregular_radial: the irregular atomic solution, "free" (the free-space
    model of :func:`irregular_boundary_radial`) or "singular" (the singular
    radial solver through the atom's potential, :func:`singular_boundary_radial`).
    complex_radial: at a complex energy, the regular atomic solution of the
    radial equation at that energy (complex, as the reference's Sphere with
    Ecomp computes it) instead of the real-energy one.
    """
    from . import abi
    g = st.grid
    if irregular:
        fdm_comp = True
        if eimag_ry <= 0.0:
            raise ValueError("the irregular solution is the complex-energy (FDM_comp) one: eimag_ry > 0")
    ei = CL.energy_inputs(st, energy_ev, e_fermi_ev)
    if relativistic is None:
        relativistic = spinorbit
    nspino = 2 if spinorbit else 1
    nlmsa = (nspino * (ei.lmaxa + 1) ** 2).astype(np.int32)
    nlmso = nspino * (ei.lmaxso + 1) ** 2
    ri = CL.newind(st, nlmsa, nlmso, nspino, irregular=irregular)
    nspinp = st.nspin
    n_ri = 2 if fdm_comp else 1
    rads = [CL.boundary_radial(st, ei.enervide, ei.lmaxa, eimag_ry if complex_radial else 0.0)]
    if fdm_comp:
        if irregular_radial == "singular":
            rads.append(singular_boundary_radial(st, ei.enervide, ei.lmaxa, eimag_ry))
        elif irregular_radial == "free":
            rads.append(irregular_boundary_radial(st, ei.enervide, ei.lmaxa))
        else:
            raise ValueError("irregular_radial is 'free' or 'singular'")
    phi = np.zeros((g.nbtm, ei.nlmagm, nspinp, nspino, n_ri, st.natome, 2), order="F")

    def harmonic(ia, nb, L, m):
        lm = L * L + L + m
        if ylm_comp:
            return yc(m, st.Ylmato[:nb, lm, ia], st.Ylmato[:nb, lm - 2 * m, ia])
        return st.Ylmato[:nb, lm, ia].astype(np.complex128)

    for ia in range(st.natome):
        nb = int(g.nbord[ia])
        for L in range(int(ei.lmaxa[ia]) + 1):
            for m in range(-L, L + 1):
                for isol in range(1, nspino + 1):
                    for ispo in range(1, nspino + 1):
                        mr = m + ispo - isol
                        if abs(mr) > L:
                            continue
                        w = _so_weight(L, m, isol, ispo, so_coupling) if spinorbit else 1.0
                        for isp in range(1, nspinp + 1):
                            # spin-orbit: the spin index of phiato is the component ispo
                            if spinorbit and isp != ispo:
                                continue
                            for iri, rad in enumerate(rads):
                                u = rad[(isp, ia, L)]
                                v = w * u * harmonic(ia, nb, L, mr)
                                lm0 = L * L + L + mr
                                phi[:nb, lm0, isp - 1, isol - 1, iri, ia, 0] = v.real
                                phi[:nb, lm0, isp - 1, isol - 1, iri, ia, 1] = v.imag
    nspinr = st.nspin if spinorbit else 1
    bes = np.asfortranarray(np.repeat(ei.besselr, nspinr, axis=2))
    neu = np.asfortranarray(np.repeat(ei.neumanr, nspinr, axis=2))
    ecomp = {}
    if eimag_ry > 0.0:
        # phiso with E_comp: k = sqrt(Ecinetic + i Eimag), fnorm = sqrt(k / pi)
        konde = np.sqrt(complex(ei.ecinetic_out, eimag_ry))
        fnormc = np.sqrt(konde / np.pi)
        zc = konde * g.xyz[3, g.isrt - 1]
        bc, nc = cbessneu(fnormc, zc, ei.lmaxso)
        arrs = []
        for a in (bc, nc):
            out = np.zeros((2, g.nsort, ei.lmaxso + 1, nspinr), order="F")
            for isp in range(nspinr):
                out[0, :, :, isp] = a.real
                out[1, :, :, isp] = a.imag
            arrs.append(out)
        ecomp = dict(E_comp=1, Eimag=eimag_ry, nsort_c=g.nsort, nsort_r=0, Bessel=arrs[0], Neuman=arrs[1],
                     Besselr=None, Neumanr=None)
    if gradvr is None:
        gradvr = gradpot(st, g.cgrad, g.ivois)
    d = abi.energy_dict(st, ei, ri)
    d.update(nlmso=nlmso, nligne=ri.nligne, nligneso=ri.nligneso, nlmsa=nlmsa, nphiato7=2, nspinp=nspinp,
             nspinr=nspinr, nicm=g.npoint, Cal_comp=1, E_comp=0, Basereel=int(basereel), Relativiste=int(relativistic),
             Spinorbite=int(spinorbit), Ylm_comp=int(ylm_comp), ispin=1, phiato=phi, Besselr=bes, Neumanr=neu,
             gradvr=np.asfortranarray(gradvr), new_=ri.new, newinv=ri.newinv, lb1=ri.lb1, lb2=ri.lb2, ianew=ri.ianew)
    d.update(ecomp)
    d.update(n_RI=n_ri, n_ato_RI=2 if irregular else 1, irregular=int(irregular), Test_reg=0)
    return d


def pt_so_structure(rsort_ang: float = 1.6, adimp_ang: float = 0.25, e_max_ev: float = 35.0) -> CL.Structure:
    """Small Pt L-edge-like case for the complex path: the absorber alone inside a
    1.6 A sphere, two spin blocks of one non-magnetic potential."""
    return CL.build_structure(CL.pt_cluster(0.5), adimp_ang, rsort_ang, e_max_ev, nspin=2)
