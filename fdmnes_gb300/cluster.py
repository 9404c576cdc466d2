"""Synthetic cluster, FDM grid and per-energy inputs of the FDM solve.

This module produces every array that the reference's ``mat_solve``
(``source/mat_solve_gaussian.f90:5``) receives, for a cluster without
symmetry reduction (point group C1, one representation, cubic grid, 4th-order
stencil).  It stands in for the reference's upstream producers so that the
GPU solve can be driven without the Fortran host:

* cluster and grid      ``reseau``  source/general.f90:9439-9680
* stencil + neighbours  ``laplac``  source/general.f90:9732-9888
* boundary points       ``bordure`` source/general.f90:9895-10136
* real harmonics        ``Ylmpt``/``cylm``/``ylmcr`` source/general.f90:11505-11725
* l cut-offs            ``clmax``   source/general.f90:11445-11503
* harmonic tables       ``lmrep``   source/general.f90:11227-11340 (C1: all L,m)
* radial solutions      ``coef_sch_rad``/``Sch_radial`` source/sphere.f90:324-733
* boundary functions    ``cal_phiato`` source/sphere.f90:3186-3370, ``f_interp2`` source/tools.f90:504
* row numbering         ``newind``  source/mat.f90:1761-1921
* outer Bessel/Neumann  ``phiso``/``cbessneur`` source/mat.f90:739-1028, source/sphere.f90:7356

The potential is a model (the reference's self-consistent ``potex`` is out of
scope): a superposition of Thomas-Fermi screened Coulomb potentials, shifted
so that the interstitial average equals a stated constant.

All quantities are in the reference's internal units: lengths in bohr,
energies in Rydberg.  Index-valued arrays hold 1-based Fortran indices and
every array is Fortran-ordered with the reference's shape, so that its memory
is exactly what the Fortran caller would pass through the C-ABI.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, List, Optional, Sequence

import numpy as np

# Physical constants (source/main.f90:55-84)
BOHR = 0.52917721067
RYDB = 13.605693009
ALFA_SF = 0.0072973525664
EPS4 = 1e-4
EPS6 = 1e-6
EPS10 = 1e-10
EPSPOS = 1e-4
SQRT_2 = math.sqrt(2.0)
QUATRE_PI = 4.0 * math.pi

F = dict(order="F")


def _f64(shape):
    return np.zeros(shape, dtype=np.float64, order="F")


def _i32(shape):
    return np.zeros(shape, dtype=np.int32, order="F")


# ---------------------------------------------------------------------------
# Crystal clusters
# ---------------------------------------------------------------------------

@dataclasses.dataclass
class Cluster:
    """Atoms of the calculation cluster, absorber first, sorted by distance."""
    name: str
    pos: np.ndarray          # (3, natome) bohr, absorber at the origin
    Z: np.ndarray            # (natome,) atomic numbers
    itype: np.ndarray        # (natome,) prototype index: 0 = absorber, >=1 others
    rmt: np.ndarray          # (ntype_proto,) FDM atom radius (bohr) per prototype
    rmtg: np.ndarray         # (ntype_proto,) radius used by clmax (bohr) per prototype
    zproto: np.ndarray       # (ntype_proto,) Z per prototype
    pot_atoms: np.ndarray    # (3, nall) bohr: all atoms used to superpose the potential
    pot_Z: np.ndarray        # (nall,)
    pot_zeff: np.ndarray     # (nall,) Z used in the screened Coulomb (Z+1 on the absorber)

    @property
    def natome(self) -> int:
        return self.pos.shape[1]


def _fdm_rmt_angstrom(Z: int) -> float:
    """FDM atom radius: 1.0 A for Z > 21, linear down to 0.3 A for H.

    Follows the default of source/lecture.f90:7072-7106 in its simple form.
    """
    if Z > 21:
        return 1.0
    return 0.3 + (1.0 - 0.3) * (Z - 1) / 20.0


def fcc_cluster(name: str, a_ang: float, Z: int, r_cluster_ang: float,
                r_pot_ang: float, rmtg_ang: float) -> Cluster:
    """fcc crystal cluster centred on an atom (the absorber)."""
    n = int(math.ceil(r_pot_ang / a_ang)) + 1
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    pts = []
    for ix in range(-n, n + 1):
        for iy in range(-n, n + 1):
            for iz in range(-n, n + 1):
                for b in basis:
                    p = (np.array([ix, iy, iz]) + b) * a_ang
                    pts.append(p)
    pts = np.array(pts)
    d = np.sqrt((pts ** 2).sum(1))
    order = np.lexsort((pts[:, 2], pts[:, 1], pts[:, 0], np.round(d, 6)))
    pts, d = pts[order], d[order]
    sel = d <= r_cluster_ang + 1e-6
    allp = pts[d <= r_pot_ang + 1e-6]
    pos = pts[sel].T / BOHR
    natome = pos.shape[1]
    itype = np.ones(natome, dtype=np.int32)
    itype[0] = 0
    rmt = np.array([_fdm_rmt_angstrom(Z)] * 2) / BOHR
    rmtg = np.array([rmtg_ang] * 2) / BOHR
    zproto = np.array([Z, Z])
    zeff = np.full(allp.shape[0], float(Z))
    zeff[0] = Z + 1.0  # Z+1 model of the core hole on the absorber
    return Cluster(name=name, pos=np.asfortranarray(pos), Z=np.full(natome, Z), itype=itype,
                   rmt=rmt, rmtg=rmtg, zproto=zproto,
                   pot_atoms=allp.T / BOHR, pot_Z=np.full(allp.shape[0], Z), pot_zeff=zeff)


def rutile_cluster(r_cluster_ang: float, a_ang: float = 4.594, c_ang: float = 2.959, u: float = 0.305,
                   r_pot_ang: float = 8.0) -> Cluster:
    """Rutile TiO2 (P4_2/mnm) cluster centred on a Ti absorber.

    Ti at (0,0,0) and (1/2,1/2,1/2); O at (u,u,0), (-u,-u,0), (1/2+u,1/2-u,1/2),
    (1/2-u,1/2+u,1/2).  Prototypes: 0 = Ti absorber, 1 = Ti, 2 = O.
    """
    basis = [(22, (0.0, 0.0, 0.0)), (22, (0.5, 0.5, 0.5)),
             (8, (u, u, 0.0)), (8, (-u, -u, 0.0)), (8, (0.5 + u, 0.5 - u, 0.5)), (8, (0.5 - u, 0.5 + u, 0.5))]
    na = int(math.ceil(r_pot_ang / a_ang)) + 1
    nc = int(math.ceil(r_pot_ang / c_ang)) + 1
    pts, zs = [], []
    for ix in range(-na, na + 1):
        for iy in range(-na, na + 1):
            for iz in range(-nc, nc + 1):
                for Z, (bx, by, bz) in basis:
                    pts.append(((ix + bx) * a_ang, (iy + by) * a_ang, (iz + bz) * c_ang))
                    zs.append(Z)
    pts = np.array(pts)
    zs = np.array(zs)
    d = np.sqrt((pts ** 2).sum(1))
    order = np.lexsort((pts[:, 2], pts[:, 1], pts[:, 0], np.round(d, 6)))
    pts, zs, d = pts[order], zs[order], d[order]
    sel = d <= r_cluster_ang + 1e-6
    allsel = d <= r_pot_ang + 1e-6
    pos = pts[sel].T / BOHR
    Zc = zs[sel]
    itype = np.where(Zc == 22, 1, 2).astype(np.int32)
    itype[0] = 0
    zproto = np.array([22, 22, 8])
    rmt = np.array([_fdm_rmt_angstrom(int(z)) for z in zproto]) / BOHR
    rmtg = np.array([1.04, 1.04, 0.91]) / BOHR
    allp, allz = pts[allsel], zs[allsel]
    zeff = allz.astype(np.float64)
    zeff[0] = allz[0] + 1.0  # Z+1 model of the core hole on the absorber
    return Cluster(name="TiO2", pos=np.asfortranarray(pos), Z=Zc, itype=itype, rmt=rmt, rmtg=rmtg,
                   zproto=zproto, pot_atoms=allp.T / BOHR, pot_Z=allz, pot_zeff=zeff)


def move_shell(cl: Cluster, shell_radius_ang: float, delta_ang: float, tol_ang: float = 0.01) -> Cluster:
    """The cluster with every atom at distance shell_radius_ang (+- tol) from the
    absorber moved radially by delta_ang, in the cluster and in the atoms that
    build the potential."""
    def moved(pos):
        out = np.array(pos, dtype=np.float64, copy=True)
        d = np.sqrt((out ** 2).sum(0))
        sel = np.abs(d * BOHR - shell_radius_ang) < tol_ang
        out[:, sel] *= (d[sel] + delta_ang / BOHR) / d[sel]
        return out
    return dataclasses.replace(cl, pos=np.asfortranarray(moved(cl.pos)), pot_atoms=moved(cl.pot_atoms))


def cu_cluster(r_cluster_ang: float = 2.6) -> Cluster:
    """fcc Cu, a = 3.61 A, absorber at the origin (13 atoms within 2.6 A)."""
    return fcc_cluster("Cu", 3.61, 29, r_cluster_ang, r_pot_ang=8.0, rmtg_ang=1.28)


def pt_cluster(r_cluster_ang: float = 4.0) -> Cluster:
    """fcc Pt, a = 3.92 A."""
    return fcc_cluster("Pt", 3.92, 78, r_cluster_ang, r_pot_ang=8.0, rmtg_ang=1.39)


# ---------------------------------------------------------------------------
# Model potential
# ---------------------------------------------------------------------------

def _screened_coulomb(r, zeff):
    """Thomas-Fermi screened Coulomb potential in Ry, r in bohr."""
    a_tf = 0.8853 / zeff ** (1.0 / 3.0)
    rr = np.maximum(r, 1e-8)
    return -2.0 * zeff / rr * np.exp(-rr / (2.0 * a_tf))


# ---------------------------------------------------------------------------
# Grid (reseau + laplac + bordure) for C1 and a cubic lattice
# ---------------------------------------------------------------------------

@dataclasses.dataclass
class Grid:
    adimp: float
    rsort: float
    iord: int
    nvois: int
    npoint: int
    npso: int
    npr: int
    indice: np.ndarray     # (npso, 3) int
    xyz: np.ndarray        # (4, npso) F
    numia: np.ndarray      # (npso,) int32
    rvol: np.ndarray       # (npoint,)
    clapl: np.ndarray      # (0:nvois)
    cgrad: np.ndarray      # (nvois,)
    ivois: np.ndarray      # (npso, nvois) F, 1-based
    isvois: np.ndarray     # (npso, nvois) F
    nbord: np.ndarray      # (natome,)
    nbordf: np.ndarray
    ibord: np.ndarray      # (nbtm, natome) F, 1-based
    isbord: np.ndarray
    poidsa: np.ndarray     # (nbm, natome) F
    nsort: int
    nsortf: int
    isrt: np.ndarray       # (nsort,) 1-based
    poidso: np.ndarray     # (nsortf,)

    @property
    def nbtm(self) -> int:
        return self.ibord.shape[0]

    @property
    def nbm(self) -> int:
        return self.poidsa.shape[0]


def _exchange_sort(key: np.ndarray) -> np.ndarray:
    """Permutation produced by the exchange sort of source/general.f90:9529-9543.

    For each position i, every later position j whose key is strictly smaller
    than the current key at i is swapped with i.  ``key`` holds the squared
    integer distance, which is exactly ordered (radii of distinct classes differ
    by far more than ``epspos``).  The swap chain of one i is a rotation through
    the successive strict running minima of the suffix, which is applied here
    with one vectorised scan per position.
    """
    a = key.astype(np.int64).copy()
    perm = np.arange(len(a))
    n = len(a)
    for i in range(n - 1):
        s = a[i + 1:]
        c0 = a[i]
        run = np.minimum.accumulate(s)
        before = np.empty_like(run)
        before[0] = c0
        if len(run) > 1:
            before[1:] = np.minimum(run[:-1], c0)
        hits = np.nonzero(s < before)[0]
        if hits.size == 0:
            continue
        pos = hits + i + 1
        chain = np.concatenate(([i], pos))
        # value at i moves to pos[0], value at pos[k] moves to pos[k+1], last goes to i
        vals = a[chain].copy()
        pv = perm[chain].copy()
        a[chain[1:]] = vals[:-1]
        perm[chain[1:]] = pv[:-1]
        a[i] = vals[-1]
        perm[i] = pv[-1]
    return perm


def build_grid(cl: Cluster, adimp_ang: float, rsort_ang: float, iord: int = 4) -> Grid:
    """Grid points, stencil, neighbours and boundary tables (C1, cubic)."""
    adimp = adimp_ang / BOHR
    rsort = rsort_ang / BOHR
    nvois = 3 * iord
    # nbpoint/reseau: radius of kept points in grid units
    rmax = rsort / adimp + SQRT_2 * iord / 2 + EPSPOS
    nx = int(math.ceil(rmax)) + 1
    r = np.arange(-nx, nx + 1)
    IX, IY, IZ = np.meshgrid(r, r, r, indexing="ij")
    IX, IY, IZ = IX.ravel(), IY.ravel(), IZ.ravel()
    n2 = IX * IX + IY * IY + IZ * IZ
    dist = np.sqrt(n2.astype(np.float64))
    keep = dist <= rmax  # loop order ix, iy, iz as in the reference (C order here)
    IX, IY, IZ, n2, dist = IX[keep], IY[keep], IZ[keep], n2[keep], dist[keep]
    perm = _exchange_sort(n2)
    IX, IY, IZ, dist = IX[perm], IY[perm], IZ[perm], dist[perm]
    npso = len(IX)
    indice = np.stack([IX, IY, IZ], axis=1).astype(np.int32)
    xyz = _f64((4, npso))
    xyz[0], xyz[1], xyz[2] = IX * adimp, IY * adimp, IZ * adimp
    xyz[3] = adimp * dist
    inside = xyz[3] > rsort + EPSPOS
    npoint = int(np.argmax(inside)) if inside.any() else npso
    numia = np.zeros(npso, dtype=np.int32)
    numia[npoint:] = -2
    # atoms: posrel in C1 is the plain distance; the last atom wins
    for ia in range(cl.natome):
        it = cl.itype[ia]
        d = np.sqrt(((xyz[:3, :npoint] - cl.pos[:, ia:ia + 1]) ** 2).sum(0))
        numia[:npoint][d < cl.rmt[it] + EPSPOS] = ia + 1
    npr = int((numia[:npoint] == 0).sum())
    # rvol: C1 maps each point onto itself once; normalised by the max (=1)
    rvol = np.ones(npoint, dtype=np.float64)

    # laplac: coefficients
    ad2 = adimp ** 2
    coeford = [1.0, 0.0]
    if iord == 2:
        cl_ = 1.0 / ad2
    else:
        cl_ = (4.0 / 3.0) / ad2
        coeford[1] = -1.0 / 16
    clapl = np.zeros(nvois + 1)
    indpro = np.zeros((nvois + 1, 3), dtype=np.int32)
    iv = 0
    for io in range(1, iord // 2 + 1):
        for i in range(3):
            for s in (-1, 1):
                iv += 1
                clapl[iv] = coeford[io - 1] * cl_
                indpro[iv, i] = s * io
    clapl[0] = -clapl[1:].sum()
    coeford = [1.0, 0.0]
    if iord == 2:
        cd = 1.0 / (2 * adimp)
    else:
        cd = (4.0 / 3.0) / (2 * adimp)
        coeford[1] = -1.0 / 8
    cgrad = np.zeros(nvois)
    iv = 0
    for io in range(1, iord // 2 + 1):
        for i in range(3):
            for s in (-1, 1):
                cgrad[iv] = s * coeford[io - 1] * cd
                iv += 1
    # neighbour table via mpres lookup
    mpres = np.zeros((2 * nx + 1,) * 3, dtype=np.int64)
    mpres[IX + nx, IY + nx, IZ + nx] = np.arange(1, npso + 1)
    ivois = _i32((npso, nvois))
    isvois = _i32((npso, nvois))
    for iv in range(1, nvois + 1):
        la = indice + indpro[iv][None, :]
        ok = (np.abs(la) <= nx).all(1)
        j = np.zeros(npso, dtype=np.int64)
        j[ok] = mpres[la[ok, 0] + nx, la[ok, 1] + nx, la[ok, 2] + nx]
        ivois[:, iv - 1] = j
        isvois[:, iv - 1] = np.where(ok, 1, 0)

    # bordure (C1, not Green)
    natome = cl.natome
    nv = 2 * nvois // iord
    ibord_l: List[List[int]] = [[] for _ in range(natome)]
    isrt_l: List[int] = []
    pdsort = 0.0
    pdharm = np.zeros(natome)
    iss = 0
    ibp = np.zeros(natome, dtype=np.int64)
    for i in range(1, npoint + 1):
        if numia[i - 1] != 0:
            continue
        for iv in range(1, nv + 1):
            j = ivois[i - 1, iv - 1]
            if j == 0:
                continue
            ia = numia[j - 1]
            if ia == -2:
                if iss != i:
                    pdsort += rvol[i - 1]
                    isrt_l.append(i)
                iss = i
            elif ia > 0:
                if ibp[ia - 1] != i:
                    pdharm[ia - 1] += rvol[i - 1]
                    ibord_l[ia - 1].append(i)
                ibp[ia - 1] = i
    nbordf = np.array([len(b) for b in ibord_l], dtype=np.int32)
    for i in range(1, npoint + 1):
        ia = numia[i - 1]
        if ia < 1:
            continue
        for iv in range(1, nvois + 1):
            j = ivois[i - 1, iv - 1]
            if j == 0:
                raise RuntimeError("bordure: neighbour outside the grid box")
            if numia[j - 1] != 0:
                continue
            ibord_l[ia - 1].append(i)
            break
    nbord = np.array([len(b) for b in ibord_l], dtype=np.int32)
    nsortf = len(isrt_l)
    for i in range(npoint + 1, npso + 1):
        for iv in range(1, nvois + 1):
            j = ivois[i - 1, iv - 1]
            if j == 0:
                continue
            if numia[j - 1] != 0:
                continue
            isrt_l.append(i)
            break
    nsort = len(isrt_l)
    nbtm = max(1, int(nbord.max()))
    nbm = max(1, int(nbordf.max()))
    ibord = _i32((nbtm, natome))
    isbord = _i32((nbtm, natome))
    poidsa = _f64((nbm, natome))
    for ia in range(natome):
        nb = len(ibord_l[ia])
        ibord[:nb, ia] = ibord_l[ia]
        isbord[:nb, ia] = 1
        if nbordf[ia] > 0:
            fac = QUATRE_PI / pdharm[ia]
            idx = np.array(ibord_l[ia][:nbordf[ia]]) - 1
            poidsa[:nbordf[ia], ia] = fac * rvol[idx]
    isrt = np.array(isrt_l, dtype=np.int32)
    poidso = np.zeros(max(nsortf, 1))
    if nsortf > 0:
        poidso[:nsortf] = QUATRE_PI / pdsort * rvol[isrt[:nsortf] - 1]
    return Grid(adimp=adimp, rsort=rsort, iord=iord, nvois=nvois, npoint=npoint, npso=npso, npr=npr,
                indice=indice, xyz=xyz, numia=numia, rvol=rvol, clapl=clapl, cgrad=cgrad,
                ivois=ivois, isvois=isvois, nbord=nbord, nbordf=nbordf, ibord=ibord, isbord=isbord,
                poidsa=poidsa, nsort=nsort, nsortf=nsortf, isrt=isrt, poidso=poidso)


# ---------------------------------------------------------------------------
# Harmonics (cylm + ylmcr), vectorised over points
# ---------------------------------------------------------------------------

def cylm(lmax: int, v: np.ndarray, r: np.ndarray) -> np.ndarray:
    """Complex Y_lm, m >= 0, index L(L+1)/2 + m (0-based): source/general.f90:11611-11690.

    v: (3, n), r: (n,).  Returns (nlmc, n) complex.
    """
    n = v.shape[1]
    nlmc = (lmax + 1) * (lmax + 2) // 2
    Y = np.zeros((nlmc, n), dtype=np.complex128)
    cos_t = np.where(r > EPS6, v[2] / np.where(r > EPS6, r, 1.0), 1.0)
    den = np.sqrt(v[0] ** 2 + v[1] ** 2)
    big = den > EPS6
    dsafe = np.where(big, den, 1.0)
    rsafe = np.where(r > 0, r, 1.0)
    exphi = np.where(big, (v[0] + 1j * v[1]) / dsafe, 1.0 + 0j)
    sin_t = np.where(big, np.sqrt(np.maximum(1 - cos_t ** 2, 0.0)), 0.0)
    ste = np.where(big, (v[0] + 1j * v[1]) / rsafe, 0.0 + 0j)
    cot_t = np.where(big, cos_t / np.where(sin_t != 0, sin_t, 1.0), 0.0)
    Y[0] = 1.0 / math.sqrt(QUATRE_PI)
    for L in range(1, lmax + 1):
        lm = (L + 1) * (L + 2) // 2 - 1
        lm1 = L * (L + 1) // 2 - 1
        f = -math.sqrt(1 + 0.5 / L)
        Y[lm] = f * ste * Y[lm1]
    if lmax > 0:
        Y[1] = math.sqrt(3.0 / QUATRE_PI) * cos_t
    for L in range(2, lmax + 1):
        lm = (L + 1) * (L + 2) // 2 - 2
        lm1 = (L * L + L) // 2 - 2
        f = -math.sqrt((2 * L + 1.0) / (2 * L - 2))
        Y[lm] = f * ste * Y[lm1]
    exphi_c = np.conj(exphi)
    for L in range(2, lmax + 1):
        lm0 = (L * L + L) // 2
        for m in range(L - 2, 0, -1):
            lm = lm0 + m  # 0-based of (lm0 + m + 1)
            f = -2 * (m + 1.0) / math.sqrt(L * (L + 1.0) - m * (m + 1.0))
            g = -math.sqrt((L * (L + 1.0) - (m + 1.0) * (m + 2.0)) / (L * (L + 1.0) - m * (m + 1.0)))
            val = exphi_c * (cot_t * f * Y[lm + 1] + exphi_c * g * Y[lm + 2])
            Y[lm] = np.where(np.abs(sin_t) > EPS10, val, 0.0)
    for L in range(2, lmax + 1):
        lm = L * (L + 1) // 2
        lm1 = (L - 1) * L // 2
        lm2 = (L - 2) * (L - 1) // 2
        f = math.sqrt((2 * L + 1.0) / (2 * L - 1.0)) * (2 * L - 1.0) / L
        g = -math.sqrt((2 * L + 1.0) / (2 * L - 3.0)) * (L - 1.0) / L
        Y[lm] = f * cos_t * Y[lm1] + g * Y[lm2]
    return Y


def ylmcr(lmax: int, Yc: np.ndarray) -> np.ndarray:
    """Real harmonics, index L^2+L+m (0-based): source/general.f90:11696-11725."""
    nlmr = (lmax + 1) ** 2
    Yr = np.zeros((nlmr, Yc.shape[1]))
    lm = 0
    for L in range(lmax + 1):
        l2 = (L * L + L) // 2
        for m in range(-L, L + 1):
            c = Yc[l2 + abs(m)]
            if m < 0:
                Yr[lm] = (-1) ** m * SQRT_2 * c.imag
            elif m == 0:
                Yr[lm] = c.real
            else:
                Yr[lm] = (-1) ** m * SQRT_2 * c.real
            lm += 1
    return Yr


def real_ylm(lmax: int, v: np.ndarray) -> np.ndarray:
    r = np.sqrt((v ** 2).sum(0))
    return ylmcr(lmax, cylm(lmax, v, r))


# ---------------------------------------------------------------------------
# clmax (source/general.f90:11445-11503)
# ---------------------------------------------------------------------------

def clmax(energ: float, R: float, lmax0: int, Z: int, lmaxfree: bool) -> int:
    kR = math.sqrt(energ) * R if (energ > 0 and R > EPS10) else 0.0
    base = int(0.5 + 0.5 * math.sqrt(1 + 4 * kR * kR))
    if lmax0 < 0:
        lmax = base - lmax0
    elif Z < 0:
        lmax = lmax0
    else:
        lmax = base + 1
    if Z < 0:
        lmax = max(1, lmax)
    elif Z == 1:
        lmax = 2
    elif Z == 0 or (1 < Z <= 54):
        lmax = max(2, lmax)
    elif Z > 54:
        lmax = max(3, lmax)
    if not lmaxfree:
        if 0 < Z < 3:
            lmax = min(lmax, 3)
        elif Z < 19:
            lmax = min(lmax, 4)
        elif Z < 37:
            lmax = min(lmax, 5)
        elif Z < 55:
            lmax = min(lmax, 6)
        elif Z < 87:
            lmax = min(lmax, 7)
        else:
            lmax = min(lmax, 8)
    if lmax0 >= 0:
        lmax = min(lmax, lmax0)
    return lmax


# ---------------------------------------------------------------------------
# Radial solutions (coef_sch_rad + Sch_radial, non-relativistic, no spin-orbit)
# ---------------------------------------------------------------------------

def radial_mesh(Z: int, rmax: float, n_per_decade: int = 120) -> np.ndarray:
    """Logarithmic radial mesh from 1e-4/Z bohr out to rmax (bohr)."""
    r0 = 1e-4 / Z
    nr = int(math.ceil(math.log10(rmax / r0) * n_per_decade)) + 3
    return r0 * 10.0 ** (np.arange(nr) / n_per_decade)


def sch_radial(r: np.ndarray, V: np.ndarray, enervide: float, ecinetic: float, L: int, Z: float,
               eimag: float = 0.0) -> np.ndarray:
    """Regular radial solution R_L(r) = u_L(r)/r on mesh r.

    Three-point finite-difference recursion of source/sphere.f90:324-396
    (coefficients) and :583-695 (outward integration), started from the
    expansion at the origin of :519-523 with p = L+1.  Renormalisation is
    off (the reference default, source/lecture.f90:2156).  With eimag > 0
    (a complex energy) the solution is complex: the expansion gains the
    imaginary term ci r^(p+2), ci = -Eimag / (4L + 6) (:471, :548), and the
    recursion -i Eimag on its diagonal (:631-633).
    """
    if eimag != 0.0:
        return _sch_radial_complex(r, V, enervide, ecinetic, L, Z, eimag)
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
    clapl0 = -claplm - claplp
    f2 = 1.0 / r ** 2
    vme = V - enervide
    g0 = -clapl0 + vme
    gm = -claplm
    gp = -claplp
    br = -Z / (L + 1.0)
    cr = -(2 * Z * br + ecinetic) / (4 * L + 6)
    p = L + 1.0
    u = np.zeros(nr)
    u[0:2] = (1 + br * r[0:2] + cr * r[0:2] ** 2) * r[0:2] ** p
    L2 = L * (L + 1)
    for ir in range(1, nr - 1):
        td = g0[ir] + L2 * f2[ir]
        u[ir + 1] = -(td * u[ir] + gm[ir] * u[ir - 1]) / gp[ir]
    return u / r


def _sch_radial_complex(r, V, enervide, ecinetic, L, Z, eimag):
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
    br = -Z / (L + 1.0)
    cr = -(2 * Z * br + ecinetic) / (4 * L + 6)
    ci = -eimag / (4 * L + 6)
    p = L + 1.0
    u = np.zeros(nr, dtype=np.complex128)
    u[0:2] = (1 + br * r[0:2] + cr * r[0:2] ** 2) * r[0:2] ** p + 1j * ci * r[0:2] ** (p + 2)
    L2 = L * (L + 1)
    for ir in range(1, nr - 1):
        td = g0[ir] + L2 * f2[ir]
        u[ir + 1] = -(td * u[ir] + gm[ir] * u[ir - 1] - 1j * eimag * u[ir]) / gp[ir]
    return u / r


def f_interp2(x, rm, r0, rp, fm, f0, fp):
    """Quadratic interpolation through three points: source/tools.f90:504-522."""
    dp0 = rp - r0
    dpm = rp - rm
    d0m = r0 - rm
    a = (fm * dp0 - f0 * dpm + fp * d0m) / (d0m * dp0 * dpm)
    b = (f0 - fm) / d0m - a * (r0 + rm)
    c = f0 - a * r0 ** 2 - b * r0
    return a * x ** 2 + b * x + c


# ---------------------------------------------------------------------------
# Bessel / Neumann (cbessneur, source/sphere.f90:7356-7384)
# ---------------------------------------------------------------------------

def cbessneur(fnorm: float, z: np.ndarray, lmax: int):
    """fnorm * j_l(z), fnorm * n_l(z) by upward recursion; z: (n,)."""
    bs = np.zeros((len(z), lmax + 1))
    nm = np.zeros((len(z), lmax + 1))
    nm[:, 0] = -fnorm * np.cos(z) / z
    bs[:, 0] = fnorm * np.sin(z) / z
    if lmax == 0:
        return bs, nm
    nm[:, 1] = nm[:, 0] / z - bs[:, 0]
    bs[:, 1] = bs[:, 0] / z + nm[:, 0]
    for L in range(2, lmax + 1):
        L1 = 2 * L - 1
        nm[:, L] = L1 * nm[:, L - 1] / z - nm[:, L - 2]
        bs[:, L] = L1 * bs[:, L - 1] / z - bs[:, L - 2]
    return bs, nm


# ---------------------------------------------------------------------------
# The full static structure and per-energy inputs
# ---------------------------------------------------------------------------

@dataclasses.dataclass
class Structure:
    """Energy-independent inputs of one FDM problem (one site, C1)."""
    cluster: Cluster
    grid: Grid
    lmaxat_max: np.ndarray     # (nproto,) largest atom lmax over the spectrum
    lmaxso_max: int
    nlmmax: int
    nlmomax: int
    Ylmato: np.ndarray         # (nbtm, nlmmax, natome) F
    Ylmso: np.ndarray          # (nsort, nlmomax) F
    rrel: np.ndarray           # (nbtm, natome) distance of boundary points to their atom
    lato: np.ndarray           # (nlmsam, natome) F  (ngrph = 1)
    mato: np.ndarray
    iato: np.ndarray
    lso: np.ndarray            # (nso1,)
    mso: np.ndarray
    iso: np.ndarray
    distai: np.ndarray         # (natome,)
    Vr: np.ndarray             # (npoint, nspin) F   model potential (energy independent)
    V0bd: float                # interstitial average (Ry)
    radial_r: List[np.ndarray]   # per prototype radial mesh
    radial_V: List[np.ndarray]   # per prototype radial potential
    nspin: int = 1
    spin_split: float = 0.0    # Ry: spin block 1 is shifted by -split/2, block 2 by +split/2

    @property
    def natome(self):
        return self.cluster.natome

    def spin_shift(self, ispin: int) -> float:
        """Potential shift (Ry) of spin block ispin (1-based)."""
        if self.nspin == 1:
            return 0.0
        return (-0.5 if ispin == 1 else 0.5) * self.spin_split


def build_structure(cl: Cluster, adimp_ang: float, rsort_ang: float, e_max_ev: float,
                    e_fermi_ev: float = -5.0, v0_ev: float = -12.0, lmax_abs: int = 3,
                    nspin: int = 1, spin_split_ev: float = 0.0) -> Structure:
    """Static structure of a C1 FDM problem sized for energies up to e_max_ev."""
    g = build_grid(cl, adimp_ang, rsort_ang)
    natome = cl.natome
    # potential at grid points: superposition, then shifted
    pts = g.xyz[:3, :g.npoint]
    V = np.zeros(g.npoint)
    for k in range(cl.pot_atoms.shape[1]):
        d = np.sqrt(((pts - cl.pot_atoms[:, k:k + 1]) ** 2).sum(0))
        V += _screened_coulomb(d, cl.pot_zeff[k])
    inter = g.numia[:g.npoint] == 0
    v0 = v0_ev / RYDB
    shift = v0 - V[inter].mean()
    V += shift
    Vr = _f64((g.npoint, nspin))
    for isp in range(nspin):
        sgn = 0.0 if nspin == 1 else (-0.5 if isp == 0 else 0.5)
        Vr[:, isp] = V + sgn * spin_split_ev / RYDB
    # radial potentials per prototype: own screened Coulomb + neighbours' monopole + shift
    nproto = len(cl.rmt)
    radial_r, radial_V = [], []
    for ipr in range(nproto):
        ia = int(np.nonzero(cl.itype == ipr)[0][0]) if (cl.itype == ipr).any() else 0
        Zp = int(cl.zproto[ipr])
        r = radial_mesh(Zp, cl.rmt[ipr] + 3 * g.adimp)
        # atom ia's own potential + others at distance
        own = np.argmin(((cl.pot_atoms - cl.pos[:, ia:ia + 1]) ** 2).sum(0))
        Vrad = _screened_coulomb(r, cl.pot_zeff[own])
        for k in range(cl.pot_atoms.shape[1]):
            if k == own:
                continue
            d = math.sqrt(((cl.pot_atoms[:, k] - cl.pos[:, ia]) ** 2).sum())
            Vrad = Vrad + _screened_coulomb(np.array([d]), cl.pot_zeff[k])[0]
        radial_r.append(r)
        radial_V.append(Vrad + shift)
    # l cut-offs at the highest energy (tables sized by them)
    ec_max = (e_max_ev + e_fermi_ev) / RYDB - v0
    lmaxat_max = np.zeros(nproto, dtype=np.int32)
    for ipr in range(nproto):
        lmaxat_max[ipr] = clmax(ec_max, cl.rmtg[ipr], -1, int(cl.zproto[ipr]), False)
    lmaxat_max[0] = max(lmaxat_max[0], lmax_abs)
    lmaxso_max = clmax(ec_max, g.rsort, -5, -1, True)
    nlmmax = int((lmaxat_max.max() + 1) ** 2)
    nlmomax = (lmaxso_max + 1) ** 2
    # Ylmpt
    Ylmato = _f64((g.nbtm, nlmmax, natome))
    rrel = _f64((g.nbtm, natome))
    for ia in range(natome):
        nb = g.nbord[ia]
        idx = g.ibord[:nb, ia] - 1
        v = g.xyz[:3, idx] - cl.pos[:, ia:ia + 1]
        lmax = int(lmaxat_max[cl.itype[ia]])
        Ylmato[:nb, :(lmax + 1) ** 2, ia] = real_ylm(lmax, v).T
        rrel[:nb, ia] = np.sqrt((v ** 2).sum(0))
    Ylmso = _f64((g.nsort, nlmomax))
    v = g.xyz[:3, g.isrt - 1]
    Ylmso[:, :] = real_ylm(lmaxso_max, v).T
    # lmrep tables (C1: L = 0..lmax, m = -L..L, nspino = 1)
    nlmsam = nlmmax
    lato = _i32((nlmsam, natome))
    mato = _i32((nlmsam, natome))
    iato = _i32((nlmsam, natome))
    lato[:] = 10000
    for ia in range(natome):
        lmax = int(lmaxat_max[cl.itype[ia]])
        k = 0
        for L in range(lmax + 1):
            for m in range(-L, L + 1):
                lato[k, ia], mato[k, ia], iato[k, ia] = L, m, 1
                k += 1
    lso = np.zeros(nlmomax, dtype=np.int32)
    mso = np.zeros(nlmomax, dtype=np.int32)
    iso = np.ones(nlmomax, dtype=np.int32)
    k = 0
    for L in range(lmaxso_max + 1):
        for m in range(-L, L + 1):
            lso[k], mso[k] = L, m
            k += 1
    distai = np.sqrt((cl.pos ** 2).sum(0))
    return Structure(cluster=cl, grid=g, lmaxat_max=lmaxat_max, lmaxso_max=lmaxso_max,
                     nlmmax=nlmmax, nlmomax=nlmomax, Ylmato=Ylmato, Ylmso=Ylmso, rrel=rrel,
                     lato=lato, mato=mato, iato=iato, lso=lso, mso=mso, iso=iso, distai=distai,
                     Vr=Vr, V0bd=v0, radial_r=radial_r, radial_V=radial_V, nspin=nspin,
                     spin_split=spin_split_ev / RYDB)


@dataclasses.dataclass
class EnergyInputs:
    """Per-energy inputs of one ``mat_solve`` call (real case)."""
    energy_ev: float
    enervide: float            # Ry
    eimag: float
    ecinetic_out: float        # Ry
    lmaxa: np.ndarray          # (natome,)
    lmaxso: int
    nlmsa: np.ndarray          # (natome,)
    nlmso: int
    nlmagm: int
    phiato: Optional[np.ndarray]   # (nbtm, nlmagm, nspinp=nspin, nspino=1, n_RI=1, natome, nphiato7=1) F
    besselr: Optional[np.ndarray]  # (nsort, 0:lmaxso, nspinr=1) F; None: generated on the device
    neumanr: Optional[np.ndarray]
    ispin: int = 1


def boundary_radial(st: Structure, enervide: float, lmaxa: np.ndarray, eimag: float = 0.0) -> Dict[tuple, np.ndarray]:
    """Radial solutions u_L(r) of every atom at its boundary points (Sch_radial,
    then f_interp2 as in cal_phiato), keyed by (spin block, atom index 0-based,
    L) for every spin block of the structure and L <= lmaxa[ia]; complex at a
    complex energy (eimag > 0)."""
    cl, g = st.cluster, st.grid
    out: Dict[tuple, np.ndarray] = {}
    ur_cache: Dict[tuple, np.ndarray] = {}
    for isp in range(1, st.nspin + 1):
        dvs = st.spin_shift(isp)
        ecs = enervide - (st.V0bd + dvs)
        for ia in range(cl.natome):
            ipr = int(cl.itype[ia])
            r = st.radial_r[ipr]
            Vrad = st.radial_V[ipr] + dvs
            nb = int(g.nbord[ia])
            rr = st.rrel[:nb, ia]
            idx = np.searchsorted(r, rr, side="right")   # first r(i) > rrel, 0-based
            idx = np.clip(idx, 2, len(r) - 1)
            for L in range(int(lmaxa[ia]) + 1):
                key = (isp, ipr, L)
                if key not in ur_cache:
                    ur_cache[key] = sch_radial(r, Vrad, enervide, ecs, L, float(cl.zproto[ipr]) +
                                               (1.0 if ipr == 0 else 0.0), eimag)
                u = ur_cache[key]
                out[(isp, ia, L)] = f_interp2(rr, r[idx - 2], r[idx - 1], r[idx], u[idx - 2], u[idx - 1], u[idx])
    return out


def radial_tables(st: Structure) -> dict:
    """The structure's radial data in the layout of fdmgpu_radial: per atom type
    the radial mesh and spherical potential, the spin shifts, the charge of the
    expansion at the origin (Z, plus one for the absorber's type, as
    boundary_radial uses), atom types (1-based), boundary distances and the
    radii of the outer points."""
    cl, g = st.cluster, st.grid
    ntype = len(st.radial_r)
    nr = np.array([len(r) for r in st.radial_r], dtype=np.int32)
    nr_max = int(nr.max())
    r = np.zeros((nr_max, ntype), order="F")
    V = np.zeros((nr_max, ntype), order="F")
    for t in range(ntype):
        r[:nr[t], t] = st.radial_r[t]
        V[:nr[t], t] = st.radial_V[t]
    return dict(ntype=ntype, nr_max=nr_max, nspin=st.nspin, nr=nr, r=r, V=V,
                dv_spin=np.array([st.spin_shift(i) for i in range(1, st.nspin + 1)]),
                z_origin=np.array([float(cl.zproto[t]) + (1.0 if t == 0 else 0.0) for t in range(ntype)]),
                itype=(np.asarray(cl.itype, dtype=np.int32) + 1), rrel=st.rrel,
                rsort=np.ascontiguousarray(g.xyz[3, g.isrt - 1]), v0bd=st.V0bd)


def energy_inputs(st: Structure, energy_ev: float, e_fermi_ev: float = -5.0, ispin: int = 1,
                  functions: bool = True) -> EnergyInputs:
    """Per-energy inputs: l cut-offs, atomic boundary functions, Bessel/Neumann.
    With functions=False only the cut-offs and sizes are formed (phiato,
    besselr and neumanr are None): the library then generates them on the
    device from the structure's radial tables (radial_tables)."""
    cl, g = st.cluster, st.grid
    enervide = (energy_ev + e_fermi_ev) / RYDB
    dv = st.spin_shift(ispin)
    ecin = enervide - (st.V0bd + dv)
    ecin_out = ecin
    if ecin_out < EPS10:
        raise ValueError("kinetic energy in the outer sphere must be positive for the real path")
    nproto = len(cl.rmt)
    lmaxat = np.zeros(nproto, dtype=np.int32)
    for ipr in range(nproto):
        lmaxat[ipr] = min(clmax(ecin, cl.rmtg[ipr], -1, int(cl.zproto[ipr]), False), st.lmaxat_max[ipr])
    lmaxat[0] = max(lmaxat[0], min(3, st.lmaxat_max[0]))
    lmaxso = min(clmax(ecin_out, g.rsort, -5, -1, True), st.lmaxso_max)
    natome = cl.natome
    lmaxa = np.array([lmaxat[cl.itype[ia]] for ia in range(natome)], dtype=np.int32)
    nlmsa = ((lmaxa + 1) ** 2).astype(np.int32)
    nlmso = (lmaxso + 1) ** 2
    lmax_g = int(lmaxat.max())
    nlmagm = (lmax_g + 1) ** 2
    if not functions:
        return EnergyInputs(energy_ev=energy_ev, enervide=enervide, eimag=0.0, ecinetic_out=ecin_out,
                            lmaxa=lmaxa, lmaxso=lmaxso, nlmsa=nlmsa, nlmso=nlmso, nlmagm=nlmagm,
                            phiato=None, besselr=None, neumanr=None, ispin=ispin)
    # radial solutions per prototype, spin and L, then cal_phiato per atom.
    # phiato holds every spin block (nspinp = nspin): the grid rows of
    # calcMatRow read it at min(ispin, nspin) (source/mat.f90:1144,1296-1304).
    nspinp = st.nspin
    phiato = np.zeros((g.nbtm, nlmagm, nspinp, 1, 1, natome, 1), order="F")
    for (isp, ia, L), phi in boundary_radial(st, enervide, lmaxa).items():
        nb = int(g.nbord[ia])
        for m in range(-L, L + 1):
            lm = L * L + L + m
            phiato[:nb, lm, isp - 1, 0, 0, ia, 0] = phi * st.Ylmato[:nb, lm, ia]
    # phiso, non-Rydberg, real branch
    konder = math.sqrt(ecin_out)
    fnorm = math.sqrt(konder / math.pi)
    zr = konder * g.xyz[3, g.isrt - 1]
    bs, nm = cbessneur(fnorm, zr, lmaxso)
    besselr = np.asfortranarray(bs.reshape(g.nsort, lmaxso + 1, 1))
    neumanr = np.asfortranarray(nm.reshape(g.nsort, lmaxso + 1, 1))
    return EnergyInputs(energy_ev=energy_ev, enervide=enervide, eimag=0.0, ecinetic_out=ecin_out,
                        lmaxa=lmaxa, lmaxso=lmaxso, nlmsa=nlmsa, nlmso=nlmso, nlmagm=nlmagm,
                        phiato=phiato, besselr=besselr, neumanr=neumanr, ispin=ispin)


# ---------------------------------------------------------------------------
# newind (source/mat.f90:1761-1921), regular solution, nspino = 1 or 2
# ---------------------------------------------------------------------------

@dataclasses.dataclass
class RowIndex:
    nligne: int
    nligneso: int
    new: np.ndarray      # (0:npoint) 1-based rows
    newinv: np.ndarray   # (nligne,)
    ianew: np.ndarray    # (natome,)
    lb1: np.ndarray      # (nligne,)
    lb2: np.ndarray


def newind(st: Structure, nlmsa: np.ndarray, nlmso: int, nspino: int = 1, irregular: bool = False) -> RowIndex:
    """Row numbering and profile of the FDM matrix (source/mat.f90:1761-1921).
    irregular: the irregular cluster solution of FDM_comp with both atomic
    solutions (Test_reg = 0, source/mat.f90:140-147): 2 nlmsa amplitude rows per
    atom and no outer-sphere rows; nligneso = nligne."""
    g = st.grid
    natome = st.natome
    npoint = g.npoint
    n_ato_ri = 2 if irregular else 1
    if irregular:
        nligne = nspino * g.npr + n_ato_ri * int(nlmsa.sum())
    else:
        nligne = nspino * g.npr + nlmso + int(nlmsa.sum())
    numia = g.numia
    new = np.zeros(npoint + 1, dtype=np.int64)   # new[0] = new(0)
    inter = numia[:npoint] == 0
    new[1:][inter] = nspino * np.arange(1, int(inter.sum()) + 1)
    ianew = np.zeros(natome, dtype=np.int64)
    npf, npf1 = 1, 0
    r4 = g.xyz[3]
    for ia in range(natome):
        i = npf
        while i <= npoint:
            if numia[i - 1] == 0 and r4[i - 1] >= st.distai[ia]:
                break
            i += 1
        npf = i
        if npf1 == npf:
            ianew[ia] = ianew[ia - 1] + n_ato_ri * nlmsa[ia - 1]
        else:
            ianew[ia] = new[npf] - nspino
        npf1 = npf
        sel = np.arange(npf, npoint + 1)
        sel = sel[numia[sel - 1] == 0]
        new[sel] += n_ato_ri * nlmsa[ia]
    lb1 = np.arange(1, nligne + 1, dtype=np.int64)
    lb2 = lb1.copy()
    n = nspino - 1
    ivois = g.ivois
    for i in range(1, npoint + 1):
        if numia[i - 1] != 0:
            continue
        ii = new[i]
        for iv in range(g.nvois):
            j = ivois[i - 1, iv]
            if j == 0:
                raise RuntimeError("newind: missing neighbour")
            ia = numia[j - 1]
            if ia == 0:
                lb1[ii - 1] = min(lb1[ii - 1], new[j] - n)
                lb2[ii - 1] = max(lb2[ii - 1], new[j])
            elif ia > 0:
                lb1[ii - 1] = min(lb1[ii - 1], ianew[ia - 1] + 1)
                lb2[ii - 1] = max(lb2[ii - 1], ianew[ia - 1] + n_ato_ri * nlmsa[ia - 1])
            elif ia == -2:
                lb2[ii - 1] = nligne
        if nspino == 2:      # the point's spin-1 row has the same span
            lb1[ii - 2] = lb1[ii - 1]
            lb2[ii - 2] = lb2[ii - 1]
    for ia in range(natome):
        lb11 = ianew[ia] + 1
        lb22 = ianew[ia] + n_ato_ri * nlmsa[ia]
        for ib in range(g.nbordf[ia]):
            lb11 = min(lb11, new[g.ibord[ib, ia]] - n)
            lb22 = max(lb22, new[g.ibord[ib, ia]])
        for L in range(1, n_ato_ri * nlmsa[ia] + 1):
            lb1[ianew[ia] + L - 1] = lb11
            lb2[ianew[ia] + L - 1] = lb22
    if not irregular:   # there is no scattered amplitude for the irregular solution
        lb11 = nligne - nlmso + 1
        for ib in range(g.nsortf):
            lb11 = min(lb11, new[g.isrt[ib]] - n)
        lb1[nligne - nlmso:] = lb11
        lb2[nligne - nlmso:] = nligne
    lb1 = np.minimum.accumulate(lb1[::-1])[::-1].copy()
    newinv = np.zeros(nligne, dtype=np.int64)
    for i in range(1, npoint + 1):
        ii = new[i]
        if ii != 0:
            newinv[ii - 1] = i
            if nspino == 2:
                newinv[ii - 2] = i
    for ia in range(natome):
        newinv[ianew[ia]:ianew[ia] + n_ato_ri * nlmsa[ia]] = -(ia + 1)
    return RowIndex(nligne=nligne, nligneso=nligne if irregular else nligne - nlmso, new=new.astype(np.int32),
                    newinv=newinv.astype(np.int32), ianew=ianew.astype(np.int32),
                    lb1=lb1.astype(np.int32), lb2=lb2.astype(np.int32))


# ---------------------------------------------------------------------------
# Named workloads
# ---------------------------------------------------------------------------

def cu_structure(adimp_ang: float = 0.25, rsort_ang: float = 3.0, r_cluster_ang: float = 2.6,
                 e_max_ev: float = 35.0) -> Structure:
    """fcc Cu K-edge, 13-atom cluster, FDM radius 3.0 A, step 0.25 A, C1."""
    return build_structure(cu_cluster(r_cluster_ang), adimp_ang, rsort_ang, e_max_ev)


def small_cu_structure(rsort_ang: float = 1.6, adimp_ang: float = 0.25, e_max_ev: float = 35.0) -> Structure:
    """Small Cu case for fast parity tests: absorber only inside a 1.6 A sphere."""
    return build_structure(cu_cluster(0.5), adimp_ang, rsort_ang, e_max_ev)


def energy_grid(e_min: float, e_max: float, step: float) -> np.ndarray:
    n = int(round((e_max - e_min) / step)) + 1
    return e_min + step * np.arange(n)
