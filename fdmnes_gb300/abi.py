"""ctypes mirror of include/fdmgpu.h and helpers that fill it from numpy arrays.

The structs restate the argument list of the reference's ``mat_solve``
(source/mat_solve_gaussian.f90:5-67).  Arrays are passed in their Fortran
layout with 1-based index values; the ``keep`` lists hold references so that
the numpy buffers outlive the struct.
"""
from __future__ import annotations

import ctypes as C
from typing import List

import numpy as np

from . import cluster as CL

P_I32 = C.POINTER(C.c_int32)
P_F64 = C.POINTER(C.c_double)


class FdmGrid(C.Structure):
    _fields_ = [(n, C.c_int32) for n in (
        "npoint", "npsom", "nvois", "natome", "nbm", "nbtm", "nim", "nsm", "nsort", "nsortf", "nstm",
        "nspin", "nlmmax", "nlmomax", "nlmsam", "nso1", "ngrph", "nspino")] + [
        ("ivois", P_I32), ("isvois", P_I32), ("numia", P_I32), ("nbord", P_I32), ("nbordf", P_I32),
        ("ibord", P_I32), ("isbord", P_I32), ("isrt", P_I32), ("lato", P_I32), ("mato", P_I32),
        ("iato", P_I32), ("lso", P_I32), ("mso", P_I32), ("iso", P_I32),
        ("clapl", P_F64), ("cgrad", P_F64), ("rvol", P_F64), ("poidsa", P_F64), ("poidso", P_F64),
        ("Ylmato", P_F64), ("Ylmso", P_F64), ("Kar", P_F64), ("Kari", P_F64)]


class FdmEnergy(C.Structure):
    _fields_ = [(n, C.c_int32) for n in (
        "nligne", "nligneso", "nlmso", "lmaxso", "nlmagm", "nphiato1", "nphiato7", "nspinp", "n_RI",
        "n_ato_RI", "nspinr", "nsort_r", "nsort_c", "igrph", "ispin", "nicm",
        "Cal_comp", "E_comp", "Basereel", "Base_hexa", "irregular", "Relativiste", "Spinorbite",
        "Repres_comp", "Ylm_comp", "Test_reg")] + [
        ("Enervide", C.c_double), ("Eimag", C.c_double),
        ("new_", P_I32), ("newinv", P_I32), ("lb1", P_I32), ("lb2", P_I32), ("ianew", P_I32),
        ("nlmsa", P_I32), ("Vr", P_F64), ("gradvr", P_F64), ("phiato", P_F64),
        ("Besselr", P_F64), ("Neumanr", P_F64), ("Bessel", P_F64), ("Neuman", P_F64)]


class FdmInfo(C.Structure):
    _fields_ = [("nnz_profile", C.c_int64), ("flops_factor", C.c_double), ("flops_solve", C.c_double),
                ("refine_iters", C.c_int32), ("residual", C.c_double),
                ("ms_assemble", C.c_double), ("ms_factor", C.c_double), ("ms_solve", C.c_double),
                ("ms_refine", C.c_double), ("n_fallback", C.c_int32), ("n_kernels", C.c_int64),
                ("ms_residual_first", C.c_double), ("flops_residual", C.c_double),
                ("ms_escalate_factor", C.c_double), ("flops_escalate_factor", C.c_double),
                ("n_wide_refactor", C.c_int32), ("ms_wide_refactor", C.c_double),
                ("flops_wide_refactor", C.c_double), ("ms_refine_loop", C.c_double),
                ("refine_steps", C.c_int64)]


def _pi(a: np.ndarray, keep: List):
    a = np.asfortranarray(a, dtype=np.int32)
    keep.append(a)
    return a.ctypes.data_as(P_I32)


def _pd(a: np.ndarray, keep: List):
    a = np.asfortranarray(a, dtype=np.float64)
    keep.append(a)
    return a.ctypes.data_as(P_F64)


def grid_dict(st: CL.Structure) -> dict:
    """The energy-independent mat_solve arguments of a Structure as plain arrays."""
    g = st.grid
    kar = np.zeros((64, 1), order="F")
    kar[:, 0] = 1.0      # C1: identity character on every operation index used
    return dict(
        npoint=g.npoint, npsom=g.npso, nvois=g.nvois, natome=st.natome, nbm=g.nbm, nbtm=g.nbtm, nim=g.npoint,
        nsm=max(g.nsortf, 1), nsort=g.nsort, nsortf=g.nsortf, nstm=g.nsort, nspin=st.nspin, nlmmax=st.nlmmax,
        nlmomax=st.nlmomax, nlmsam=st.lato.shape[0], nso1=st.lso.shape[0], ngrph=1, nspino=1,
        ivois=g.ivois, isvois=g.isvois, numia=g.numia, nbord=g.nbord, nbordf=g.nbordf, ibord=g.ibord,
        isbord=g.isbord, isrt=g.isrt, lato=st.lato, mato=st.mato, iato=st.iato, lso=st.lso, mso=st.mso,
        iso=st.iso, clapl=g.clapl, cgrad=g.cgrad, rvol=g.rvol, poidsa=g.poidsa, poidso=g.poidso,
        Ylmato=st.Ylmato, Ylmso=st.Ylmso, Kar=kar, Kari=np.zeros((64, 1), order="F"))


class FdmRadial(C.Structure):
    _fields_ = [("ntype", C.c_int32), ("nr_max", C.c_int32), ("nspin", C.c_int32), ("nr", P_I32),
                ("r", P_F64), ("V", P_F64), ("dv_spin", P_F64), ("z_origin", P_F64), ("itype", P_I32),
                ("rrel", P_F64), ("rsort", P_F64), ("v0bd", C.c_double)]


class RadialArgs:
    """An FdmRadial struct from a Structure (cluster.radial_tables)."""

    def __init__(self, st):
        self.keep: List = []
        self.d = CL.radial_tables(st)
        self.s = _fill(FdmRadial, self.d, self.keep)


def energy_dict(st: CL.Structure, ei: CL.EnergyInputs, ri: CL.RowIndex) -> dict:
    """The per-call mat_solve arguments of one energy (real path) as plain arrays.
    Inputs left None (phiato, Bessel, Neumann) are passed as NULL: the library
    generates them on the device."""
    g = st.grid
    nspinp = ei.phiato.shape[2] if ei.phiato is not None else st.nspin
    return dict(
        nligne=ri.nligne, nligneso=ri.nligneso, nlmso=ei.nlmso, lmaxso=ei.lmaxso, nlmagm=ei.nlmagm,
        nphiato1=g.nbtm, nphiato7=1, nspinp=nspinp, n_RI=1, n_ato_RI=1, nspinr=1, nsort_r=g.nsort, nsort_c=0,
        igrph=1, ispin=ei.ispin, nicm=1, Cal_comp=0, E_comp=0, Basereel=1, Base_hexa=0, irregular=0,
        Relativiste=0, Spinorbite=0, Repres_comp=0, Ylm_comp=0, Test_reg=0,
        Enervide=ei.enervide, Eimag=ei.eimag, new_=ri.new, newinv=ri.newinv, lb1=ri.lb1, lb2=ri.lb2,
        ianew=ri.ianew, nlmsa=ei.nlmsa, Vr=st.Vr, gradvr=np.zeros((1, 3, 1), order="F"), phiato=ei.phiato,
        Besselr=ei.besselr, Neumanr=ei.neumanr)


def _fill(struct_cls, d: dict, keep: List):
    s = struct_cls()
    for name, typ in struct_cls._fields_:
        v = d.get(name)
        if v is None:
            continue
        if typ is P_I32:
            setattr(s, name, _pi(np.asarray(v), keep))
        elif typ is P_F64:
            setattr(s, name, _pd(np.asarray(v), keep))
        else:
            setattr(s, name, typ(v.item() if isinstance(v, np.ndarray) else v).value)
    return s


class GridArgs:
    """An FdmGrid struct built from a Structure or from grid_dict() arrays."""

    def __init__(self, src):
        self.keep: List = []
        self.d = grid_dict(src) if isinstance(src, CL.Structure) else src
        self.s = _fill(FdmGrid, self.d, self.keep)

    @property
    def ptr(self):
        return C.byref(self.s)


class EnergyArgs:
    """An FdmEnergy struct for one energy, from (Structure, EnergyInputs, RowIndex)
    or from energy_dict() arrays."""

    def __init__(self, st, ei=None, ri=None):
        self.keep: List = []
        self.d = energy_dict(st, ei, ri) if ei is not None else st
        self.s = _fill(FdmEnergy, self.d, self.keep)
        self.nligne, self.nlmso = int(self.d["nligne"]), int(self.d["nlmso"])

    @property
    def ptr(self):
        return C.byref(self.s)
