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
                ("ms_refine", C.c_double)]


def _pi(a: np.ndarray, keep: List):
    a = np.asfortranarray(a, dtype=np.int32)
    keep.append(a)
    return a.ctypes.data_as(P_I32)


def _pd(a: np.ndarray, keep: List):
    a = np.asfortranarray(a, dtype=np.float64)
    keep.append(a)
    return a.ctypes.data_as(P_F64)


class GridArgs:
    """An FdmGrid struct built from a Structure (keeps its buffers alive)."""

    def __init__(self, st: CL.Structure):
        g = st.grid
        self.keep: List = []
        k = self.keep
        s = FdmGrid()
        s.npoint, s.npsom, s.nvois, s.natome = g.npoint, g.npso, g.nvois, st.natome
        s.nbm, s.nbtm, s.nim, s.nsm = g.nbm, g.nbtm, g.npoint, max(g.nsortf, 1)
        s.nsort, s.nsortf, s.nstm, s.nspin = g.nsort, g.nsortf, g.nsort, st.nspin
        s.nlmmax, s.nlmomax = st.nlmmax, st.nlmomax
        s.nlmsam, s.nso1, s.ngrph, s.nspino = st.lato.shape[0], st.lso.shape[0], 1, 1
        s.ivois, s.isvois, s.numia = _pi(g.ivois, k), _pi(g.isvois, k), _pi(g.numia, k)
        s.nbord, s.nbordf = _pi(g.nbord, k), _pi(g.nbordf, k)
        s.ibord, s.isbord, s.isrt = _pi(g.ibord, k), _pi(g.isbord, k), _pi(g.isrt, k)
        s.lato, s.mato, s.iato = _pi(st.lato, k), _pi(st.mato, k), _pi(st.iato, k)
        s.lso, s.mso, s.iso = _pi(st.lso, k), _pi(st.mso, k), _pi(st.iso, k)
        s.clapl, s.cgrad, s.rvol = _pd(g.clapl, k), _pd(g.cgrad, k), _pd(g.rvol, k)
        s.poidsa, s.poidso = _pd(g.poidsa, k), _pd(g.poidso, k)
        s.Ylmato, s.Ylmso = _pd(st.Ylmato, k), _pd(st.Ylmso, k)
        kar = np.zeros((64, 1), order="F")
        kar[:, 0] = 1.0      # C1: identity character on every operation index used
        s.Kar, s.Kari = _pd(kar, k), _pd(np.zeros((64, 1), order="F"), k)
        self.s = s

    @property
    def ptr(self):
        return C.byref(self.s)


class EnergyArgs:
    """An FdmEnergy struct for one energy (real path, regular solution)."""

    def __init__(self, st: CL.Structure, ei: CL.EnergyInputs, ri: CL.RowIndex):
        g = st.grid
        self.keep: List = []
        k = self.keep
        s = FdmEnergy()
        s.nligne, s.nligneso, s.nlmso, s.lmaxso = ri.nligne, ri.nligneso, ei.nlmso, ei.lmaxso
        s.nlmagm, s.nphiato1, s.nphiato7, s.nspinp = ei.nlmagm, g.nbtm, 1, 1
        s.n_RI, s.n_ato_RI, s.nspinr = 1, 1, 1
        s.nsort_r, s.nsort_c, s.igrph, s.ispin, s.nicm = g.nsort, 0, 1, ei.ispin, 1
        s.Cal_comp = s.E_comp = s.Base_hexa = s.irregular = s.Relativiste = 0
        s.Spinorbite = s.Repres_comp = s.Ylm_comp = s.Test_reg = 0
        s.Basereel = 1
        s.Enervide, s.Eimag = ei.enervide, ei.eimag
        s.new_, s.newinv = _pi(ri.new, k), _pi(ri.newinv, k)
        s.lb1, s.lb2, s.ianew, s.nlmsa = _pi(ri.lb1, k), _pi(ri.lb2, k), _pi(ri.ianew, k), _pi(ei.nlmsa, k)
        s.Vr = _pd(st.Vr, k)
        s.gradvr = _pd(np.zeros((1, 3, 1), order="F"), k)
        s.phiato = _pd(ei.phiato, k)
        s.Besselr, s.Neumanr = _pd(ei.besselr, k), _pd(ei.neumanr, k)
        s.Bessel = s.Neuman = None
        self.s = s
        self.nligne, self.nlmso = ri.nligne, ei.nlmso

    @property
    def ptr(self):
        return C.byref(self.s)
