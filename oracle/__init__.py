"""CPU oracle of the FDM assembly + Gaussian solve (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package.  It loads oracle/_build/liboracle.so, built by ``make -C oracle``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
# the same sources at -O3 (the reference's build level), for the timed CPU baseline only
LIB_TIMED_PATH = os.path.join(HERE, "_build", "liboracle_timed.so")
_lib = None
_use_timed = False


def use_timed_build(on: bool = True) -> None:
    """Route this process's oracle calls to the -O3 build (bench.py's CPU
    baseline).  Must be called before the first oracle call of the process."""
    global _use_timed
    if _lib is not None and on != _use_timed:
        raise RuntimeError("oracle library already loaded")
    _use_timed = on


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        path = LIB_TIMED_PATH if _use_timed else LIB_PATH
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        vp = C.c_void_p
        L.oracle_mat_solve.argtypes = [vp, vp, vp, C.POINTER(C.c_int64), C.POINTER(C.c_double),
                                       C.POINTER(C.c_double), C.POINTER(C.c_int32)]
        L.oracle_assemble_dense.argtypes = [vp, vp, vp, vp]
        L.oracle_assemble_csr.argtypes = [vp, vp, vp, vp, vp, vp]
        L.oracle_assemble_csr_c.argtypes = [vp, vp, vp, vp, vp, vp]
        L.oracle_newind.argtypes = [vp, vp, vp, vp, C.c_int, C.c_int32, vp, vp, vp, vp, vp]
        L.oracle_newind_irregular.argtypes = [vp, vp, vp, vp, C.c_int32, vp, vp, vp, vp, vp]
        L.oracle_cbessneur.argtypes = [C.c_double, C.c_double, C.c_int, vp, vp]
        L.oracle_invcomp.argtypes = [C.c_int, vp]
        L.oracle_taull.argtypes = [vp, vp, C.c_int, vp, vp, C.POINTER(C.c_int32)]
        L.oracle_mat_solve_c.argtypes = [vp, vp, vp, vp, C.POINTER(C.c_int64), C.POINTER(C.c_double),
                                         C.POINTER(C.c_double), C.POINTER(C.c_int32)]
        L.oracle_assemble_dense_c.argtypes = [vp, vp, vp, vp]
        L.oracle_taull_c.argtypes = [vp, vp, C.c_int, vp, vp, C.c_int, vp, C.POINTER(C.c_int32)]
        L.oracle_cbessneu.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, vp, vp]
        L.oracle_tau_ri.argtypes = [vp, vp, vp, vp, vp, vp, vp, C.c_int, vp, C.POINTER(C.c_int32)]
        _lib = L
    return _lib


def mat_solve(grid_args, energy_args):
    """Solution smr (nlmso, nligne) Fortran-ordered, plus timing and nnz."""
    n, m = energy_args.nligne, energy_args.nlmso
    smr = np.zeros((m, n), order="F")
    nnz = C.c_int64(0)
    tf, tt = C.c_double(0), C.c_double(0)
    bad = C.c_int32(0)
    st = lib().oracle_mat_solve(C.addressof(grid_args.s), C.addressof(energy_args.s), smr.ctypes.data,
                                C.byref(nnz), C.byref(tf), C.byref(tt), C.byref(bad))
    if st != 0:
        raise RuntimeError(f"oracle_mat_solve failed with status {st} (row {bad.value})")
    return smr, dict(nnz=nnz.value, time_fill=tf.value, time_tria=tt.value)


def assemble_dense(grid_args, energy_args):
    n, m = energy_args.nligne, energy_args.nlmso
    A = np.zeros((n, n), order="F")
    B = np.zeros((m, n), order="F")
    st = lib().oracle_assemble_dense(C.addressof(grid_args.s), C.addressof(energy_args.s), A.ctypes.data,
                                     B.ctypes.data)
    if st != 0:
        raise RuntimeError(f"oracle_assemble_dense failed with status {st}")
    return A, B


def taull(grid_args, energy_args, smr, iaabs=1):
    nl = C.c_int32(0)
    out = np.zeros(2 * 64 * 64)
    smr = np.asfortranarray(smr)
    st = lib().oracle_taull(C.addressof(grid_args.s), C.addressof(energy_args.s), iaabs, smr.ctypes.data,
                            out.ctypes.data, C.byref(nl))
    if st != 0:
        raise RuntimeError(f"oracle_taull failed with status {st}")
    k = nl.value
    t = out[:2 * k * k].view(np.complex128).reshape((k, k), order="F")
    return t.copy()


def newind(grid_args, xyz4, distai, nlmsa, nlmso, nligne, npoint, natome, irregular=False):
    """Row numbering and profile; irregular: FDM_comp's irregular solution
    (both atomic solutions, no outer-sphere rows; nlmso is then unused)."""
    new = np.zeros(npoint + 1, dtype=np.int32)
    newinv = np.zeros(nligne, dtype=np.int32)
    ianew = np.zeros(natome, dtype=np.int32)
    lb1 = np.zeros(nligne, dtype=np.int32)
    lb2 = np.zeros(nligne, dtype=np.int32)
    xyz4 = np.ascontiguousarray(xyz4, dtype=np.float64)
    distai = np.ascontiguousarray(distai, dtype=np.float64)
    nlmsa = np.ascontiguousarray(nlmsa, dtype=np.int32)
    if irregular:
        st = lib().oracle_newind_irregular(C.addressof(grid_args.s), xyz4.ctypes.data, distai.ctypes.data,
                                           nlmsa.ctypes.data, nligne, new.ctypes.data, newinv.ctypes.data,
                                           ianew.ctypes.data, lb1.ctypes.data, lb2.ctypes.data)
    else:
        st = lib().oracle_newind(C.addressof(grid_args.s), xyz4.ctypes.data, distai.ctypes.data, nlmsa.ctypes.data,
                                 nlmso, nligne, new.ctypes.data, newinv.ctypes.data, ianew.ctypes.data,
                                 lb1.ctypes.data, lb2.ctypes.data)
    if st != 0:
        raise RuntimeError("oracle_newind failed")
    return new, newinv, ianew, lb1, lb2


def cbessneur(fnorm, z, lmax):
    b = np.zeros(lmax + 1)
    nm = np.zeros(lmax + 1)
    lib().oracle_cbessneur(float(fnorm), float(z), int(lmax), b.ctypes.data, nm.ctypes.data)
    return b, nm


def invcomp(a):
    a = np.asfortranarray(a, dtype=np.complex128).copy(order="F")
    st = lib().oracle_invcomp(a.shape[0], a.ctypes.data)
    if st != 0:
        raise RuntimeError("oracle_invcomp: singular")
    return a


def mat_solve_c(grid_args, energy_args):
    """Complex solution smr + i smi (nlmso, nligne), Fortran-ordered, plus nnz."""
    n, m = energy_args.nligne, energy_args.nlmso
    smr = np.zeros((m, n), order="F")
    smi = np.zeros((m, n), order="F")
    nnz = C.c_int64(0)
    tf, tt = C.c_double(0), C.c_double(0)
    bad = C.c_int32(0)
    st = lib().oracle_mat_solve_c(C.addressof(grid_args.s), C.addressof(energy_args.s), smr.ctypes.data,
                                  smi.ctypes.data, C.byref(nnz), C.byref(tf), C.byref(tt), C.byref(bad))
    if st != 0:
        raise RuntimeError(f"oracle_mat_solve_c failed with status {st} (row {bad.value})")
    return smr + 1j * smi, dict(nnz=nnz.value, time_fill=tf.value, time_tria=tt.value)


def assemble_dense_c(grid_args, energy_args):
    n, m = energy_args.nligne, energy_args.nlmso
    A = np.zeros((n, n), dtype=np.complex128, order="F")
    B = np.zeros((m, n), dtype=np.complex128, order="F")
    st = lib().oracle_assemble_dense_c(C.addressof(grid_args.s), C.addressof(energy_args.s), A.ctypes.data,
                                       B.ctypes.data)
    if st != 0:
        raise RuntimeError(f"oracle_assemble_dense_c failed with status {st}")
    return A, B


def taull_c(grid_args, energy_args, x, iaabs=1, symmetrise=True):
    """Taull (nlm, nsp, nlm, nsp) of a complex-basis solution x (nlmso, nligne)."""
    nsp = int(grid_args.d["nspino"])
    nl = C.c_int32(0)
    out = np.zeros(2 * (64 * nsp) ** 2)
    smr = np.asfortranarray(x.real)
    smi = np.asfortranarray(x.imag)
    st = lib().oracle_taull_c(C.addressof(grid_args.s), C.addressof(energy_args.s), iaabs, smr.ctypes.data,
                              smi.ctypes.data, int(bool(symmetrise)), out.ctypes.data, C.byref(nl))
    if st != 0:
        raise RuntimeError(f"oracle_taull_c failed with status {st}")
    k = nl.value
    t = out[:2 * (k * nsp) ** 2].view(np.complex128).reshape((k, nsp, k, nsp), order="F")
    return t.copy()


def tau_ri(grid_args, reg_args, x_reg, irr_args, x_irr, iaabs=1):
    """Tau_RI (nlm, nsp, nlm, nsp, 2) of FDM_comp from the regular solution
    x_reg and the irregular one x_irr (each (nlmso, nligne) complex)."""
    nsp = int(grid_args.d["nspino"])
    nl = C.c_int32(0)
    out = np.zeros(4 * (64 * nsp) ** 2)
    a = [np.asfortranarray(v) for v in (x_reg.real, x_reg.imag, x_irr.real, x_irr.imag)]
    st = lib().oracle_tau_ri(C.addressof(grid_args.s), C.addressof(reg_args.s), a[0].ctypes.data, a[1].ctypes.data,
                             C.addressof(irr_args.s), a[2].ctypes.data, a[3].ctypes.data, iaabs, out.ctypes.data,
                             C.byref(nl))
    if st != 0:
        raise RuntimeError(f"oracle_tau_ri failed with status {st}")
    k = nl.value
    t = out[:4 * (k * nsp) ** 2].view(np.complex128).reshape((k, nsp, k, nsp, 2), order="F")
    return t.copy()


def cbessneu(fnorm, z, lmax):
    """Complex fnorm * j_l(z), fnorm * n_l(z), l = 0..lmax, for complex z."""
    b = np.zeros(lmax + 1, dtype=np.complex128)
    nm = np.zeros(lmax + 1, dtype=np.complex128)
    lib().oracle_cbessneu(float(np.real(fnorm)), float(np.imag(fnorm)), float(np.real(z)), float(np.imag(z)),
                          int(lmax), b.ctypes.data, nm.ctypes.data)
    return b, nm


def assemble_csr(grid_args, energy_args, complex_=False):
    """(scipy.sparse.csr_matrix A (nligne x nligne), B (nlmso, nligne) F-ordered)
    assembled row by row with calcMatRow (real, or complex when complex_)."""
    import scipy.sparse as sp
    n, m = energy_args.nligne, energy_args.nlmso
    f = lib().oracle_assemble_csr_c if complex_ else lib().oracle_assemble_csr
    rowptr = np.zeros(n + 1, dtype=np.int64)
    st = f(C.addressof(grid_args.s), C.addressof(energy_args.s), rowptr.ctypes.data, None, None, None)
    if st != 0:
        raise RuntimeError(f"oracle assembly failed with status {st}")
    nnz = int(rowptr[-1])
    col = np.zeros(nnz, dtype=np.int32)
    dt = np.complex128 if complex_ else np.float64
    val = np.zeros(nnz, dtype=dt)
    B = np.zeros((m, n), dtype=dt, order="F")
    st = f(C.addressof(grid_args.s), C.addressof(energy_args.s), rowptr.ctypes.data, col.ctypes.data,
           val.ctypes.data, B.ctypes.data)
    if st != 0:
        raise RuntimeError(f"oracle assembly failed with status {st}")
    return sp.csr_matrix((val, col, rowptr), shape=(n, n)), B


def backward_error(A, B, X):
    """Normwise backward error max_c ||b_c - A x_c||_inf / (||A||_inf ||x_c||_inf + ||b_c||_inf)
    for X, B of shape (nrhs, n) (the smr layout) and a sparse or dense A."""
    R = B.T - A @ X.T
    nA = float(abs(A).sum(axis=1).max())
    num = np.abs(R).max(axis=0)
    den = nA * np.abs(X.T).max(axis=0) + np.abs(B.T).max(axis=0)
    return float((num / den).max())
