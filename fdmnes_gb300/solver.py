"""Host-side interface to libfdmgpu.so, mirroring the reference's mat_solve path.

``FdmSolver(structure)`` uploads the energy-independent arguments once
(``fdmgpu_create``).  ``mat_solve`` is the drop-in for the reference's
``mat_solve`` (source/mat_solve_gaussian.f90:5): it returns ``smr`` with the
reference's shape (nlmso, nligne), column-major.  ``spectrum`` is the batched
path of ``mat`` (source/mat.f90:5-733): all energies in one launch sequence,
returning the absorber's Taull per energy.

There is no CPU fallback: if the CUDA library is missing or no GPU is visible
the constructor raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import List, Sequence, Tuple

import numpy as np

from . import abi
from . import cluster as CL

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfdmgpu.so")

PREC = {"fp64": 0, "mixed": 1}
STATUS = {0: "OK", 1: "ERR_ARG", 2: "ERR_UNSUPPORTED", 3: "ERR_CUDA", 4: "ERR_ZERO_PIVOT",
          5: "ERR_NOT_CONVERGED", 6: "ERR_NOMEM"}

_lib = None


class FdmError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


def load_library(path: str = LIB_PATH):
    """Load libfdmgpu.so and declare the C-ABI of include/fdmgpu.h."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with fdmnes_gb300.build.build()")
    L = C.CDLL(path)
    vp = C.c_void_p
    L.fdmgpu_version.restype = C.c_char_p
    L.fdmgpu_last_error.restype = C.c_char_p
    L.fdmgpu_create.argtypes = [vp, C.POINTER(vp)]
    L.fdmgpu_create.restype = C.c_int
    L.fdmgpu_destroy.argtypes = [vp]
    L.fdmgpu_destroy.restype = None
    L.fdmgpu_mat_solve.argtypes = [vp, vp, C.c_int32, vp, vp, vp]
    L.fdmgpu_mat_solve.restype = C.c_int
    L.fdmgpu_get_solver_params.argtypes = [C.POINTER(C.c_int32), C.c_char_p]
    L.fdmgpu_get_solver_params.restype = None
    L.fdmgpu_set_residual_mode.argtypes = [vp, C.c_int32]
    L.fdmgpu_set_refinement.argtypes = [vp, C.c_int32, C.c_int32]
    L.fdmgpu_set_refinement.restype = C.c_int
    L.fdmgpu_set_escalation.argtypes = [vp, C.c_int32]
    L.fdmgpu_set_escalation.restype = C.c_int
    L.fdmgpu_set_tolerance.argtypes = [vp, C.c_double, C.c_double]
    L.fdmgpu_set_tolerance.restype = C.c_int
    L.fdmgpu_set_autotune.argtypes = [vp, C.c_int32]
    L.fdmgpu_set_autotune.restype = C.c_int
    L.fdmgpu_set_factor_mode.argtypes = [vp, C.c_int32]
    L.fdmgpu_set_factor_mode.restype = C.c_int
    L.fdmgpu_measure_pipe_peaks.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.fdmgpu_measure_pipe_peaks.restype = C.c_int
    L.fdmgpu_batch_inputs.argtypes = [vp, C.c_int32, vp, vp, vp]
    L.fdmgpu_batch_inputs.restype = C.c_int
    L.fdmgpu_set_radial.argtypes = [vp, vp]
    L.fdmgpu_set_radial.restype = C.c_int
    L.fdmgpu_batch_xanes.argtypes = [vp, vp, vp, C.c_int32, vp, vp, vp, vp]
    L.fdmgpu_batch_xanes.restype = C.c_int
    L.fdmgpu_set_memory_budget.argtypes = [vp, C.c_double]
    L.fdmgpu_set_memory_budget.restype = C.c_int
    L.fdmgpu_set_df64_engine.argtypes = [vp, C.c_int32]
    L.fdmgpu_set_df64_engine.restype = C.c_int
    L.fdmgpu_set_solve_order.argtypes = [vp, C.c_int32]
    L.fdmgpu_set_solve_order.restype = C.c_int
    L.fdmgpu_set_tile_engine.argtypes = [vp, C.c_int32]
    L.fdmgpu_set_tile_engine.restype = C.c_int
    L.fdmgpu_get_tuning.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.fdmgpu_get_tuning.restype = C.c_int
    L.fdmgpu_set_residual_mode.restype = C.c_int
    L.fdmgpu_batch_begin.argtypes = [vp, C.c_int32, C.c_int32]
    L.fdmgpu_batch_add.argtypes = [vp, vp, C.c_int32]
    L.fdmgpu_batch_run.argtypes = [vp, vp]
    L.fdmgpu_batch_rerun.argtypes = [vp, vp]
    L.fdmgpu_batch_taull.argtypes = [vp, C.c_int32, vp, C.POINTER(C.c_int32)]
    L.fdmgpu_batch_solution.argtypes = [vp, C.c_int32, vp]
    L.fdmgpu_batch_stats.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_double),
                                     C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    L.fdmgpu_batch_vjp.argtypes = [vp, vp, vp, C.POINTER(C.c_double)]
    L.fdmgpu_batch_taull_all.argtypes = [vp, vp, C.c_int64]
    L.fdmgpu_batch_taull_all.restype = C.c_int
    L.fdmgpu_batch_tau_ri.argtypes = [vp, C.c_int32, C.c_int32, vp, C.POINTER(C.c_int32)]
    L.fdmgpu_batch_tau_ri.restype = C.c_int
    L.fdmgpu_batch_add_site.argtypes = [vp, vp, vp, C.c_int32]
    L.fdmgpu_batch_add_site.restype = C.c_int
    L.fdmgpu_update_grid_values.argtypes = [vp, vp]
    L.fdmgpu_update_grid_values.restype = C.c_int
    L.fdmgpu_batch_adjoint_dot.argtypes = [vp, vp, C.c_int32, vp]
    L.fdmgpu_batch_adjoint_dot.restype = C.c_int
    for f in ("fdmgpu_batch_begin", "fdmgpu_batch_add", "fdmgpu_batch_run", "fdmgpu_batch_rerun", "fdmgpu_batch_taull",
              "fdmgpu_batch_solution", "fdmgpu_batch_stats", "fdmgpu_batch_vjp"):
        getattr(L, f).restype = C.c_int
    _lib = L
    return L


def _check(st: int):
    if st != 0:
        raise FdmError(st, load_library().fdmgpu_last_error().decode())


def measure_pipe_peaks() -> dict:
    """FP32 and FP64 FMA rates of the current GPU in TFLOP/s (measured)."""
    f32, f64 = C.c_double(0), C.c_double(0)
    _check(load_library().fdmgpu_measure_pipe_peaks(C.byref(f32), C.byref(f64)))
    return {"fp32_tflops": f32.value, "fp64_tflops": f64.value}


def info_dict(info: abi.FdmInfo) -> dict:
    return {k: getattr(info, k) for k, _ in abi.FdmInfo._fields_}


class FdmSolver:
    """One device handle holding the static structure of a cluster."""

    def __init__(self, st):
        """st: a cluster.Structure, or the grid_dict() arrays of one."""
        self.lib = load_library()
        self.st = st
        self.grid_args = abi.GridArgs(st)
        h = C.c_void_p()
        _check(self.lib.fdmgpu_create(C.addressof(self.grid_args.s), C.byref(h)))
        self.h = h
        self._batch_args: List[abi.EnergyArgs] = []

    def set_residual(self, mode: str):
        """Residual arithmetic of the mixed path: 'df64' (default) or 'fp64'."""
        _check(self.lib.fdmgpu_set_residual_mode(self.h, {"fp64": 0, "df64": 1}[mode]))

    def set_refinement(self, mode: str = "gmres", krylov_dim: int = 12):
        """Refinement of the mixed path: 'classic' (default), 'recurrence' or 'gmres'."""
        _check(self.lib.fdmgpu_set_refinement(self.h, {"classic": 0, "gmres": 1, "recurrence": 2}[mode], krylov_dim))

    def set_escalation(self, mode: str = "df64"):
        """Re-solve of energies the FP32 factors cannot refine: 'df64_f32' (the library's
        default: double-float factors rounded to FP32, FP32 refinement), 'df64'
        (double-float refinement steps), 'df64_overlap', 'wide_df64' or 'fp64'."""
        _check(self.lib.fdmgpu_set_escalation(self.h, {"fp64": 0, "df64": 1, "df64_overlap": 2,
                                                       "wide_df64": 3, "df64_f32": 4}[mode]))

    def set_tolerance(self, tol: float = 0.0, tol_accept: float = 0.0):
        """Refinement stop (max|dx|/max|x|) and the stalled-but-accepted level; 0 = default."""
        _check(self.lib.fdmgpu_set_tolerance(self.h, tol, tol_accept))

    def set_factor_mode(self, mode: str = "fp32"):
        """Accumulation of the mixed path's FP32 factor: 'fp32' (default) or
        'wide_atom' (double-float sums at the atom-harmonic steps)."""
        _check(self.lib.fdmgpu_set_factor_mode(self.h, {"fp32": 0, "wide_atom": 1, "wide_all": 2}[mode]))

    def set_radial(self):
        """Upload the structure's radial tables, so that energies added with
        functions=False inputs (cluster.energy_inputs(..., functions=False))
        get phiato, Bessel and Neumann generated on the device."""
        self.radial_args = abi.RadialArgs(self.st)
        _check(self.lib.fdmgpu_set_radial(self.h, C.addressof(self.radial_args.s)))

    def batch_inputs(self, k: int, nlmagm: int, lmaxso: int):
        """phiato (nbtm, nlmagm, natome), Besselr and Neumanr (nsort, lmaxso+1)
        of energy k of the last run as the device holds them."""
        g = self.st.grid
        phi = np.zeros((g.nbtm, nlmagm, self.st.natome), order="F")
        bs = np.zeros((g.nsort, lmaxso + 1), order="F")
        nm = np.zeros((g.nsort, lmaxso + 1), order="F")
        _check(self.lib.fdmgpu_batch_inputs(self.h, k, phi.ctypes.data, bs.ctypes.data, nm.ctypes.data))
        return phi, bs, nm

    def set_memory_budget(self, nbytes: float = 0.0):
        """Device bytes a batch may take before it runs in chunks (0: 85% of the device)."""
        _check(self.lib.fdmgpu_set_memory_budget(self.h, float(nbytes)))

    def set_df64_engine(self, engine: str = "tcgen05"):
        """Double-float trailing update of the escalation factor on the FP32
        pipes ("simt") or on the tensor cores through integer slices ("tcgen05")."""
        _check(self.lib.fdmgpu_set_df64_engine(self.h, {"simt": 0, "tcgen05": 1}[engine]))

    def set_solve_order(self, order: str = "rows"):
        """Refinement solves of mixed batches step by step ("columns") or row by row ("rows")."""
        _check(self.lib.fdmgpu_set_solve_order(self.h, {"columns": 0, "rows": 1}[order]))

    def set_tile_engine(self, engine: str = "tcgen05"):
        """FP32 tile updates of mixed batches on the FP32 pipes ("simt"), the
        same with the streamed operand tiles staged by bulk copies
        ("simt_stream", the library's default, also the double-float updates),
        on the tensor cores as
        split-TF32 products ("tcgen05"), or the factor's trailing update only
        on the tensor cores ("tcgen05_factor")."""
        _check(self.lib.fdmgpu_set_tile_engine(self.h, {"simt": 0, "tcgen05": 1, "tcgen05_factor": 2,
                                                        "simt_stream": 3}[engine]))

    def set_autotune(self, on: bool = True):
        _check(self.lib.fdmgpu_set_autotune(self.h, 1 if on else 0))

    def tuning(self, precision: str = "mixed") -> dict:
        """Trailing-update layout chosen by the autotuner and its two trial times."""
        t, a, b = C.c_int32(0), C.c_double(0), C.c_double(0)
        _check(self.lib.fdmgpu_get_tuning(self.h, PREC[precision], C.byref(t), C.byref(a), C.byref(b)))
        return {"trailing_threads": t.value, "trial_ms_64": a.value, "trial_ms_128": b.value}

    def close(self):
        if getattr(self, "h", None):
            self.lib.fdmgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def mat_solve(self, ei: CL.EnergyInputs, ri: CL.RowIndex, precision: str = "fp64") -> Tuple[np.ndarray, dict]:
        return self.mat_solve_args(abi.EnergyArgs(self.st, ei, ri), precision)

    def mat_solve_args(self, ea: abi.EnergyArgs, precision: str = "fp64") -> Tuple[np.ndarray, dict]:
        """mat_solve on prepared arguments; returns smr (nlmso, nligne) and diagnostics."""
        smr = np.zeros((ea.nlmso, ea.nligne), order="F")
        info = abi.FdmInfo()
        st = self.lib.fdmgpu_mat_solve(self.h, C.addressof(ea.s), PREC[precision], smr.ctypes.data, None,
                                       C.addressof(info))
        if st not in (0, 5):
            _check(st)
        d = info_dict(info)
        d["converged"] = st == 0
        return smr, d

    def mat_solve_complex(self, ea: abi.EnergyArgs, precision: str = "fp64") -> Tuple[np.ndarray, dict]:
        """mat_solve of a complex (Cal_comp) problem: the solution smr + i smi
        (nlmso, nligne) and diagnostics.  The handle's grid must carry the
        problem's nspino (``complex_path.grid_dict``)."""
        smr = np.zeros((ea.nlmso, ea.nligne), order="F")
        smi = np.zeros((ea.nlmso, ea.nligne), order="F")
        info = abi.FdmInfo()
        _check(self.lib.fdmgpu_mat_solve(self.h, C.addressof(ea.s), PREC[precision], smr.ctypes.data,
                                         smi.ctypes.data, C.addressof(info)))
        return smr + 1j * smi, info_dict(info)

    def taull_c(self, k: int, nspino: int) -> np.ndarray:
        """Taull of a complex batch energy as (nlm, nspino, nlm, nspino), indexed
        by L^2 + L + m and spin on both sides."""
        t = self.taull(k)
        n = t.shape[0] // nspino
        return t.reshape((n, nspino, n, nspino), order="F").copy()

    def spectrum_begin(self, precision: str, n: int):
        _check(self.lib.fdmgpu_batch_begin(self.h, PREC[precision], n))
        self._batch_args = []

    def spectrum_add(self, ei: CL.EnergyInputs, ri: CL.RowIndex, iaabs: int = 1):
        self.spectrum_add_args(abi.EnergyArgs(self.st, ei, ri), iaabs)

    def spectrum_add_args(self, ea: abi.EnergyArgs, iaabs: int = 1, site: "FdmSolver" = None):
        """Add one energy; with site, an energy of another absorbing site (its own
        FdmSolver and grid) joins this batch."""
        if site is None or site is self:
            _check(self.lib.fdmgpu_batch_add(self.h, C.addressof(ea.s), iaabs))
        else:
            _check(self.lib.fdmgpu_batch_add_site(self.h, site.h, C.addressof(ea.s), iaabs))
            self._sites = getattr(self, "_sites", []) + [site]
        self._batch_args.append(ea)

    def spectrum_add_site(self, site: "FdmSolver", ei: CL.EnergyInputs, ri: CL.RowIndex, iaabs: int = 1):
        self.spectrum_add_args(abi.EnergyArgs(site.st, ei, ri), iaabs, site)

    def spectrum_run(self) -> dict:
        """Run the batch.  Energies whose refinement missed its tolerance are
        reported in ``info['not_converged']`` (their results stay readable)."""
        info = abi.FdmInfo()
        st = self.lib.fdmgpu_batch_run(self.h, C.addressof(info))
        if st not in (0, 5):
            _check(st)
        d = info_dict(info)
        d["not_converged"] = [k for k in range(len(self._batch_args) or 0)
                              if self.lib.fdmgpu_batch_stats(self.h, k, None, None, None, None) == 5]
        return d

    def spectrum_rerun(self) -> dict:
        """Run the last batch again on the inputs already in device memory."""
        info = abi.FdmInfo()
        st = self.lib.fdmgpu_batch_rerun(self.h, C.addressof(info))
        if st not in (0, 5):
            _check(st)
        return info_dict(info)

    def taull(self, k: int) -> np.ndarray:
        nl = C.c_int32(0)
        _check(self.lib.fdmgpu_batch_taull(self.h, k, None, C.byref(nl)))
        out = np.zeros(2 * nl.value * nl.value)
        _check(self.lib.fdmgpu_batch_taull(self.h, k, out.ctypes.data, C.byref(nl)))
        return out.view(np.complex128).reshape((nl.value, nl.value), order="F").copy()

    def tau_ri(self, k_reg: int, k_irr: int, nspino: int) -> np.ndarray:
        """Tau_RI of FDM_comp from the batch's regular solution k_reg and
        irregular solution k_irr: (nlm, nspino, nlm, nspino, 2), indexed like
        taull_c, the last index i_RI (regular, irregular atomic solution)."""
        nl = C.c_int32(0)
        _check(self.lib.fdmgpu_batch_tau_ri(self.h, k_reg, k_irr, None, C.byref(nl)))
        out = np.zeros(4 * nl.value * nl.value)
        _check(self.lib.fdmgpu_batch_tau_ri(self.h, k_reg, k_irr, out.ctypes.data, C.byref(nl)))
        n = nl.value // nspino
        return out.view(np.complex128).reshape((n, nspino, n, nspino, 2), order="F").copy()

    def taull_all(self) -> List[np.ndarray]:
        """Taull of every energy of the last batch, in one device-to-host copy."""
        sizes = []
        for k in range(len(self._batch_args)):
            nl = C.c_int32(0)
            _check(self.lib.fdmgpu_batch_taull(self.h, k, None, C.byref(nl)))
            sizes.append(nl.value)
        out = np.zeros(2 * sum(n * n for n in sizes))
        _check(self.lib.fdmgpu_batch_taull_all(self.h, out.ctypes.data, out.size))
        res, o = [], 0
        for n in sizes:
            res.append(out[o:o + 2 * n * n].view(np.complex128).reshape((n, n), order="F").copy())
            o += 2 * n * n
        return res

    def xanes(self, energies, half_width=0.78, width_per_input: bool = False, weight=None,
              tensor: bool = False):
        """Dipole absorption sigma(E) of the last batch and its Lorentzian
        convolution, computed on the device in FP64 (fdmgpu_batch_xanes).
        Returns (sigma, sigma_conv) or (sigma, sigma_conv, tensor (n, 3, 3))."""
        E = np.ascontiguousarray(energies, dtype=np.float64)
        n = len(E)
        hw = np.ascontiguousarray(np.broadcast_to(np.asarray(half_width, dtype=np.float64), (n,)))
        w = None if weight is None else np.ascontiguousarray(weight, dtype=np.float64)
        sig = np.zeros(n)
        conv = np.zeros(n)
        ten = np.zeros((n, 3, 3)) if tensor else None
        _check(self.lib.fdmgpu_batch_xanes(self.h, E.ctypes.data, hw.ctypes.data, int(width_per_input),
                                           None if w is None else w.ctypes.data, sig.ctypes.data,
                                           conv.ctypes.data, None if ten is None else ten.ctypes.data))
        return (sig, conv, ten) if tensor else (sig, conv)

    def solution(self, k: int, nlmso: int, nligne: int) -> np.ndarray:
        smr = np.zeros((nlmso, nligne), order="F")
        _check(self.lib.fdmgpu_batch_solution(self.h, k, smr.ctypes.data))
        return smr

    def stats(self, k: int) -> Tuple[int, float, bool, int]:
        """Refinement iterations, final relative correction, whether energy k was
        solved again in FP64 (precision escalation) and its GMRES steps."""
        it = C.c_int32(0)
        r = C.c_double(0)
        fb = C.c_int32(0)
        inner = C.c_int32(0)
        st = self.lib.fdmgpu_batch_stats(self.h, k, C.byref(it), C.byref(r), C.byref(fb), C.byref(inner))
        if st not in (0, 5):
            _check(st)
        return it.value, r.value, bool(fb.value), inner.value

    def vjp(self, g_taull: Sequence[np.ndarray]) -> Tuple[np.ndarray, float]:
        """Gradient of L with respect to the grid potential Vr, given the
        cotangents g_taull[k] = dL/d(Im Taull_k) (nlm x nlm real) of the energies
        of the last batch (FP64 or mixed).  Returns (dL/dVr of shape
        (npoint, nspin), device ms)."""
        flat = np.concatenate([np.asarray(g, dtype=np.float64).ravel(order="F") for g in g_taull])
        g = self.st.grid
        grad = np.zeros((g.npoint, self.st.nspin), order="F")
        ms = C.c_double(0)
        _check(self.lib.fdmgpu_batch_vjp(self.h, flat.ctypes.data, grad.ctypes.data, C.byref(ms)))
        return grad, ms.value

    def update_grid_values(self, st) -> None:
        """Switch the handle to the real-valued grid tables of st (same integer
        structure).  The energy arguments built afterwards use st."""
        ga = abi.GridArgs(st)
        _check(self.lib.fdmgpu_update_grid_values(self.h, C.addressof(ga.s)))
        self.st = st
        self.grid_args = ga

    def adjoint_dot(self, items: Sequence[Tuple[CL.EnergyInputs, CL.RowIndex]]) -> np.ndarray:
        """Per energy, Lambda^T (B' - A' X) with A', B' assembled from items (one
        per energy of the batch, same row structure) and the X, Lambda of the
        last run + vjp."""
        args = [abi.EnergyArgs(self.st, ei, ri) for ei, ri in items]
        arr = (C.c_void_p * len(args))(*[C.addressof(a.s) for a in args])
        out = np.zeros(len(args))
        _check(self.lib.fdmgpu_batch_adjoint_dot(self.h, arr, len(args), out.ctypes.data))
        return out

    def spectrum(self, items: Sequence[Tuple[CL.EnergyInputs, CL.RowIndex]], precision: str = "mixed",
                 iaabs: int = 1):
        self.spectrum_begin(precision, len(items))
        for ei, ri in items:
            self.spectrum_add(ei, ri, iaabs)
        info = self.spectrum_run()
        return self.taull_all(), info
