"""One batched mixed-precision spectrum step inside an NVTX range, for profilers.

    python -m fdmnes_gb300.profile_step [--energies N | --elist E1,E2,...]
        [--tile-engine simt|simt_stream|tcgen05|tcgen05_factor] [--df64-engine simt|tcgen05]
        [--factor-mode fp32|wide_atom|wide_all] [--escalation df64|df64_f32|wide_df64|fp64]
        [--solve-order columns|rows]

The fcc Cu cluster of the benchmark (13 atoms, FDM radius 3.0 A, step 0.25 A)
is planned and run twice (plan, graph capture, warm caches); the third run is
bracketed by the NVTX range "timed", so that

    ncu --nvtx --nvtx-include "timed/" -k regex:<kernel> -c <n> ... \\
        python -m fdmnes_gb300.profile_step --energies 11

captures only that step's launches (the kernels of the refinement loop's
graph body are not attributed to the range; for a launch list with them, skip
the first two runs' launches, ``kernels_per_run`` in the printed line, with
``-s`` and capture the third run's count with ``-c``).  Inputs (phiato, Bessel and Neumann
functions) are generated on the device, as in the benchmark.  The energies
default to an even grid over -5..35 eV; --elist picks exact ones (the energies
above about 22 eV are those whose FP32 refinement stalls and escalates).
"""
from __future__ import annotations

import argparse
import json

import numpy as np


def main(argv=None) -> dict:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--energies", type=int, default=401)
    ap.add_argument("--elist", default="", help="comma-separated energies in eV (overrides --energies)")
    ap.add_argument("--tile-engine", default="simt_stream", choices=["simt", "simt_stream", "tcgen05", "tcgen05_factor"])
    ap.add_argument("--df64-engine", default="tcgen05", choices=["simt", "tcgen05"])
    ap.add_argument("--factor-mode", default="fp32", choices=["fp32", "wide_atom", "wide_all"])
    ap.add_argument("--escalation", default="df64_f32", choices=["df64", "df64_f32", "wide_df64", "fp64"])
    ap.add_argument("--solve-order", default="columns", choices=["columns", "rows"])
    a = ap.parse_args(argv)

    import torch
    from . import build, cluster as CL, xanes
    build.build()
    from .solver import FdmSolver

    if a.elist:
        E = np.array([float(x) for x in a.elist.split(",")])
    elif a.energies == 401:
        E = CL.energy_grid(-5.0, 35.0, 0.1)
    else:
        E = np.linspace(-5.0, 35.0, a.energies)
    st = CL.cu_structure()
    items = xanes.spectrum_inputs(st, E, functions=False)
    sv = FdmSolver(st)
    sv.set_radial()
    sv.set_tolerance(1e-8, 1e-6)
    sv.set_tile_engine(a.tile_engine)
    sv.set_df64_engine(a.df64_engine)
    sv.set_factor_mode(a.factor_mode)
    sv.set_escalation(a.escalation)
    sv.set_solve_order(a.solve_order)
    sv.spectrum_begin("mixed", len(E))
    for ei, ri in items:
        sv.spectrum_add(ei, ri)
    n1 = int(sv.spectrum_run()["n_kernels"])
    n2 = int(sv.spectrum_rerun()["n_kernels"])
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("timed")
    info = sv.spectrum_rerun()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    out = {"energies": len(E), "n_kernels": int(info["n_kernels"]), "kernels_per_run": [n1, n2, int(info["n_kernels"])],
           "n_fallback": int(info["n_fallback"]),
           "ms": info["ms_assemble"] + info["ms_factor"] + info["ms_solve"] + info["ms_refine"],
           "phases_ms": {k: info[k] for k in ("ms_assemble", "ms_factor", "ms_solve", "ms_refine",
                                              "ms_refine_loop", "ms_escalate_factor")}}
    print(json.dumps(out), flush=True)
    sv.close()
    return out


if __name__ == "__main__":
    main()
