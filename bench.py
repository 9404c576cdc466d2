#!/usr/bin/env python3
"""Benchmark: FDM energy points per second on one GB300.

Workload (the batched Cu configuration): fcc Cu, 13-atom cluster, FDM sphere
3.0 A, grid step 0.25 A, no symmetry reduction, 401 energies from -5 to 35 eV
in steps of 0.1 eV, all solved in one batched launch sequence (assembly,
FP32 profile LU with tile-local pivoting, refinement of the FP64 solution,
Taull contraction).  One "step" is one full spectrum.

* value  - energies / s with the per-energy inputs already in HBM
           (fdmgpu_batch_rerun), CUDA events on the solver's stream;
* e2e    - energies / s through the C-ABI from host buffers: per step the
           inputs are packed and copied host -> device and every Taull is
           copied back (fdmgpu_batch_begin/add/run/taull);
* plain_fp64 - the same spectrum through the plain FP64 profile solve
           (the correctness path) for the mixed-vs-FP64 comparison;
* cpu_baseline - the CPU restatement of the reference's Gaussian solver
           (oracle/) timed on the host cores on a sample of energies, one
           energy per core as the reference's MPI energy loop does.

``--impl reference`` times only that CPU restatement (the reference itself is
Fortran and no Fortran compiler exists on either machine).
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

E_MIN, E_MAX, E_STEP = -5.0, 35.0, 0.1
METRIC = "FDM energy-points/sec on 1 GB300, mixed+batched vs plain FP64, at <=1e-6 rel error"
WORKLOAD_CU401 = ("Cu fcc a=3.61 A, 13-atom cluster, FDM radius 3.0 A, step 0.25 A, C1, "
                  "401 energies -5..35 eV step 0.1 eV, batched mixed precision")


def _peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"fdm_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                c = [x.strip() for x in line.split(",")]
                if len(c) < 9:
                    continue
                try:
                    sm.append(float(c[1]))
                    smax.append(float(c[2]))
                except ValueError:
                    continue
                for name, v in zip(names, c[5:9]):
                    if v.lower() == "active":
                        reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- CPU baseline
_W = {}


def _oracle_init():
    sys.path.insert(0, HERE)
    import oracle
    oracle.use_timed_build(True)  # the -O3 build of the restatement (the reference's level)
    from fdmnes_gb300 import abi, cluster as CL
    st = CL.cu_structure()
    _W["st"], _W["ga"] = st, abi.GridArgs(st)


def _oracle_worker(args):
    """One energy of the CPU restatement: the reference's per-rank work (mat_solve + Taull)."""
    energy, = args
    from fdmnes_gb300 import abi, cluster as CL
    import oracle
    st, ga = _W["st"], _W["ga"]
    ei = CL.energy_inputs(st, energy)
    ri = CL.newind(st, ei.nlmsa, ei.nlmso)
    ea = abi.EnergyArgs(st, ei, ri)
    t0 = time.perf_counter()
    X, _ = oracle.mat_solve(ga, ea)
    oracle.taull(ga, ea, X)
    return time.perf_counter() - t0


def cpu_energy_sample(n_energies: int, offset: int = 0):
    """n energies spread over the 401-point grid -5..35 eV (step 0.1 eV),
    shifted by `offset` grid points so that successive samples cover different
    energies of the spectrum."""
    grid = np.round(np.arange(401) * E_STEP + E_MIN, 10)
    idx = (np.round(np.linspace(0, 400, n_energies)).astype(int) + offset) % 401
    return grid[idx]


def cpu_baseline(n_energies: int, offset: int = 0):
    """Oracle restatement (-O3 build) on the host cores, one energy per process (spawned)."""
    import oracle
    oracle.build()
    cores = min(os.cpu_count() or 1, n_energies)
    energies = cpu_energy_sample(n_energies, offset)
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores, initializer=_oracle_init) as pool:
        per = pool.map(_oracle_worker, [(float(e),) for e in energies], chunksize=1)
    # the energies run concurrently, one per core, as the reference's MPI ranks do
    # (source/fdm.f90:3484-3497): a spectrum of n energies takes the slowest rank's time
    wall = max(per)
    return {"value": n_energies / wall, "unit": "energies/s", "cores": cores, "kind": "port",
            "build": "C++ restatement of mat_solve_gaussian + calcMatRow + Taull, g++ -O3",
            "sample": f"{n_energies} of the 401 Cu energies {E_MIN}..{E_MAX} eV (grid offset {offset}), "
                      f"one per process; single-energy solve {min(per):.2f}-{max(per):.2f} s",
            "wall_s": wall}


def _superlu_worker(args):
    """One energy through SciPy's SuperLU (splu, COLAMD ordering) on the same
    assembled matrix: a labelled stand-in for the reference's MUMPS backend
    (source/mat_solve_mumps.f90), which is not available here."""
    energy, = args
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    from fdmnes_gb300 import abi, cluster as CL
    import oracle
    st, ga = _W["st"], _W["ga"]
    ei = CL.energy_inputs(st, energy)
    ri = CL.newind(st, ei.nlmsa, ei.nlmso)
    ea = abi.EnergyArgs(st, ei, ri)
    A, B = oracle.assemble_dense(ga, ea)
    As = sp.csc_matrix(A)
    t0 = time.perf_counter()
    lu = sla.splu(As)
    lu.solve(np.ascontiguousarray(B.T))
    return time.perf_counter() - t0


def superlu_standin(n_energies: int):
    import oracle
    oracle.build()
    cores = min(os.cpu_count() or 1, n_energies)
    energies = np.linspace(E_MIN, E_MAX, n_energies)
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores, initializer=_oracle_init) as pool:
        per = pool.map(_superlu_worker, [(float(e),) for e in energies], chunksize=1)
    wall = max(per)
    return {"value": n_energies / wall, "unit": "energies/s", "cores": cores,
            "kind": "SciPy SuperLU stand-in for MUMPS (not the reference)",
            "sample": f"{n_energies} Cu energies {E_MIN}..{E_MAX} eV, one per process, factor + solve only; "
                      f"single-energy {min(per):.2f}-{max(per):.2f} s"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n = max(1, min(os.cpu_count() or 1, 16))
    cfg = {"workload": WORKLOAD_CU401, "energies": 401, "sample_energies_per_step": n,
           "sample": "each step solves n energies of the 401-point spectrum, one per host core; successive "
                     "steps take successive grid offsets"}
    times = []
    for step in range(args.warmup + args.steps):
        cb = cpu_baseline(n, offset=step)
        if step >= args.warmup:
            times.append(cb)
    v = statistics.median([c["value"] for c in times])
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "energies/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * n / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": v, "unit": "energies/s", "cores": times[0]["cores"], "kind": "port",
                             "build": times[0]["build"], "sample": times[0]["sample"]},
            "e2e": {"value": v, "unit": "energies/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU arm
def _traffic(kernel: str):
    """DRAM bytes per launch of `kernel` at the benchmark's size from the
    committed ncu capture summary (profiles/traffic.json: dram__bytes_read.sum
    + dram__bytes_write.sum per launch of a small case, scaled by the problems
    a launch processes), or None."""
    try:
        with open(os.path.join(HERE, "profiles", "traffic.json")) as f:
            t = json.load(f).get(kernel)
    except (OSError, ValueError):
        return None
    return t.get("bytes") if isinstance(t, dict) else t


def run_gpu(args):
    import torch
    import torch.distributed as dist
    from fdmnes_gb300 import build as B, cluster as CL, xanes
    from fdmnes_gb300.solver import FdmSolver, measure_pipe_peaks

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    B.build()

    step = E_STEP if args.energies == 401 else (E_MAX - E_MIN) / max(args.energies - 1, 1)
    # N ranks: an N times finer spectrum, dealt round-robin over the ranks as the
    # reference's MPI energy loop does (source/fdm.f90:3484-3497); every rank
    # solves its own energies with no device collective (weak scaling)
    from fdmnes_gb300 import shard
    all_energies = CL.energy_grid(E_MIN, E_MAX, step / world)
    mine = shard.energy_shard(len(all_energies), rank, world)
    energies = all_energies[mine]
    n_e = len(energies)
    n_all = len(all_energies)
    st = CL.cu_structure()
    items = xanes.spectrum_inputs(st, energies)                      # host-built phiato / Bessel / Neumann
    items_gen = xanes.spectrum_inputs(st, energies, functions=False)  # generated on the device
    sv = FdmSolver(st)
    sv.set_radial()
    # operating point for the metric's <= 1e-6 cross-section bar: refinement
    # stops at max|dx|/max|x| <= 1e-8 and accepts stalls up to 1e-6; the
    # library default (1e-10) is kept for parity
    TOL, TOL_ACCEPT = 1e-8, 1e-6
    sv.set_tolerance(TOL, TOL_ACCEPT)
    sv.set_factor_mode(args.factor_mode)
    sv.set_tile_engine(args.tile_engine)
    sv.set_df64_engine(args.df64_engine)
    sv.set_escalation(args.escalation)

    def barrier_sync():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

    def max_over_ranks(x):
        if world == 1:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    # plain FP64 reference spectrum (the correctness path), once, on the same
    # device-generated inputs, and its device-resident timing
    t0 = time.perf_counter()
    T64, info64 = sv.spectrum(items_gen, "fp64")
    fp64_wall = time.perf_counter() - t0
    info64 = sv.spectrum_rerun()
    fp64_ms = info64["ms_assemble"] + info64["ms_factor"] + info64["ms_solve"]
    sig64, conv64 = sv.xanes(energies, 0.78)

    # mixed precision spectrum: warm-up (plans, graphs), then timed reruns
    sv.spectrum_begin("mixed", n_e)
    for ei, ri in items_gen:
        sv.spectrum_add(ei, ri)
    info = sv.spectrum_run()
    Tm = sv.taull_all()
    sigm, convm = sv.xanes(energies, 0.78)
    err_conv = float(np.abs(convm - conv64).max() / np.abs(conv64).max())
    err_conv_host = xanes.convolved_relative_error(energies, Tm, T64)
    err_taull = max(float(np.abs(a - b).max() / np.abs(b).max()) for a, b in zip(Tm, T64))
    for _ in range(args.warmup):
        sv.spectrum_rerun()

    clk = ClockSampler()
    clk.start()
    barrier_sync()
    infos = []
    for _ in range(args.steps):
        infos.append(sv.spectrum_rerun())
    barrier_sync()
    # device time of the spectrum: sum of the phases timed by CUDA events on the solver's stream
    dev_ms = [i["ms_assemble"] + i["ms_factor"] + i["ms_solve"] + i["ms_refine"] for i in infos]
    ms_step = max_over_ranks(statistics.mean(dev_ms))
    value = n_all / (ms_step / 1000.0)

    def e2e_run(its, gen: bool):
        """Per step through the C-ABI from host buffers: pack and copy every
        energy's inputs host -> device, run, copy every Taull back."""
        times = []
        h2d = d2h = 0
        for s_ in range(args.steps):
            barrier_sync()
            t0 = time.perf_counter()
            sv.spectrum_begin("mixed", n_e)
            for ei, ri in its:
                sv.spectrum_add(ei, ri)
            sv.spectrum_run()
            out = sv.taull_all()
            barrier_sync()
            times.append(time.perf_counter() - t0)
            if s_ == 0:
                ints = sum(4 * (st.grid.npoint + 1 + 2 * st.natome) for _ in its)
                vr = sum(st.Vr[:, 0].nbytes for _ in its)
                fun = 0 if gen else sum(ei.phiato.nbytes + ei.besselr.nbytes + ei.neumanr.nbytes for ei, _ in its)
                h2d = ints + vr + fun
                d2h = sum(t.nbytes for t in out)
        return max_over_ranks(statistics.mean(times)), h2d, d2h

    e2e_s, h2d, d2h = e2e_run(items_gen, True)
    e2e_host_s, h2d_host, _ = e2e_run(items, False)
    clocks = clk.stop()

    peaks, peak_kind = _peaks()
    last = infos[-1]
    pipes = measure_pipe_peaks()  # FP32 / FP64 FMA rates of this GPU, measured here
    FP32_PIPE_TFLOPS = pipes["fp32_tflops"]

    def roof(flops, ms, kernel, note, traffic_key=None):
        ach = flops / (ms / 1000.0) / 1e12 if ms > 0 else 0.0
        return {"bound": "tensor", "achieved": ach, "peak": peaks["bf16_tflops"], "unit": "TFLOP/s",
                "frac": ach / peaks["bf16_tflops"], "traffic": _traffic(traffic_key) if traffic_key else None,
                "kernel": kernel, "peak_note": f"bf16 dense tensor peak ({peak_kind}); {note}",
                "frac_of_fp32_pipe": ach / FP32_PIPE_TFLOPS}

    # dominant phase of the step (launch list in profiles/): the double-float
    # re-factorisation of the energies FP32 refinement cannot converge
    stream = args.tile_engine == "simt_stream"
    oz = args.df64_engine == "tcgen05"
    panel = "k_diag_inv<dfl> + panel products k_strip<dfl, 3/4>" if stream else "k_diag/k_panel<dfl>"
    if oz:
        esc_kernels = (f"{panel} + integer-slice trailing update k_oz_slice + k_oz_mma (tcgen05.mma kind::f16)",
                       "k_oz_mma")
        esc_note = ("trailing update on the tensor cores: 34 exact bf16 slice products per double-float product; "
                    "flops counted as 2 per double-float multiply-add of the profile")
    else:
        esc_kernels = (f"{panel} + trailing {'strips k_strip<dfl, 0>' if stream else 'k_trailing<dfl>'}",
                       "k_strip<dfl, 0>" if stream else "k_trailing<dfl, 128>")
        esc_note = ("runs on the FP32 pipes, ~12 FP32 instructions per double-float multiply-add; flops counted "
                    "as 2 per multiply-add of the profile")
    roof_main = roof(last["flops_escalate_factor"], last["ms_escalate_factor"],
                     f"double-float escalation factor ({esc_kernels[0]}), one launch sequence per step",
                     esc_note, esc_kernels[1])
    roof_res = roof(last["flops_residual"], last["ms_residual_first"],
                    "k_residual_df, first refinement step (all energies active)",
                    "double-float residual on the FP32 pipes; 2 flops per CSR nonzero per right-hand side",
                    "k_residual_df")
    tc = args.tile_engine in ("tcgen05", "tcgen05_factor")
    fac_kernel = ("k_tc_update<0> (tcgen05 split-TF32)" if tc else
                  "k_strip<float, 0>" if stream else "k_trailing<float, 128>")
    roof_fac = roof(last["flops_factor"], last["ms_factor"],
                    f"FP32 profile LU (k_diag + k_panel + {fac_kernel})",
                    "tensor cores, three TF32 products per FP32 product" if tc else "FP32 SIMT pipes",
                    fac_kernel.split(" (")[0])
    if rank != 0:
        return
    cb = cpu_baseline(min(os.cpu_count() or 1, 16)) if not args.no_cpu else None
    slu = superlu_standin(min(os.cpu_count() or 1, 16)) if not args.no_cpu else None
    line = {
        "metric": METRIC, "value": value, "unit": "energies/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 factor + f64 refinement (df64 residual)", "data": "synthetic",
        "config": {"workload": WORKLOAD_CU401 if world == 1 and args.energies == 401 else
                   "Cu fcc a=3.61 A, 13-atom cluster, FDM radius 3.0 A, step 0.25 A, C1, "
                   f"{n_all} energies -5..35 eV step {step / world:.2g} eV, batched mixed precision",
                   "energies": n_all, "energies_per_gpu": n_e, "e_step_ev": step / world,
                   "nligne": [min(r.nligne for _, r in items), max(r.nligne for _, r in items)],
                   "nrhs": [min(e.nlmso for e, _ in items), max(e.nlmso for e, _ in items)],
                   "inputs": "phiato, Bessel and Neumann generated on the device (fdmgpu_set_radial)",
                   "l2": "working set ~100 GB per step, far above the 126 MB L2 (no flush needed)",
                   "refine_tol": TOL, "refine_tol_accept": TOL_ACCEPT, "factor_mode": args.factor_mode,
                   "tile_engine": args.tile_engine, "df64_engine": args.df64_engine, "escalation": args.escalation,
                   "autotune": {"mixed": sv.tuning("mixed"), "fp64": sv.tuning("fp64")}},
        "roofline": roof_main,
        "roofline_other": [roof_res, roof_fac],
        "pipes_measured": pipes,
        "cpu_baseline": cb and {k: cb[k] for k in ("value", "unit", "cores", "kind", "build", "sample")},
        "cpu_superlu_standin": slu,
        "e2e": {"value": n_all / e2e_s, "unit": "energies/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "inputs": "energies with NULL phiato/Bessel/Neumann: generated on the device"},
        "e2e_host_inputs": {"value": n_all / e2e_host_s, "unit": "energies/s", "h2d_bytes_per_step": int(h2d_host),
                            "d2h_bytes_per_step": int(d2h), "inputs": "phiato/Bessel/Neumann built on the host"},
        "gpu_launches": int(last["n_kernels"]),
        "clocks": clocks,
        "plain_fp64": {"value": n_e / (fp64_ms / 1000.0), "unit": "energies/s", "ms_per_step": fp64_ms,
                       "first_call_wall_s": fp64_wall, "gpu_launches": int(info64["n_kernels"])},
        "accuracy": {"convolved_rel_err_vs_fp64": err_conv, "convolved_rel_err_vs_fp64_host": err_conv_host,
                     "taull_max_rel_err_vs_fp64": err_taull, "refine_iters_max": last["refine_iters"],
                     "fp64_escalations": last["n_fallback"], "refine_steps": int(last["refine_steps"])},
        "phases_ms": {k: last[k] for k in ("ms_assemble", "ms_factor", "ms_solve", "ms_refine",
                                           "ms_refine_loop", "ms_escalate_factor")},
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_pt(args):
    """Configuration 4: fcc Pt, spin-orbit, FDM radius 4.0 A at step 0.2 A
    (19 atoms, about 51.6k complex rows), complex energies with a 0.5 eV
    broadening (E_comp, the regular solution), complex harmonics.  A step
    solves --pt-energies of the 300 energies -10..50 eV (spread over the grid
    points whose outer kinetic energy is positive) in one mixed-precision batch; the FP64 batch of the same energies is timed
    once for the comparison and the agreement."""
    import torch
    from fdmnes_gb300 import build as B, abi, cluster as CL, complex_path as CP
    from fdmnes_gb300.solver import FdmSolver
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    B.build()
    t0 = time.perf_counter()
    st = CL.build_structure(CL.pt_cluster(4.4), 0.2, 4.0, 50.0, nspin=2)
    # the outer-sphere solutions are those of a real kinetic energy: keep the
    # grid points above the outer potential of spin block 1 (0.5 eV margin)
    e_fermi = -5.0
    e_floor = (st.V0bd + st.spin_shift(1)) * CL.RYDB - e_fermi + 0.5
    grid300 = np.linspace(-10.0, 50.0, 300)
    grid_ok = grid300[grid300 > e_floor]
    energies = grid_ok[np.round(np.linspace(0, len(grid_ok) - 1, args.pt_energies)).astype(int)]
    ga = abi.GridArgs(CP.grid_dict(st, True))
    eimag_ry = 0.5 / 13.605693122994
    eas = [abi.EnergyArgs(CP.energy_dict(st, float(E), spinorbit=True, eimag_ry=eimag_ry,
                                                e_fermi_ev=e_fermi)) for E in energies]
    host_s = time.perf_counter() - t0
    sv = FdmSolver(ga.d)
    sv.set_tolerance(1e-8, 1e-6)

    def run(prec):
        sv.spectrum_begin(prec, len(eas))
        for ea in eas:
            sv.spectrum_add_args(ea)
        torch.cuda.synchronize()
        t = time.perf_counter()
        info = sv.spectrum_run()
        torch.cuda.synchronize()
        return time.perf_counter() - t, info, [sv.taull_c(k, 2) for k in range(len(eas))]

    run("mixed")  # warm-up: plan and graphs
    times, infos = [], []
    for _ in range(args.steps):
        dt, info, Tm = run("mixed")
        times.append(dt)
        infos.append(info)
    t64, info64, T64 = run("fp64")
    err = max(float(np.abs(a - b).max() / np.abs(b).max()) for a, b in zip(Tm, T64))
    wall = statistics.mean(times)
    last = infos[-1]
    nlig = [int(ea.d["nligne"]) for ea in eas]
    line = {
        "metric": METRIC, "value": len(eas) / wall, "unit": "energies/s", "n_gpus": 1, "steps": args.steps,
        "warmup": 1, "ms_per_step": 1000.0 * wall, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 factor + f64 refinement (df64 residual), real-equivalent complex",
        "data": "synthetic",
        "config": {"workload": "fcc Pt a=3.92 A, spin-orbit, 19 atoms within the FDM radius 4.0 A, step 0.2 A, "
                               "complex harmonics, complex energies (Eimag 0.5 eV), batched",
                   "energies": len(eas), "energies_ev": [float(e) for e in energies],
                   "full_configuration_energies": 300, "grid_points_above_outer_potential": int(len(grid_ok)), "nligne_complex": nlig,
                   "host_inputs_s": host_s},
        "phases_ms": {k: last[k] for k in ("ms_assemble", "ms_factor", "ms_solve", "ms_refine")},
        "factor_tflops": last["flops_factor"] / (last["ms_factor"] / 1000.0) / 1e12 if last["ms_factor"] > 0 else None,
        "fp64_escalations": last["n_fallback"],
        "plain_fp64": {"value": len(eas) / t64, "unit": "energies/s",
                       "phases_ms": {k: info64[k] for k in ("ms_assemble", "ms_factor", "ms_solve")}},
        "taull_max_rel_err_vs_fp64": err,
    }
    print(json.dumps(line), flush=True)
    sv.close()


def run_tio2(args):
    """Configuration 3: rutile TiO2, Ti K edge, two spin blocks, three
    absorbing-site clusters with FDM radii 4.0 / 4.5 / 5.0 A at step 0.2 A, in
    one batch over the sites (fdmgpu_batch_add_site) that the library splits
    into chunks fitting the device memory.  The full configuration has 200
    energies per site; a step here solves --tio2-energies of them (spread over
    the 200-point grid) for every site and spin.  One energy point is one
    energy of the spectrum over all three sites and both spins."""
    import torch
    from fdmnes_gb300 import build as B, cluster as CL, xanes
    from fdmnes_gb300.solver import FdmSolver
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    B.build()
    grid200 = np.linspace(-5.0, 35.0, 200)
    idx = np.round(np.linspace(0, 199, args.tio2_energies)).astype(int)
    energies = grid200[idx]
    radii = (4.0, 4.5, 5.0)
    sites = []
    t0 = time.perf_counter()
    for r in radii:
        st = CL.build_structure(CL.rutile_cluster(r - 0.4), 0.2, r, 35.0, nspin=2, spin_split_ev=1.5)
        sv = FdmSolver(st)
        sv.set_radial()
        sites.append((st, sv))
    host_build_s = time.perf_counter() - t0
    items = []  # (site solver, ei, ri)
    for st, sv in sites:
        for isp in (1, 2):
            for ei, ri in xanes.spectrum_inputs(st, energies, functions=False, ispin=isp):
                items.append((sv, ei, ri))
    main_sv = sites[0][1]
    main_sv.set_tolerance(1e-8, 1e-6)
    main_sv.set_tile_engine(args.tile_engine)
    main_sv.set_df64_engine(args.df64_engine)
    main_sv.set_escalation(args.escalation)

    def run():
        main_sv.spectrum_begin("mixed", len(items))
        for sv, ei, ri in items:
            if sv is main_sv:
                main_sv.spectrum_add(ei, ri)
            else:
                main_sv.spectrum_add_site(sv, ei, ri)
        return main_sv.spectrum_run()

    run()  # warm-up: plans and graphs of every chunk
    times, infos = [], []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        infos.append(run())
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    last = infos[-1]
    wall = statistics.mean(times)
    nlig = [ri.nligne for _, _, ri in items]
    n_e = len(energies)
    line = {
        "metric": METRIC, "value": n_e / wall, "unit": "energies/s", "n_gpus": 1, "steps": args.steps,
        "warmup": 1, "ms_per_step": 1000.0 * wall, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 factor + f64 refinement (df64 residual)", "data": "synthetic",
        "config": {"workload": "rutile TiO2 a=4.594 c=2.959 A u=0.305, Ti K edge, 2 spin blocks, 3 absorbing-site "
                               "clusters with FDM radii 4.0/4.5/5.0 A at step 0.2 A, batched over sites and spins",
                   "energies_per_site": n_e, "full_configuration_energies": 200, "problems": len(items),
                   "nligne": [min(nlig), max(nlig)], "chunks": "fdmgpu_set_memory_budget default (85% of HBM)",
                   "host_structure_build_s": host_build_s, "tile_engine": args.tile_engine,
                   "escalation": args.escalation},
        "phases_ms": {k: last[k] for k in ("ms_assemble", "ms_factor", "ms_solve", "ms_refine")},
        "flops_factor": last["flops_factor"],
        "factor_tflops": last["flops_factor"] / (last["ms_factor"] / 1000.0) / 1e12 if last["ms_factor"] > 0 else None,
        "fp64_escalations": last["n_fallback"], "wide_refactors": last["n_wide_refactor"],
        "projected_full_spectrum_s": wall * 200.0 / n_e,
    }
    print(json.dumps(line), flush=True)
    for _, sv in sites:
        sv.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--energies", type=int, default=401,
                    help="energies of the spectrum over -5..35 eV (401: step 0.1 eV; 41: step 1 eV)")
    ap.add_argument("--factor-mode", default="fp32", choices=["fp32", "wide_atom", "wide_all"],
                    help="accumulation of the FP32 factor (wide_atom: double-float sums at the atom-harmonic steps)")
    ap.add_argument("--tile-engine", default="simt_stream", choices=["simt", "simt_stream", "tcgen05", "tcgen05_factor"],
                    help="FP32 tile updates on the FP32 pipes or on the tensor cores (split TF32)")
    ap.add_argument("--df64-engine", default="tcgen05", choices=["simt", "tcgen05"],
                    help="double-float escalation trailing update: FP32 pipes or tensor-core integer slices")
    ap.add_argument("--escalation", default="df64_f32", choices=["df64", "df64_f32", "wide_df64", "fp64"],
                    help="re-solve of energies whose FP32 refinement stalls")
    ap.add_argument("--config", default="cu401", choices=["cu401", "tio2", "pt"],
                    help="cu401: the 401-energy Cu spectrum (the metric's configuration); tio2: the rutile "
                         "three-site, two-spin batch; pt: the Pt spin-orbit complex-energy batch")
    ap.add_argument("--tio2-energies", type=int, default=4, help="energies per site of the tio2 configuration")
    ap.add_argument("--pt-energies", type=int, default=2, help="energies of the pt configuration")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.config == "tio2":
        run_tio2(args)
    elif args.config == "pt":
        run_pt(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
