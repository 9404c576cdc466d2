"""The FP32 tile updates on the tensor cores (split-TF32 tcgen05.mma).

The mixed path factors in FP32 and refines in FP64; with
FDMGPU_ENGINE_TCGEN05 its trailing update and its refinement-solve updates
run as three TF32 products of hi/lo operand pairs.  Parity bars are those of
the FP32-pipe engine: the refined solution equals the oracle's to 1e-8
(double-float residual) or 1e-10 (FP64 residual).  The products must be as
accurate as FP32 products: the refinement needs about as many steps as with
the FP32-pipe updates (a TF32-only product, ~1e-3 relative, would stall the
refinement of these matrices, whose equilibrated condition numbers reach
1e6-4e7).
"""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def solver_mod():
    from fdmnes_gb300 import build
    build.build()
    from fdmnes_gb300 import solver
    return solver


def test_golden_mixed_tcgen05_matches_oracle(solver_mod, golden):
    from fdmnes_gb300 import abi
    grid, energies = golden
    sv = solver_mod.FdmSolver(grid)
    sv.set_tile_engine("tcgen05")
    for mode, tol in (("df64", 1e-8), ("fp64", 1e-10)):
        sv.set_residual(mode)
        for e in energies:
            X, info = sv.mat_solve_args(abi.EnergyArgs(e), "mixed")
            assert info["converged"]
            assert rel(X, e["smr"]) < tol, (mode, rel(X, e["smr"]))
    sv.close()


def test_small_cluster_tcgen05_batch(solver_mod, oracle_lib):
    from fdmnes_gb300 import abi, cluster as CL
    st = CL.small_cu_structure()
    ga = abi.GridArgs(st)
    energies = (-5.0, 3.0, 12.0, 27.0, 35.0)
    items, refs = [], []
    for E in energies:
        ei = CL.energy_inputs(st, E)
        ri = CL.newind(st, ei.nlmsa, ei.nlmso)
        ea = abi.EnergyArgs(st, ei, ri)
        Xo, _ = oracle_lib.mat_solve(ga, ea)
        refs.append(oracle_lib.taull(ga, ea, Xo))
        items.append((ei, ri))
    sv = solver_mod.FdmSolver(st)
    sv.set_tile_engine("tcgen05")
    T, info = sv.spectrum(items, "mixed")
    for k, To in enumerate(refs):
        assert rel(T[k], To) < 1e-8, (energies[k], rel(T[k], To))
    sv.close()


def test_full_cu_tcgen05_refines_like_fp32_pipes(solver_mod):
    """Nine energies of the 13-atom Cu spectrum: the tensor-core engine gives
    the FP64 cross-section to <= 1e-6 (convolved) and needs about as many
    refinement steps per energy as the FP32-pipe engine."""
    from fdmnes_gb300 import cluster as CL, xanes
    st = CL.cu_structure()
    energies = np.linspace(-5.0, 35.0, 9)
    items = xanes.spectrum_inputs(st, energies)
    sv = solver_mod.FdmSolver(st)
    T64, _ = sv.spectrum(items, "fp64")
    sv.set_tolerance(1e-8, 1e-6)
    its = {}
    for engine in ("simt", "tcgen05"):
        sv.set_tile_engine(engine)
        Tm, info = sv.spectrum(items, "mixed")
        err = xanes.convolved_relative_error(energies, Tm, T64)
        assert err < 1e-6, (engine, err)
        its[engine] = [sv.stats(k)[0] for k in range(len(items))]
    # per energy a few more steps at most, and no more steps in total than
    # one and a half times those of the FP32 pipes
    for k in range(len(items)):
        assert its["tcgen05"][k] <= 2 * its["simt"][k] + 10, (energies[k], its)
    assert sum(its["tcgen05"]) <= 1.5 * sum(its["simt"]) + 5, its
    sv.close()


def test_tcgen05_with_wide_atom_steps(solver_mod):
    """Steps marked for wide accumulation stay on the FP32 pipes while the
    others run on the tensor cores, in the same launch sequence."""
    from fdmnes_gb300 import cluster as CL, xanes
    st = CL.cu_structure()
    energies = np.array([8.0, 26.0, 34.0])
    items = xanes.spectrum_inputs(st, energies)
    sv = solver_mod.FdmSolver(st)
    T64, _ = sv.spectrum(items, "fp64")
    sv.set_tolerance(1e-8, 1e-6)
    sv.set_factor_mode("wide_atom")
    sv.set_tile_engine("tcgen05")
    Tm, info = sv.spectrum(items, "mixed")
    assert xanes.convolved_relative_error(energies, Tm, T64) < 1e-6
    assert max(rel(a, b) for a, b in zip(Tm, T64)) < 1e-5
    sv.close()


def test_chunked_batch_equals_one_batch(solver_mod):
    """A batch above the memory budget runs in consecutive chunks of energies
    (each planned and launched on its own) and gives the same Taull, bit for
    bit, as one batch: the kernels treat every energy independently."""
    from fdmnes_gb300 import cluster as CL, xanes
    st = CL.cu_structure()
    energies = np.linspace(-5.0, 35.0, 7)
    items = xanes.spectrum_inputs(st, energies)
    sv = solver_mod.FdmSolver(st)
    sv.set_tolerance(1e-8, 1e-6)
    for prec in ("fp64", "mixed"):
        sv.set_memory_budget(0.0)
        T1, i1 = sv.spectrum(items, prec)
        s1 = [sv.stats(k)[:3] for k in range(len(items))]
        sv.set_memory_budget(4e8)   # one to three Cu energies per chunk
        T2, i2 = sv.spectrum(items, prec)
        assert all(np.array_equal(a, b) for a, b in zip(T1, T2)), prec
        assert [sv.stats(k)[:3] for k in range(len(items))] == s1
        with pytest.raises(solver_mod.FdmError):
            sv.solution(0, items[0][0].nlmso, items[0][1].nligne)
    sv.set_memory_budget(0.0)
    sv.close()


def test_row_solves_match_column_solves(solver_mod, golden):
    """Refinement solves row by row (each row's strip summed in registers,
    one launch per tile row) against the step-by-step solves: the refined
    solution meets the oracle bars (1e-8 with the df64 residual), and on full
    Cu energies the cross-section bar and about the same refinement steps."""
    from fdmnes_gb300 import abi, cluster as CL, xanes
    grid, energies = golden
    sv = solver_mod.FdmSolver(grid)
    sv.set_solve_order("rows")
    for e in energies:
        X, info = sv.mat_solve_args(abi.EnergyArgs(e), "mixed")
        assert info["converged"]
        assert rel(X, e["smr"]) < 1e-8
    sv.close()
    st = CL.cu_structure()
    E = np.array([2.0, 14.0, 26.0, 34.0])
    items = xanes.spectrum_inputs(st, E)
    sv = solver_mod.FdmSolver(st)
    T64, _ = sv.spectrum(items, "fp64")
    sv.set_tolerance(1e-8, 1e-6)
    its = {}
    for order in ("columns", "rows"):
        sv.set_solve_order(order)
        Tm, _ = sv.spectrum(items, "mixed")
        assert xanes.convolved_relative_error(E, Tm, T64) < 1e-6, order
        its[order] = [sv.stats(k)[0] for k in range(len(items))]
    assert sum(its["rows"]) <= sum(its["columns"]) + 8, its
    sv.close()


def test_escalation_on_tensor_cores_integer_slices(solver_mod):
    """The double-float escalation factor with its trailing update on the
    tensor cores (rows and columns cut into exact 7-bit integer slices, one
    exact FP32 accumulator per slice order): on full Cu energies whose FP32
    refinement stalls (benchmark tolerances), the escalated energies reach
    the acceptance level as with the FP32-pipe double-float update, and the
    spectrum meets the FP64 bars (Taull 1e-5, convolved 1e-6)."""
    from fdmnes_gb300 import cluster as CL, xanes
    st = CL.cu_structure()
    E = np.array([2.0, 22.0, 26.0, 30.0, 34.0])
    items = xanes.spectrum_inputs(st, E)
    sv = solver_mod.FdmSolver(st)
    T64, _ = sv.spectrum(items, "fp64")
    sv.set_tolerance(1e-8, 1e-6)
    res = {}
    for eng in ("simt", "tcgen05"):
        sv.set_df64_engine(eng)
        Tm, info = sv.spectrum(items, "mixed")
        assert info["n_fallback"] >= 1, eng
        assert not info["not_converged"], (eng, info["not_converged"])
        assert max(rel(a, b) for a, b in zip(Tm, T64)) < 1e-5, eng
        assert xanes.convolved_relative_error(E, Tm, T64) < 1e-6, eng
        res[eng] = [sv.stats(k) for k in range(len(items))]
    assert [r[2] for r in res["simt"]] == [r[2] for r in res["tcgen05"]]
    sv.set_df64_engine("simt")
    sv.close()


def test_streamed_strips_match_one_tile_kernels(solver_mod, golden):
    """The bulk-copy-staged strip updates (one shared operand tile per CTA,
    the streamed tiles in a two-stage ring) sum every product in the same k
    order as the one-tile kernels: the refined solutions meet the oracle bars,
    and on full Cu energies (with escalated ones, whose double-float factor
    runs as strips with its panel as products with the inverted diagonal
    triangles, and with the wide-accumulation factor mode) the FP32 energies
    agree with the one-tile engine's to 1e-9, the escalations are the same
    and every energy meets the FP64 bars."""
    from fdmnes_gb300 import abi, cluster as CL, xanes
    grid, energies = golden
    sv = solver_mod.FdmSolver(grid)
    sv.set_tile_engine("simt_stream")
    for mode, tol in (("df64", 1e-8), ("fp64", 1e-10)):
        sv.set_residual(mode)
        for e in energies:
            X, info = sv.mat_solve_args(abi.EnergyArgs(e), "mixed")
            assert info["converged"]
            assert rel(X, e["smr"]) < tol, (mode, rel(X, e["smr"]))
    sv.close()
    st = CL.cu_structure()
    E = np.array([2.0, 14.0, 26.0, 30.0, 34.0])
    items = xanes.spectrum_inputs(st, E)
    sv = solver_mod.FdmSolver(st)
    T64, _ = sv.spectrum(items, "fp64")
    sv.set_tolerance(1e-8, 1e-6)
    for factor in ("fp32", "wide_atom"):
        sv.set_factor_mode(factor)
        out = {}
        for engine in ("simt", "simt_stream"):
            sv.set_tile_engine(engine)
            T, info = sv.spectrum(items, "mixed")
            esc = [sv.stats(k)[2] for k in range(len(E))]
            out[engine] = (T, esc)
            assert xanes.convolved_relative_error(E, T, T64) < 1e-6, (factor, engine)
            assert max(rel(a, b) for a, b in zip(T, T64)) < 1e-5, (factor, engine)
        assert out["simt"][1] == out["simt_stream"][1], factor
        if factor == "fp32":
            assert any(out["simt"][1])
        # FP32 energies: the same sums; escalated ones: the double-float panel
        # differs (products with the inverted triangles), each meets the bars
        for k in range(len(E)):
            if not out["simt"][1][k]:
                assert rel(out["simt"][0][k], out["simt_stream"][0][k]) < 1e-9, (factor, E[k])
    sv.set_factor_mode("fp32")
    sv.set_tile_engine("simt")
    sv.close()
