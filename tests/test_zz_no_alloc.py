"""fdmgpu_taull_noalloc: Taull from a device-resident smr with the working
matrix in the library's static device scratch (no device allocation).

It is compared with fdmgpu_batch_taull on the same solutions: both contract
the same smr with the same elimination order, so they agree to 1e-12
relative (max |diff| / max |ref|).  Two calls are issued back to back on one
stream before a single synchronisation, the second overwriting the scratch
the first used.  The file is named so that it is collected last and also runs
after every other GPU test.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

TOL = 1e-12
SCRATCH_BYTES = 2 * 1024 * 1024
MAX_NLMSO = 512


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fdmnes_gb300 import build
    build.build()
    return torch


def _bind(lib):
    f = lib.fdmgpu_taull_noalloc
    f.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    lib.fdmgpu_last_error.restype = C.c_char_p
    return f


def _batch_results(torch, st, energies):
    """FP64 batch solve: per energy (smr on the device, Taull of the batch path, ianew_abs, nlm_abs)."""
    from fdmnes_gb300 import cluster as CL
    from fdmnes_gb300.solver import FdmSolver
    sv = FdmSolver(st)
    items = []
    for E in energies:
        ei = CL.energy_inputs(st, E)
        items.append((ei, CL.newind(st, ei.nlmsa, ei.nlmso)))
    T, _ = sv.spectrum(items, "fp64")
    out = []
    for k, (ei, ri) in enumerate(items):
        smr = sv.solution(k, ei.nlmso, ri.nligne)
        d_smr = torch.from_numpy(np.asfortranarray(smr).ravel(order="F").copy()).to("cuda")
        out.append((d_smr, ei.nlmso, ri.nligne, int(ri.ianew[0]), int(ei.nlmsa[0]), T[k]))
    return sv, out


def _two_calls_in_a_row(torch, f, cases):
    stream = torch.cuda.current_stream()
    taulls, status = [], torch.full((len(cases),), -1, dtype=torch.int32, device="cuda")
    for i, (d_smr, nlmso, nligne, ianew, m, _) in enumerate(cases):
        t = torch.empty(2 * m * m, dtype=torch.float64, device="cuda")
        st = f(d_smr.data_ptr(), nlmso, nligne, ianew, m, t.data_ptr(), status[i:].data_ptr(), stream.cuda_stream)
        assert st == 0
        taulls.append(t)
    torch.cuda.synchronize()
    assert status.tolist() == [0] * len(cases)
    for t, (_, _, _, _, m, ref) in zip(taulls, cases):
        got = t.cpu().numpy().view(np.complex128).reshape((m, m), order="F")
        assert rel(got, ref) < TOL, rel(got, ref)


def test_noalloc_taull_small_cluster(torch_cuda):
    from fdmnes_gb300 import cluster as CL
    sv, cases = _batch_results(torch_cuda, CL.small_cu_structure(), [3.0, 27.0])
    f = _bind(sv.lib)
    _two_calls_in_a_row(torch_cuda, f, cases)
    _two_calls_in_a_row(torch_cuda, f, cases[::-1])
    sv.close()


def test_noalloc_taull_full_cluster_largest_harmonics(torch_cuda):
    """Full 13-atom cluster at 35 eV: nlmso = 256, nlm_abs = 36, a 1.14 MiB working matrix."""
    from fdmnes_gb300 import cluster as CL
    sv, cases = _batch_results(torch_cuda, CL.cu_structure(), [35.0, -5.0])
    assert cases[0][1] * (cases[0][1] + cases[0][4]) * 16 > SCRATCH_BYTES // 2
    _two_calls_in_a_row(torch_cuda, _bind(sv.lib), cases)
    sv.close()


def test_noalloc_rejects_sizes_beyond_the_scratch(torch_cuda):
    from fdmnes_gb300 import cluster as CL
    from fdmnes_gb300.solver import FdmSolver
    sv = FdmSolver(CL.small_cu_structure())
    f = _bind(sv.lib)
    smr = torch_cuda.zeros(600 * 700, dtype=torch_cuda.float64, device="cuda")
    out = torch_cuda.zeros(2 * 64 * 64, dtype=torch_cuda.float64, device="cuda")
    assert f(smr.data_ptr(), MAX_NLMSO + 1, 700, 0, 4, out.data_ptr(), None, None) == 1
    assert b"FDMGPU_TAULL_NOALLOC_MAX_NLMSO" in sv.lib.fdmgpu_last_error()
    n, m = 360, 40  # 360 * 400 * 16 bytes > 2 MiB
    assert n * (n + m) * 16 > SCRATCH_BYTES
    assert f(smr.data_ptr(), n, 700, 0, m, out.data_ptr(), None, None) == 1
    assert b"static scratch" in sv.lib.fdmgpu_last_error()
    assert f(smr.data_ptr(), 8, 16, 12, 8, out.data_ptr(), None, None) == 1  # absorber rows past nligne
    assert f(None, 8, 16, 0, 8, out.data_ptr(), None, None) == 1
    sv.close()


def test_noalloc_reports_a_singular_normalisation(torch_cuda):
    """nlmso = 2 with the outer block S = [[0, 1], [-1, 0]]: norm = I + iS is
    singular, and the kernel's status word reads FDMGPU_ERR_ZERO_PIVOT (a
    division by zero in the back substitution, no fault).  A regular call
    afterwards reports FDMGPU_OK again."""
    from fdmnes_gb300 import cluster as CL
    from fdmnes_gb300.solver import FdmSolver
    sv = FdmSolver(CL.small_cu_structure())
    f = _bind(sv.lib)
    # smr (nlmso = 2, nligne = 4) column-major: columns 1-2 the absorber rows,
    # columns 3-4 the outer rows, S(i, j) = smr(i, outer row j)
    smr = np.array([[1.0, 0.5, 0.0, 1.0],
                    [0.25, 1.0, -1.0, 0.0]])
    d_smr = torch_cuda.from_numpy(smr.ravel(order="F").copy()).to("cuda")
    out = torch_cuda.zeros(2 * 2 * 2, dtype=torch_cuda.float64, device="cuda")
    status = torch_cuda.full((1,), -1, dtype=torch_cuda.int32, device="cuda")
    stream = torch_cuda.cuda.current_stream().cuda_stream
    assert f(d_smr.data_ptr(), 2, 4, 0, 2, out.data_ptr(), status.data_ptr(), stream) == 0
    torch_cuda.cuda.synchronize()
    assert int(status.item()) == 4  # FDMGPU_ERR_ZERO_PIVOT
    smr[:, 2:] = [[0.0, 0.5], [-0.25, 0.0]]  # I + iS regular
    d_smr = torch_cuda.from_numpy(smr.ravel(order="F").copy()).to("cuda")
    assert f(d_smr.data_ptr(), 2, 4, 0, 2, out.data_ptr(), status.data_ptr(), stream) == 0
    torch_cuda.cuda.synchronize()
    assert int(status.item()) == 0
    sv.close()
