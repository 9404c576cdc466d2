import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def golden():
    """Golden problem: grid arrays, per-energy arrays and oracle outputs."""
    d = np.load(os.path.join(GOLDEN, "golden_problem.npz"))
    grid = {k[2:]: d[k] for k in d.files if k.startswith("g_")}
    energies = []
    for k in range(len(d["energies"])):
        pre = f"e{k}_"
        e = {n[len(pre):]: d[n] for n in d.files if n.startswith(pre)}
        energies.append(e)
    for dd in [grid] + energies:
        for n, v in list(dd.items()):
            if v.ndim == 0:
                dd[n] = v.item()
    return grid, energies


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.fixture(scope="session")
def golden_complex():
    """Complex spin-orbit golden problem: grid and energy arguments (dicts of
    arrays and scalars) and the oracle's solution and Taull."""
    d = np.load(os.path.join(GOLDEN, "golden_complex.npz"))

    def part(pre):
        out = {k[len(pre):]: d[k] for k in d.files if k.startswith(pre)}
        return {k: (v.item() if v.ndim == 0 else v) for k, v in out.items()}

    return part("g_"), part("e_"), d["smr"] + 1j * d["smi"], d["taull"]
