import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libnekgpu.so")


# Files whose code builds on the rest (the splitting step's gradient
# operators on the geometry, the pressure preconditioner and the element
# shards on the operator, gather-scatter and Krylov solves the other files
# test) run after them, so that a failure there is reported after, not
# instead of, the results of what it builds on.
_BUILT_ON_THE_REST = ("test_gpu_gradops.py", "test_gpu_h1mg.py", "test_gpu_plan4.py",
                      "test_gpu_plan4_step.py", "test_gpu_shard.py")


def pytest_collection_modifyitems(session, config, items):
    def rank(item):
        name = os.path.basename(str(item.fspath))
        if name.startswith("test_zz"):
            return 2
        return 1 if name in _BUILT_ON_THE_REST else 0
    items.sort(key=rank)  # stable: file order kept within each rank


@pytest.fixture(scope="session")
def oracle():
    from oracle import nekref
    nekref.build()
    return nekref


def rng_unit_vector(seed):
    r = np.random.default_rng(seed)
    v = r.standard_normal(3)
    return v / np.linalg.norm(v)


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if needed) and load libnekgpu.so; skip when no GPU is visible."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from nek5000_gb300 import build
    build.build()
    from nek5000_gb300 import NekGpu
    return NekGpu


def rank_spread(oracle, P, solve):
    """Largest relative change of the oracle's solution when its dot products
    are summed as P = 2, 3, 4, 7, 8 ranks would; returns (1-rank solution, spread)."""
    base = solve(P["ops"])
    worst = 0.0
    for nt in (2, 3, 4, 7, 8):
        ops = oracle.Ops(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"], nt)
        worst = max(worst, np.linalg.norm(solve(ops) - base) / np.linalg.norm(base))
    return base, worst
