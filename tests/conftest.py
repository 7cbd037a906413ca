"""Shared test helpers.

Markers: `gpu` = needs a CUDA device (the parity tests against the oracle);
everything else runs on the CPU (oracle vs golden fixtures, host logic, ABI
surface of libpmlg.so).
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

P998 = 998244353


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (parity tests of the CUDA path)")


def golden(name: str):
    return json.loads((GOLDEN / f"{name}.json").read_text())


def pm_from_seed(r: int, c: int, length: int, p: int, seed: int) -> np.ndarray:
    """Fixture input: seeded SplitMix64 matrix, or all (p-1) when seed == -1."""
    import oracle
    if seed == -1:
        return np.full((r, c, length), p - 1, dtype=np.uint64)
    return oracle.rand_poly_mat(r, c, length, p, seed)


def vec_from_seed(n: int, p: int, seed: int) -> np.ndarray:
    import oracle
    if seed == -1:
        return np.full(n, p - 1, dtype=np.uint64)
    return oracle.rand_vec(n, p, seed)


def as_u64(nested) -> np.ndarray:
    return np.array(nested, dtype=object).astype(np.uint64)


def cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def ctx():
    """One pml_gb300 context for the GPU tests."""
    if not cuda_available():
        pytest.skip("no CUDA device")
    import pml_gb300
    c = pml_gb300.Context(0)
    yield c
    c.close()


def to_dev(a: np.ndarray):
    """uint64 numpy array -> int64 CUDA tensor holding the same bits."""
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint64).view(np.int64)).cuda()


def to_host(t) -> np.ndarray:
    return t.cpu().numpy().view(np.uint64)
