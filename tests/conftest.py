"""Shared test setup: markers, in-tree builds, golden fixtures."""
from __future__ import annotations

import glob
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")


@pytest.fixture(scope="session")
def built():
    """Builds the native libraries and the oracle once per session."""
    from vnec_gb300 import build as B
    from oracle import oracle as O

    B.build()
    O.build()
    return True


def golden_cases() -> list[str]:
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as z:
        return {k: z[k] for k in z.files}


def golden_manifest() -> dict:
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


class Csr:
    """Minimal CSR holder with the attributes the bindings read."""

    def __init__(self, n_rows, n_cols, row_ptr, col, val):
        self.n_rows, self.n_cols = int(n_rows), int(n_cols)
        self.row_ptr = np.asarray(row_ptr, dtype=np.int64)
        self.col = np.asarray(col, dtype=np.int32)
        self.val = np.asarray(val)

    @property
    def nnz(self) -> int:
        return int(self.row_ptr[-1])


def golden_csr(g: dict) -> Csr:
    return Csr(g["n_rows"], g["n_cols"], g["row_ptr"], g["col"], g["val"])


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False
