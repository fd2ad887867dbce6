"""Test configuration: the `gpu` marker and shared fixtures.

`-m "not gpu"` runs on any machine (oracle against the golden fixtures and the
reference pin, host logic, ABI exports); `-m gpu` runs the CUDA library
against the oracle on a GB300.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libxdem")


@pytest.fixture(scope="session")
def oracle():
    from oracle.pyoracle import Oracle, build_oracle
    build_oracle()
    return Oracle()


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    from metakonga_gb300 import _lib
    _lib.lib()          # raises if libxdem was not built
    return torch


def force_error(f, f_ref, mass, g=9.81):
    """max_i |F_i - F_ref_i| / max(|F_ref_i|, m_i g): per-particle error
    normalised by the particle's own force scale (never below its weight)."""
    f = np.asarray(f, np.float64).reshape(-1, 3)
    f_ref = np.asarray(f_ref, np.float64).reshape(-1, 3)
    num = np.linalg.norm(f - f_ref, axis=1)
    den = np.maximum(np.linalg.norm(f_ref, axis=1), np.asarray(mass) * g)
    return float((num / den).max()) if num.size else 0.0
