"""Shared test set-up: import paths, the `gpu` marker, mesh fixtures."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "fea-visualizer_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

REFERENCE_ASSETS = "/root/reference/assets/fem_meshes"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def has_reference_assets():
    return os.path.isdir(REFERENCE_ASSETS)


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def fea():
    """The built CUDA library on a visible GPU; GPU tests fail loudly without it."""
    import fea_gb300
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    fea_gb300.load()
    return fea_gb300


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def f32(x):
    return float(np.float32(x))


def oracle_step(oracle_mod, S, eq, dt, u, v, n, **kw):
    """FP64 oracle steps with the float32-rounded parameters the ABI carries
    (the reference's parameter structs hold floats, EquationParameters.hpp)."""
    for key in ("kappa", "Du", "Dv", "F", "k", "adv_sign"):
        if key in kw:
            kw[key] = f32(kw[key])
    p = oracle_mod.params(eq, f32(dt), tol=1e-14, **kw)
    a = None
    if eq == oracle_mod.WAVE and kw.get("wave_scheme", 0) == 1:
        a = S.newmark_init(p, u)
    return S.step(p, u, v, a, nsteps=n)
