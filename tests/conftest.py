"""Shared test set-up: import paths, the `gpu` marker, mesh fixtures."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "fea-visualizer_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

# The reference checkout's mesh folder (assets/fem_meshes), when one is
# present: only the tests that re-read the OBJ files need it.  The meshes
# themselves travel as tests/golden/reference_meshes.npz.
REFERENCE_ASSETS = os.environ.get("FEA_REFERENCE_ASSETS", "")
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def has_reference_assets():
    return bool(REFERENCE_ASSETS) and os.path.isdir(REFERENCE_ASSETS)


def reference_meshes():
    """The reference's icosphere.obj and tube.obj as committed fixtures:
    name -> (xyz float32 [V, 3], tri uint32 [T, 3])."""
    from make_golden import load_fixture
    return load_fixture()


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


def device_field(s, which):
    """Unknown-indexed state field of a handle in its precision (float64 for
    FP64 handles), read through the device API."""
    import torch
    dt = torch.float64 if s.precision == 1 else torch.float32
    t = [torch.zeros(s.info.num_unknowns, dtype=dt, device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    s.get_fields_device(t[0].data_ptr(), t[1].data_ptr())
    return t[which].cpu().numpy().astype(np.float64)
