"""CPU tests of the C ABI boundary: the library builds, loads and exports every
function that include/fea_gpu.h declares; defaults mirror the reference's
EquationParameters.hpp; creating a solver without a GPU fails loudly."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "fea_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(fea_\w+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    import sys
    sys.path.insert(0, ROOT)
    import __graft_entry__ as ge
    ge.build_library()
    from fea_gb300 import binding
    return binding.load()


def test_header_declares_the_solver_interface():
    names = declared_functions()
    for n in ("fea_create", "fea_destroy", "fea_advance_time", "fea_clear_values",
              "fea_has_numerical_instability", "fea_set_values", "fea_get_values", "fea_get_matrix"):
        assert n in names
    assert len(names) >= 30


def test_every_declared_symbol_is_exported(lib):
    for n in declared_functions():
        assert hasattr(lib, n), n


def test_binding_signatures_cover_header():
    from fea_gb300 import binding
    names = set(declared_functions()) - {"fea_last_error", "fea_version"}
    assert names == set(binding.SIGNATURES)


def test_param_defaults_mirror_reference(lib):
    from fea_gb300 import binding
    p = binding.default_params()
    # EquationParameters.hpp:8-49
    assert (p.heat_time_step, p.heat_conductivity) == (np.float32(0.01), np.float32(0.05))
    assert (p.advdiff_time_step, p.advdiff_c) == (np.float32(0.001), np.float32(0.25))
    assert list(p.advdiff_velocity) == [1.0, 0.0, 0.0]
    assert (p.wave_time_step, p.wave_c) == (np.float32(0.05), np.float32(0.05))
    assert (p.rd_time_step, p.rd_Du, p.rd_Dv) == (np.float32(0.001), np.float32(0.08), np.float32(0.04))
    assert (p.rd_feed_rate, p.rd_kill_rate) == (np.float32(0.035), np.float32(0.06))
    assert p.equation == binding.WAVE  # FEMContext.hpp:31
    assert p.reaction_mode == 0 and p.wave_scheme == 0 and p.advection_scheme == 0


def test_struct_layouts_match_header(lib):
    """Sizes of the ctypes mirrors equal the C structs (compiled probe)."""
    import subprocess
    import tempfile
    from fea_gb300 import binding
    src = ('#include <stdio.h>\n#include "fea_gpu.h"\nint main(){printf("%zu %zu %zu %zu\\n",'
           'sizeof(fea_params),sizeof(fea_info),sizeof(fea_status),sizeof(fea_instance_desc));return 0;}\n')
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "p.c")
        exe = os.path.join(d, "p")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        sizes = [int(x) for x in subprocess.run([exe], capture_output=True, text=True).stdout.split()]
    assert sizes == [C.sizeof(binding.Params), C.sizeof(binding.Info), C.sizeof(binding.Status),
                     C.sizeof(binding.InstanceDesc)]


def test_argument_errors_without_gpu(lib):
    from fea_gb300 import binding
    h = C.c_void_p()
    xyz = np.zeros((3, 3), np.float32)
    tri = np.array([[0, 1, 2]], np.uint32)
    rc = lib.fea_create(xyz.ctypes.data, 3, tri.ctypes.data, 0, None, 0, 0, None, C.byref(h))
    assert rc == -4  # empty mesh: FEA_ERR_BAD_MESH
    rc = lib.fea_create(xyz.ctypes.data, 3, tri.ctypes.data, 1, None, 7, 0, None, C.byref(h))
    assert rc == -1  # bad boundary condition
    assert lib.fea_params_default(None) == -1
    assert lib.fea_advance_time(None, 1) == -1
    # batched: no instances, an empty instance mesh, a null handle
    assert lib.fea_batch_create(None, 0, 0, 0.0, 0, C.byref(h)) == -1
    d = (binding.InstanceDesc * 1)()
    d[0].vertices, d[0].num_vertices = xyz.ctypes.data, 3
    d[0].triangles, d[0].num_triangles = tri.ctypes.data, 0
    d[0].time_step = 0.5
    assert lib.fea_batch_create(d, 1, 0, 0.0, 0, C.byref(h)) == -4
    d[0].num_triangles = 1
    d[0].time_step = 0.0
    assert lib.fea_batch_create(d, 1, 0, 0.0, 0, C.byref(h)) == -1
    assert lib.fea_batch_advance_time(None, 1) == -1
    assert lib.fea_batch_destroy(None) == 0


def test_no_cpu_fallback_without_gpu(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    from fea_gb300 import binding, meshgen
    with pytest.raises(binding.FeaError) as ei:
        binding.CUDASolver(*meshgen.icosphere(1))
    assert ei.value.code == -3
    xyz, tri = meshgen.icosphere(1)
    with pytest.raises(binding.FeaError) as ei:
        binding.BatchSolver([dict(vertices=xyz, triangles=tri, time_step=0.5)])
    assert ei.value.code == -3
