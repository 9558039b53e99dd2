"""The C ABI library: it builds for sm_103a, loads, and exports every
function include/rpm_gpu.h declares.  No compute call is made without a GPU."""
import ctypes
import os
import re
import shutil

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "rpm_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rpm_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from rpmplv2_gb300 import build
    if not os.path.exists(build.LIB):
        if shutil.which(build.nvcc()) is None and not os.path.exists(build.nvcc()):
            pytest.skip("nvcc not available to build the library")
        build.build()
    return ctypes.CDLL(build.LIB)


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_lists_every_symbol():
    from rpmplv2_gb300.engine import ABI_SYMBOLS
    assert sorted(ABI_SYMBOLS) == declared_functions()


def test_host_only_entry_points(lib):
    lib.rpm_box_aabb.argtypes = [ctypes.c_void_p] * 4
    import numpy as np
    from rpmplv2_gb300 import scenes
    out = np.zeros(6, np.float32)
    for quat in ([0, 0, 0, 1], [0.1, 0.2, 0.3, 0.9]):
        dim, pos, q = (np.asarray(v, np.float32) for v in ([0.2, 0.3, 0.4], [1, 2, 3], quat))
        assert lib.rpm_box_aabb(dim.ctypes.data, pos.ctypes.data, q.ctypes.data, out.ctypes.data) == 0
        assert np.array_equal(out, scenes.box_aabb(dim, pos, q))
    lib.rpm_last_error_string.restype = ctypes.c_char_p
    assert lib.rpm_box_aabb(None, None, None, None) == -1
    assert b"NULL" in lib.rpm_last_error_string()


def test_no_cpu_fallback_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from rpmplv2_gb300.engine import Engine
    with pytest.raises(Exception):
        Engine(0)


def test_adapter_library_defines_the_space(lib):
    """librpm_adapter.so (base::RealVectorSpaceGPU over the StateSpace shim)
    loads and defines the four overriding virtuals and the batched forms."""
    from rpmplv2_gb300 import build
    path = build.build_adapter()
    ctypes.CDLL(path)
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm not available")
    import subprocess
    syms = subprocess.run([nm, "-D", "-C", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    for name in ("RealVectorSpaceGPU::isValid(std::shared_ptr<base::State>)",
                 "RealVectorSpaceGPU::isValid(std::shared_ptr<base::State>, std::shared_ptr<base::State>)",
                 "RealVectorSpaceGPU::computeDistance(", "RealVectorSpaceGPU::computeDistanceUnderestimation(",
                 "RealVectorSpaceGPU::isValidBatch(", "RealVectorSpaceGPU::computeDistanceBatch(",
                 "RealVectorSpaceGPU::isValidEdgesBatch(", "RealVectorSpaceGPU::updateObstacles(",
                 "vtable for base::RealVectorSpaceGPU"):
        assert name in syms, name
    undef = subprocess.run([nm, "-D", "--undefined-only", path], capture_output=True, text=True, check=True).stdout
    assert "rpm_distance_nearest" in undef and "rpm_check_configs" in undef
