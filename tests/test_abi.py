"""The C-ABI library builds for sm_103a, loads without a GPU, and exports every declared symbol."""
import ctypes
import os
import re
import subprocess

import pytest

from tests.conftest import ROOT

HEADER = os.path.join(ROOT, "include", "difftactile_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:int|size_t|void)\s+(dt_\w+)\s*\(", src, flags=re.M)
    assert names, "no declarations parsed"
    return names


@pytest.fixture(scope="module")
def lib_path():
    from difftactile_gb300 import build
    return build.build()


def test_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (dt_\w+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"declared but not exported: {missing}"


def test_struct_layout_matches_ctypes(lib_path):
    from difftactile_gb300 import _native
    lib = _native.load(lib_path)  # loads without a GPU; only size queries are called
    assert lib.dt_abi_version() == 8
    assert lib.dt_sizeof_world() == ctypes.sizeof(_native.DtWorld)
    assert lib.dt_sizeof_env() == ctypes.sizeof(_native.DtEnv)
    assert lib.dt_sizeof_sensor() == ctypes.sizeof(_native.DtSensor)
    assert lib.dt_sizeof_material() == ctypes.sizeof(_native.DtMaterial)


def test_ctypes_signatures_cover_header():
    from difftactile_gb300 import _native
    missing = [n for n in declared_functions() if n not in _native.SIGNATURES]
    assert not missing, f"no ctypes signature for {missing}"


def test_build_targets_sm103a_only():
    from difftactile_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_last_error_without_a_failure(lib_path):
    """dt_last_error reports (and clears) the CUDA error behind a DT_ERR_LAUNCH; with none recorded it
    returns 0 and names cudaSuccess.  Host-only: no device is touched."""
    from difftactile_gb300 import _native
    _native.load(lib_path)
    code, msg = _native.last_error()
    assert code == 0 and msg.startswith("cudaSuccess")
