"""CPU-side checks of the drop-in boundary: the C-ABI library builds, loads
and exports every function declared in include/wql.h.  No device calls."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    with open(os.path.join(ROOT, "include", "wql.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^\s*int\s+(wql_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def built_lib():
    import shutil
    if shutil.which("nvcc") is None:
        pytest.skip("nvcc not available")
    import wql_build
    return wql_build.build()


def test_header_declares_the_abi():
    names = declared_functions()
    assert "wql_step" in names and "wql_scenario_create_from_in" in names
    assert len(names) >= 15


def test_library_exports_every_declared_symbol(built_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (wql_\w+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_library_loads_and_binding_matches_header(built_lib):
    import ctypes
    import wql
    L = ctypes.CDLL(built_lib)
    for name in declared_functions():
        assert hasattr(L, name), name
    assert sorted(wql.EXPORTS) == declared_functions()


def test_error_path_without_device(built_lib):
    """wql_ctx_create reports an error code instead of aborting when no GPU
    is visible (this container has none)."""
    import wql
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is visible")
    except ImportError:
        pass
    with pytest.raises(wql.WqlError) as e:
        wql.Context(0)
    assert e.value.code == 3
