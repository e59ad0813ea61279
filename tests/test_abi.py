"""The C-ABI library: it builds for sm_103a, loads, and exports every declared entry point.

No compute call is made here (these run on machines without a GPU).
"""
import ctypes
import importlib.util
import os
import re
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build_module():
    spec = importlib.util.spec_from_file_location("_mh_build_lib", os.path.join(REPO, "marinehydro.jl_gb300",
                                                                                "build_lib.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.fixture(scope="module")
def libpath():
    return _build_module().build()


def declared_functions():
    names = []
    inc = os.path.join(REPO, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"\b(mh_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "mh_assemble_matrices" in names and "mh_hydrodynamic_coefficients" in names
    assert len(names) >= 15


def test_library_exports_every_declared_symbol(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (mh_[a-z0-9_]+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_library_loads_and_reports_version(libpath, mh):
    L = mh.load_library()
    with open(os.path.join(REPO, "include", "marinehydro_gb300.h")) as f:
        declared = int(re.search(r"#define MH_ABI_VERSION (\d+)", f.read()).group(1))
    assert L.mh_abi_version() == declared
    for n in declared_functions():
        assert hasattr(L, n)


def test_python_binding_lists_every_declared_symbol(mh):
    from importlib import import_module  # noqa: F401

    lib_mod = __import__("marinehydro_gb300._lib", fromlist=["EXPORTS"])
    assert sorted(lib_mod.EXPORTS) == declared_functions()


def test_null_and_bad_arguments_are_rejected_without_a_gpu(libpath, mh):
    """Argument checks happen before any device work: a NULL context or output is an error code."""
    L = mh.load_library()
    assert L.mh_create(0, None) == 1  # MH_ERR_ARG
    assert L.mh_destroy(None) == 0
    assert L.mh_last_error(None) == b"null context"
    assert L.mh_assemble_matrices(None, None, ctypes.c_double(1.0), 35, 1, 1, None, None, None, 0) == 1
    assert L.mh_linsolve(None, 3, 1, None, None, None, 0, 0) == 1
    assert L.mh_mesh_panels(None) == -1
    assert L.mh_mesh_set_lid(None, 1) == 1


def test_kernel_sources_target_sm103a():
    b = _build_module()
    assert b.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    for src in b.sources():
        assert src.endswith(".cu")
