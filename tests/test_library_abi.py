"""The C-ABI library loads and exports every entry point declared in include/jfgpu.h (CPU only: no compute)."""
import ctypes
import os
import re

import pytest

from jellyfysh_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    with open(os.path.join(ROOT, "include", "jfgpu.h")) as handle:
        text = handle.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(jfgpu_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def library():
    if not os.path.exists(_lib.LIBRARY_PATH):
        import jellyfysh_gb300.build as build
        build.build()
    return _lib.load_library()


def test_header_declares_the_engine_and_potentials():
    names = declared_functions()
    for name in ("jfgpu_engine_create", "jfgpu_chains_run", "jfgpu_lennard_jones_displacement",
                 "jfgpu_merged_image_coulomb_derivative"):
        assert name in names


def test_every_declared_symbol_is_exported(library):
    for name in declared_functions():
        assert hasattr(library, name), name
        assert name in _lib.SIGNATURES, name


def test_host_only_entry_points(library):
    assert library.jfgpu_version() >= 1
    assert library.jfgpu_error_string(2) == b"invalid argument"
    # argument validation happens before any device work
    handle = ctypes.c_void_p()
    assert library.jfgpu_engine_create(None, 0, None, ctypes.byref(handle)) == 2
    assert library.jfgpu_engine_layout(None, None) == 2
    assert library.jfgpu_chains_set_block_warps(None, 4) == 2
    assert library.jfgpu_chains_set_refine_limit(None, 4) == 2
