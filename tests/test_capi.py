"""The C-ABI library loads without a GPU and exports what include/*.h declares."""
import ctypes as C
import glob
import os
import re

import pytest

from pairs_gb300 import _capi, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:int|int64_t|void|double)\s+\**(pg_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _capi.load()


def test_header_declares_entry_points():
    names = declared_functions()
    assert "pg_lj_force" in names and "pg_build_neighbor_lists" in names
    assert len(names) >= 10


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header(lib):
    # every entry point the header declares has a ctypes signature
    assert set(declared_functions()) <= set(_capi.SIGNATURES)


def test_struct_layout_matches(lib):
    _capi.check_layout(lib)
    assert lib.pg_version() >= 1


def test_workspace_size_positive(lib):
    assert lib.pg_workspace_bytes(1 << 20, 40 ** 3) > (1 << 20) * 32


def test_argument_errors_without_gpu(lib):
    # null descriptors are rejected before any CUDA call
    assert lib.pg_build_neighbor_lists(None, None, None, None, 7.84, None, None) == _capi.PG_ERR_ARGUMENT
    assert lib.pg_lj_force(None, None, None, None, None, 0, 0, None, _capi.PgWorkspace(), None) == _capi.PG_ERR_ARGUMENT
    assert lib.pg_permute(-1, None, None, None, 4, None) == _capi.PG_ERR_ARGUMENT
