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


def _grid(dims, cell_len):
    cells = _capi.PgCells()
    for d in range(3):
        cells.dims[d] = dims[d]
        cells.cell_len[d] = cell_len[d]
    cells.ncells = dims[0] * dims[1] * dims[2]
    return cells


@pytest.mark.parametrize("dims,cell_len", [((0, 4, 4), (1.0, 1.0, 1.0)), ((4, -1, -4), (1.0, 1.0, 1.0)),
                                           ((4, 4, 4), (1.0, 0.0, 1.0)), ((4, 4, 4), (1.0, float("nan"), 1.0))])
def test_bad_cell_grid_is_rejected_before_any_device_work(lib, dims, cell_len):
    """A grid with an empty axis or a non-positive cell length would give negative cell
    indices in the binning kernel: every entry point that bins or scans cells returns
    PG_ERR_ARGUMENT first.  The device pointers below are never dereferenced (no CUDA
    call happens on this path, which is why it runs without a GPU)."""
    fake = C.c_void_p(0x1000)
    box = _capi.PgBox()
    p = _capi.PgParticles()
    p.n = p.capacity = 10
    p.pos = fake
    cells = _grid(dims, cell_len)
    ws = _capi.PgWorkspace(fake, 1 << 20)
    assert lib.pg_bin_particles(C.byref(box), C.byref(p), C.byref(cells), ws, fake, None) == _capi.PG_ERR_ARGUMENT
    assert lib.pg_bin_particles_noalloc(C.byref(box), C.byref(p), C.byref(cells), fake, None) == \
        _capi.PG_ERR_ARGUMENT
    lst = _capi.PgNeighborList()
    assert lib.pg_build_neighbor_lists(C.byref(box), C.byref(p), C.byref(cells), C.byref(lst), 7.84, fake,
                                       None) == _capi.PG_ERR_ARGUMENT


def test_grid_product_must_match_ncells(lib):
    fake = C.c_void_p(0x1000)
    box = _capi.PgBox()
    p = _capi.PgParticles()
    p.n = p.capacity = 10
    p.pos = fake
    cells = _grid((4, 4, 4), (1.0, 1.0, 1.0))
    cells.ncells = 63
    ws = _capi.PgWorkspace(fake, 1 << 20)
    assert lib.pg_bin_particles(C.byref(box), C.byref(p), C.byref(cells), ws, fake, None) == _capi.PG_ERR_ARGUMENT
