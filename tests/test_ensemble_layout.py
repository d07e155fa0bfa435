"""Host logic of the batched ensemble's per-replica cell grids (pairs_gb300.ensemble.replica_grid).

Cells of >= r_list / reach per axis; pair-cluster lists need every stencil cell visited
once, so 2 reach + 1 cells per axis; reach 0 takes per replica the largest cells that
give such a grid.  Boxes as in the ensemble workload (trimmed fcc, rho 0.6..0.9).
"""
import pytest

from pairs_gb300.ensemble import replica_grid

R_LIST = 2.8


def side(n, rho):
    return (n / rho) ** (1.0 / 3.0)


def test_fixed_layouts():
    L = [side(2000, 0.6)] * 3                     # 14.94: 5 cells of >= 2.8, 10 of >= 1.4
    assert replica_grid(L, R_LIST, 1) == ([5, 5, 5], 1, 1)
    assert replica_grid(L, R_LIST, 2) == ([10, 10, 10], 2, 2)
    assert replica_grid(L, R_LIST, 3) == ([10, 5, 5], 2, 1)


def test_reach0_takes_the_largest_cells_that_fit():
    assert replica_grid([side(2000, 0.6)] * 3, R_LIST, 0) == ([5, 5, 5], 1, 1)
    # 864 atoms at rho 0.7: 10.72 -> 3 cells of >= r_list, enough for reach 1
    assert replica_grid([side(864, 0.7)] * 3, R_LIST, 0) == ([3, 3, 3], 1, 1)
    # 500 atoms at rho 0.9: 8.22 -> 2 cells of >= r_list; x halves give 5 but y, z need 3:
    # cells of >= r_list / 2 on every axis
    assert replica_grid([side(500, 0.9)] * 3, R_LIST, 0) == ([5, 5, 5], 2, 2)
    # a box long in x only: halved x cells with full y, z cells
    assert replica_grid([7.5, 9.0, 9.0], R_LIST, 0) == ([5, 3, 3], 2, 1)


def test_pair_lists_refuse_a_grid_that_revisits_cells():
    small = [side(500, 0.9)] * 3
    with pytest.raises(ValueError, match="pair-cluster"):
        replica_grid(small, R_LIST, 1, pair_lists=True)
    # per-particle lists take the grid as it is
    assert replica_grid(small, R_LIST, 1) == ([2, 2, 2], 1, 1)
    # too small even at reach 2 (4 half cells): refused with reach 0 too
    with pytest.raises(ValueError, match="pair-cluster"):
        replica_grid([6.5] * 3, R_LIST, 0, pair_lists=True)
