"""The bench's byte accounting on CPU: the split-PML cell counts behind its
"with the shell's stored parts" roofline figure, against a brute-force count
over small grids, and the per-cell stored parts of the FP32 shell's rule
(a component is split where one of its two curl axes is a PML axis)."""
import itertools
import os
import sys
from types import SimpleNamespace

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _spec(n, npml, periodic=(False, False, False)):
    return SimpleNamespace(n=n, periodic=periodic, pml={"npml": npml},
                           cells=lambda: n[0] * n[1] * n[2])


def _axes_inside(spec):
    """Per cell, how many axes' PML it lies in (0..3), by enumeration."""
    counts = np.zeros(spec.n[::-1], dtype=np.int32)  # [z][y][x]
    for a in range(3):
        n = spec.n[a]
        lo, hi = (0, 0) if spec.periodic[a] or n == 1 else spec.pml["npml"][a]
        idx = np.arange(n)
        inside = (idx < lo) | (idx >= n - hi)
        shape = [1, 1, 1]
        shape[2 - a] = n
        counts += inside.reshape(shape).astype(np.int32)
    return counts


@pytest.mark.parametrize("n,npml,periodic", [
    ((40, 36, 30), ((4, 4), (5, 3), (6, 2)), (False, False, False)),
    ((64, 64, 1), ((8, 8), (8, 8), (0, 0)), (False, False, False)),
    ((32, 24, 48), ((3, 3), (3, 3), (10, 10)), (True, True, False)),
    ((20, 20, 20), ((0, 0), (0, 0), (0, 0)), (False, False, False)),
])
def test_pml_cells_by_axes_matches_enumeration(n, npml, periodic):
    spec = _spec(n, npml, periodic)
    c = _axes_inside(spec)
    one, more = bench.pml_cells_by_axes(spec)
    assert one == int(np.sum(c == 1))
    assert more == int(np.sum(c >= 2))


def test_no_pml_means_no_shell_cells():
    spec = SimpleNamespace(n=(16, 16, 16), periodic=(False,) * 3, pml=None, cells=lambda: 16 ** 3)
    assert bench.pml_cells_by_axes(spec) == (0, 0)


def test_fp32_shell_stored_parts_per_cell():
    """E and H each: Ex curls along (y, z), Ey along (z, x), Ez along (x, y).
    One stored part per split component: 4 in one axis's PML, 6 in more."""
    curl_axes = {0: {1, 2}, 1: {2, 0}, 2: {0, 1}}
    for k in (1, 2, 3):
        for axes in itertools.combinations(range(3), k):
            split = sum(1 for c in range(3) if curl_axes[c] & set(axes))
            assert 2 * split == (4 if k == 1 else 6)


def test_algorithmic_bytes_per_cell():
    assert bench.alg_bytes("E", 4) == 17 and bench.alg_bytes("H", 4) == 20
    assert bench.alg_bytes("step", 4) == 25 and bench.alg_bytes("step", 8) == 49
