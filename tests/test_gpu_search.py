"""GPU neighbour search (lpm_find_bonds, lpm_find_neighbors) against the
host k-d tree search, which applies the reference's createBonds arithmetic:
bit-exact bond lists, layers and order on regular, perturbed, polycrystal
and notched lattices."""
import math

import numpy as np
import pytest

from lpm_cases import lat, pkg

capi = pkg.capi
pytestmark = pytest.mark.gpu


def cases():
    out = []
    out.append(("hex", lat.hex_plate(31, 31, 0.5), lat.UnitCell(lat.HEXAGON2D, 0.25)))
    sc = lat.sc_cuboid(12, 12, 12, 0.2)
    out.append(("sc", sc, lat.UnitCell(lat.SIMPLECUBIC3D, 0.1)))
    rng = np.random.default_rng(2)
    out.append(("sc-perturbed", sc + rng.normal(0, 0.01, sc.shape), lat.UnitCell(lat.SIMPLECUBIC3D, 0.1)))
    xyz, _ = lat.bcc_polycrystal(8, 0.2, 5, 3)
    out.append(("bcc-poly", xyz, lat.UnitCell(lat.BCC3D, 0.2 * math.sqrt(3.0) / 4.0)))
    xyz, _, _, _, cell, _ = lat.ct_specimen(10.0, 0.4, 0.3)
    out.append(("ct", xyz, cell))
    return out


@pytest.mark.parametrize("name,xyz,cell", cases(), ids=[c[0] for c in cases()])
def test_gpu_bond_search_is_bit_exact(name, xyz, cell):
    p1, p2, layer = capi.find_bonds(xyz, cell)
    q1, q2, ql = lat.find_bonds(xyz, cell)
    assert np.array_equal(p1, q1) and np.array_equal(p2, q2) and np.array_equal(layer, ql)


def test_gpu_nonlocal_search_is_bit_exact():
    xyz = lat.hex_plate(25, 25, 0.5)
    ptr, idx = capi.find_neighbors(xyz, 1.5 * 0.64)
    qptr, qidx = lat.nonlocal_neighbors(xyz, 1.5 * 0.64)
    assert np.array_equal(ptr, qptr) and np.array_equal(idx, qidx)
    # per-particle radii
    r = np.where(xyz[:, 0] < 6.0, 0.9, 1.3)
    ptr, idx = capi.find_neighbors(xyz, r)
    for i in range(0, len(xyz), 37):
        d = np.sqrt(((xyz - xyz[i]) ** 2).sum(1))
        assert np.array_equal(idx[ptr[i]:ptr[i + 1]], np.where(d < r[i])[0])
