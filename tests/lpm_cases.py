"""Shared set-up for the tests: golden fixtures, lattices, oracle/GPU pairs."""
import os

import numpy as np

import __graft_entry__ as ge

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

pkg = ge.load_package()
lat = pkg.lattice
oracle = ge.load_oracle()


def golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def golden_meta(d):
    out = {}
    for item in d["_meta"][1:]:
        k, v = str(item).split("=", 1)
        out[k] = v
    return out


def cell_for(d):
    """UnitCell of a golden fixture (hex for 2-D cases, SC otherwise)."""
    meta = golden_meta(d)
    a = float(meta.get("a", 0.5))
    kind = str(d["_meta"][0])
    if kind.endswith("hex"):
        return lat.UnitCell(lat.HEXAGON2D, a / 2)
    return lat.UnitCell(lat.SIMPLECUBIC3D, a / 2)


def inputs_from_golden(d):
    """(dim, xyz0, p1, p2, layer, Kn, Tv, cell) exactly as the reference held them."""
    cell = cell_for(d)
    xyz0 = d["xyz0"].reshape(-1, 3)
    return (cell.dim, xyz0, d["bond_p1"].astype(np.int32), d["bond_p2"].astype(np.int32),
            d["bond_layer"].astype(np.int32), d["Kn"], d["Tv"], cell)


def make_oracle(dim, xyz, p1, p2, layer, Kn, Tv, cell):
    return oracle.OracleSystem(dim, xyz, p1, p2, layer, Kn, Tv, cell.particle_volume, cell.nneighbors)


def make_gpu(dim, xyz, p1, p2, layer, Kn, Tv, cell):
    return pkg.capi.Lattice(dim, xyz, p1, p2, layer, Kn, Tv, cell.particle_volume, cell.nneighbors)


def mask3(d, n, dim):
    m = np.zeros((n, 3), np.int32)
    m[:, :dim] = d["mask"].reshape(n, dim)
    return m


def dense_from_csc(outer, inner, values, n):
    import scipy.sparse as sp
    return sp.csc_matrix((values, inner, outer), shape=(n, n)).toarray()


def dense_from_bsr(cptr, cidx, blocks, n, dim):
    K = np.zeros((n * dim, n * dim))
    for i in range(n):
        for q in range(cptr[i], cptr[i + 1]):
            j = cidx[q]
            K[dim * i:dim * i + dim, dim * j:dim * j + dim] = blocks[q]
    return K


def plate(ncol, nrow, a=0.5, E=69e3, nu=0.3, layout="row"):
    """Configuration-1 form: hexagonal plate with its bond list and constants."""
    cell = lat.UnitCell(lat.HEXAGON2D, a / 2)
    xyz = lat.hex_plate(ncol, nrow, a)
    p1, p2, layer = lat.find_bonds(xyz, cell)
    Kn, Tv = lat.bond_constants(cell, layer, cell.elastic_constants(E, nu, plane_stress=True, layout=layout))
    return 2, xyz, p1, p2, layer, Kn, Tv, cell


def cube(n, a=0.2, E=200e3, nu=0.3, layout="row"):
    """Configuration-2 form: simple cubic block of n^3 particles."""
    cell = lat.UnitCell(lat.SIMPLECUBIC3D, a / 2)
    xyz = lat.sc_cuboid(n, n, n, a)
    p1, p2, layer = lat.find_bonds(xyz, cell)
    Kn, Tv = lat.bond_constants(cell, layer, cell.elastic_constants(E, nu, layout=layout))
    return 3, xyz, p1, p2, layer, Kn, Tv, cell


def tension_bcs(xyz, dim, du):
    """Groups and BC arrays of the two load cases.

    2-D: bottom row fixed in y, bottom-left particle fixed in x, top row
    pulled in y.  3-D: bottom face clamped, top face pulled in z.
    Returns (groups dict, bc list builder for capi, apply/d arrays for the oracle)."""
    ax = 1 if dim == 2 else 2
    c = xyz[:, ax]
    bottom = np.where(c < c.min() + 1e-9)[0]
    top = np.where(c > c.max() - 1e-9)[0]
    n = len(xyz)
    apply = np.zeros((n, 3), np.int32)
    d = np.zeros((n, 3))
    if dim == 2:
        apply[bottom, 1] = 1
        apply[bottom[0], 0] = 1
    else:
        apply[bottom, :] = 1
    apply[top, ax] = 1
    d[top, ax] = du
    return dict(bottom=bottom, top=top, corner=bottom[:1]), apply, d


def gpu_bcs(g, groups, dim, du):
    gb = g.add_group(groups["bottom"])
    gt = g.add_group(groups["top"])
    if dim == 2:
        gc = g.add_group(groups["corner"])
        return [("disp", gb, 1, 0.0), ("disp", gc, 0, 0.0), ("disp", gt, 1, du)]
    return [("disp", gb, 0, 0.0), ("disp", gb, 1, 0.0), ("disp", gb, 2, 0.0), ("disp", gt, 2, du)]


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    s = np.abs(b).max()
    return float(np.abs(a - b).max() / (s if s > 0 else 1.0))
