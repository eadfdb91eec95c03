"""Configuration-4 form: BCC Voronoi polycrystal with the J2 law.

CPU: the generator (seeded, inside the box, no two particles closer than the
overlap threshold, grains from their own Voronoi cells).  GPU: tension past
yield and unloading through lpm_load_step, against the oracle step by step
(positions, J2 state variables, plastic bond stretch)."""
import math

import numpy as np
import pytest

from lpm_cases import lat, make_gpu, make_oracle, oracle, pkg

capi = pkg.capi
E, NU, SIGY, H = 110e3, 0.34, 900.0, 1e3


def polycrystal(ncell=6, a=0.2, ngrain=4, seed=11):
    xyz, gid = lat.bcc_polycrystal(ncell, a, ngrain, seed)
    cell = lat.UnitCell(lat.BCC3D, a * math.sqrt(3.0) / 4.0)
    keep = lat.prune_weak(xyz, cell, 6)
    xyz, gid = xyz[keep], gid[keep]
    p1, p2, layer = lat.find_bonds(xyz, cell)
    Kn, Tv = lat.bond_constants(cell, layer, cell.elastic_constants(E, NU, layout="row"))
    return xyz, gid, (3, xyz, p1, p2, layer, Kn, Tv, cell)


def test_polycrystal_generator():
    from scipy.spatial import cKDTree

    a, ncell = 0.2, 8
    xyz, gid = lat.bcc_polycrystal(ncell, a, 6, 5)
    xyz2, gid2 = lat.bcc_polycrystal(ncell, a, 6, 5)
    assert np.array_equal(xyz, xyz2) and np.array_equal(gid, gid2)
    assert xyz.min() >= 0.0 and xyz.max() <= ncell * a
    d = cKDTree(xyz).query(xyz, k=2)[0][:, 1]
    assert d.min() >= 0.5 * a * math.sqrt(3.0) / 2.0
    assert len(np.unique(gid)) == 6
    # about two sites per cubic cell
    assert abs(len(xyz) / (2 * ncell ** 3) - 1.0) < 0.15
    # every particle is closest to its own grain's seed
    rng = np.random.default_rng(5)
    seeds = rng.random((6, 3)) * ncell * a
    assert np.array_equal(cKDTree(seeds).query(xyz)[1], gid)
    R = lat.random_rotations(200, np.random.default_rng(1))
    assert np.abs(np.einsum("nij,nkj->nik", R, R) - np.eye(3)).max() < 1e-12
    assert np.abs(np.linalg.det(R) - 1.0).max() < 1e-12


@pytest.mark.gpu
def test_polycrystal_j2_tension_and_unloading_match_oracle():
    xyz, gid, args = polycrystal()
    n = len(xyz)
    o = make_oracle(*args)
    g = make_gpu(*args)
    params = [E, NU, SIGY, 0.0, H, 0.0, 0.0]
    o.set_law(2, params)
    g.set_law(capi.LAW_J2, params)
    o.update()
    g.update()
    z = xyz[:, 2]
    # grips: the slabs within half a cell of the two faces
    bottom, top = np.where(z < 0.1)[0], np.where(z > z.max() - 0.1)[0]
    L = z.max() - z.min()
    du = 0.004 * L
    gb, gt = g.add_group(bottom), g.add_group(top)
    apply = np.zeros((n, 3), np.int32)
    apply[bottom, :] = 1
    apply[top, 2] = 1
    plastic = False
    for step, sgn in enumerate([1, 1, 1, 1, -1, -1]):
        dd = np.zeros((n, 3))
        dd[top, 2] = sgn * du
        bcs = [("disp", gb, 0, 0.0), ("disp", gb, 1, 0.0), ("disp", gb, 2, 0.0), ("disp", gt, 2, sgn * du)]
        ro = o.load_step(apply, dd, sym=1, bc_elim=1, max_iter=60, tol=1e-9, cg_tol=1e-12)
        rg = g.load_step(bcs, solver=capi.SOLVER_FATIGUE_STATIC, tangent=capi.TANGENT_SYMMETRIC,
                         precision=capi.PREC_FP64, max_iter=60, tol=1e-9, cg_tol=1e-12)
        assert ro >= 0 and rg["status"] == 0, (step, ro, rg)
        u_o = o.get(oracle.XYZ) - xyz
        u_g = g.download(capi.F_XYZ) - xyz
        s_o, s_g = o.state(), g.state()
        lp_o, lp_g = o.get_bond(oracle.DLP), g.download(capi.B_DLP)
        print("[parity] polycrystal step %d: displacement %.3e, state %.3e, plastic stretch %.3e" % (
            step, np.abs(u_g - u_o).max() / np.abs(u_o).max(),
            np.abs(s_g - s_o).max() / max(np.abs(s_o).max(), 1e-30),
            np.abs(lp_g - lp_o).max() / max(np.abs(lp_o).max(), 1e-30)))
        assert np.abs(u_g - u_o).max() <= 1e-8 * np.abs(u_o).max(), step
        assert np.abs(s_g - s_o).max() <= 1e-8 * max(np.abs(s_o).max(), 1e-30), step
        assert np.abs(lp_g - lp_o).max() <= 1e-8 * max(np.abs(lp_o).max(), 1e-30), step
        plastic = plastic or np.abs(lp_o).max() > 0
    assert plastic
    g.close()
