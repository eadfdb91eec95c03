"""Tangent-linear sensitivity of a J2 load history (lpm_tangent_begin):
the reaction curve of a BCC polycrystal pulled past yield and unloaded, and
a squared-error response of that curve against a seeded target, with
respect to the yield stress and the hardening modulus, against central
differences of whole forward runs."""
import math

import numpy as np
import pytest

from lpm_cases import gpu_bcs, lat, make_gpu, pkg, plate, tension_bcs

capi = pkg.capi
pytestmark = pytest.mark.gpu
E, NU, SIGY, XI, H = 110e3, 0.34, 900.0, 0.3, 1e3
STEPS = [1, 1, 1, 1, -1, -1]
OPTS = dict(solver=capi.SOLVER_FATIGUE_STATIC, tangent=capi.TANGENT_SYMMETRIC, precision=capi.PREC_FP64,
            max_iter=60, tol=1e-12, cg_tol=1e-13)


def polycrystal(ncell=5, a=0.2, ngrain=3, seed=11):
    xyz, gid = lat.bcc_polycrystal(ncell, a, ngrain, seed)
    cell = lat.UnitCell(lat.BCC3D, a * math.sqrt(3.0) / 4.0)
    keep = lat.prune_weak(xyz, cell, 6)
    xyz = xyz[keep]
    p1, p2, layer = lat.find_bonds(xyz, cell)
    Kn, Tv = lat.bond_constants(cell, layer, cell.elastic_constants(E, NU, layout="row"))
    return (3, xyz, p1, p2, layer, Kn, Tv, cell)


def run(args, sigy, h, dirs=None):
    """Reaction curve (sum of Pin_z over the top grip per step), and with
    dirs its tangents along each direction."""
    g = make_gpu(*args)
    xyz = args[1]
    g.set_law(capi.LAW_J2, [E, NU, sigy, XI, h, 0.0, 0.0])
    g.update()
    z = xyz[:, 2]
    bottom, top = np.where(z < 0.1)[0], np.where(z > z.max() - 0.1)[0]
    du = 0.004 * (z.max() - z.min())
    gb, gt = g.add_group(bottom), g.add_group(top)
    steps = [[("disp", gb, 0, 0.0), ("disp", gb, 1, 0.0), ("disp", gb, 2, 0.0), ("disp", gt, 2, sgn * du)]
             for sgn in STEPS]
    if dirs is not None:
        R, dR = pkg.adjoint.reaction_curve_sensitivity(g, steps, top, 2, dirs, tangent_tol=1e-13, **OPTS)
    else:
        R, dR = [], None
        for bcs in steps:
            r = g.load_step(bcs, **OPTS)
            assert r["status"] == 0, r
            R.append(g.download(capi.F_PIN)[top, 2].sum())
        R = np.array(R)
    plastic = np.abs(g.download(capi.B_DLP)).max() > 0
    g.close()
    return R, dR, plastic


def test_j2_reaction_curve_tangents_match_central_differences():
    args = polycrystal()
    d_sigy = [0, 0, 1, 0, 0, 0, 0]
    d_h = [0, 0, 0, 0, 1, 0, 0]
    R, dR, plastic = run(args, SIGY, H, [d_sigy, d_h])
    assert plastic
    # dR/dsigma_y and dR/dH per step against central differences
    for k, (hs, hh) in enumerate([(1e-5 * SIGY, 0.0), (0.0, 1e-5 * H)]):
        rp = run(args, SIGY + hs, H + hh)[0]
        rm = run(args, SIGY - hs, H - hh)[0]
        fd = (rp - rm) / (2 * (hs + hh))
        assert np.abs(fd).max() > 0
        assert np.abs(dR[:, k] - fd).max() <= 1e-5 * np.abs(fd).max(), (k, dR[:, k], fd)
    # a squared error of the curve against a seeded target
    target = R * (1.0 + 0.05 * np.random.default_rng(3).standard_normal(len(R)))
    grad = 2.0 * (R - target) @ dR
    for k, (hs, hh) in enumerate([(1e-5 * SIGY, 0.0), (0.0, 1e-5 * H)]):
        jp = ((run(args, SIGY + hs, H + hh)[0] - target) ** 2).sum()
        jm = ((run(args, SIGY - hs, H - hh)[0] - target) ** 2).sum()
        fdj = (jp - jm) / (2 * (hs + hh))
        assert abs(grad[k] - fdj) <= 1e-5 * abs(fdj), (k, grad[k], fdj)


def test_j2_tangents_on_a_hexagonal_plate():
    """The 2-D path: a hexagonal plate pulled past yield, per-step reaction
    tangents along the yield stress against central differences."""
    args = plate(9, 9, E=E, nu=NU)
    dim, xyz = args[0], args[1]
    L = xyz[:, 1].max() - xyz[:, 1].min()
    du = 0.006 * L
    groups, _, _ = tension_bcs(xyz, dim, du)

    def curve(sigy, dirs=None):
        g = make_gpu(*args)
        g.set_law(capi.LAW_J2, [E, NU, sigy, XI, H, 0.0, 0.0])
        g.update()
        bcs = gpu_bcs(g, groups, dim, du)
        if dirs is not None:
            g.tangent_begin(dirs, tol=1e-13)
        R, dR = [], []
        for _ in range(4):
            r = g.load_step(bcs, **OPTS)
            assert r["status"] == 0, r
            R.append(g.download(capi.F_PIN)[groups["top"], 1].sum())
            if dirs is not None:
                dR.append(g.tangent_get(0, capi.T_PIN)[groups["top"], 1].sum())
        plastic = np.abs(g.download(capi.B_DLP)).max() > 0
        g.close()
        return np.array(R), np.array(dR), plastic

    _, dR, plastic = curve(SIGY, [[0, 0, 1, 0, 0, 0, 0]])
    assert plastic
    h = 1e-5 * SIGY
    fd = (curve(SIGY + h)[0] - curve(SIGY - h)[0]) / (2 * h)
    assert np.abs(fd).max() > 0
    assert np.abs(dR - fd).max() <= 1e-5 * np.abs(fd).max(), (dR, fd)


def test_j2_tangent_along_youngs_modulus():
    """A direction in E changes the return map's shear modulus and, through
    the UnitCell map, every bond's constants (lpm_tangent_bond_constants):
    per-step reaction tangents against central differences of runs with the
    constants rebuilt at E +- h."""
    d0, xyz, p1, p2, layer, _, _, cell = plate(9, 9, E=E, nu=NU)
    L = xyz[:, 1].max() - xyz[:, 1].min()
    du = 0.006 * L
    groups, _, _ = tension_bcs(xyz, 2, du)

    def curve(e, tangent=False):
        Kn, Tv = lat.bond_constants(cell, layer, cell.elastic_constants(e, NU, plane_stress=True, layout="row"))
        g = make_gpu(2, xyz, p1, p2, layer, Kn, Tv, cell)
        g.set_law(capi.LAW_J2, [e, NU, SIGY, XI, H, 0.0, 0.0])
        g.update()
        bcs = gpu_bcs(g, groups, 2, du)
        if tangent:
            dm = cell.elastic_constants_grad(e, NU, plane_stress=True, layout="row")[0]
            dKn, dTv = lat.bond_constants(cell, layer, dm)
            g.tangent_begin([[1.0, 0, 0, 0, 0, 0, 0]], tol=1e-13, dbond=[(dKn, dTv)])
        R, dR = [], []
        for _ in range(4):
            r = g.load_step(bcs, **OPTS)
            assert r["status"] == 0, r
            R.append(g.download(capi.F_PIN)[groups["top"], 1].sum())
            if tangent:
                dR.append(g.tangent_get(0, capi.T_PIN)[groups["top"], 1].sum())
        plastic = np.abs(g.download(capi.B_DLP)).max() > 0
        g.close()
        return np.array(R), np.array(dR), plastic

    _, dR, plastic = curve(E, True)
    assert plastic
    h = 1e-5 * E
    fd = (curve(E + h)[0] - curve(E - h)[0]) / (2 * h)
    assert np.abs(dR - fd).max() <= 1e-5 * np.abs(fd).max(), (dR, fd)


def test_tangent_refuses_other_laws():
    args = polycrystal(4, ngrain=2)
    g = make_gpu(*args)
    g.update()
    with pytest.raises(capi.LpmError):
        g.tangent_begin([[0.0]])
    g.close()
