"""Adjoint of the load step (lpm_backward_step, lpm_apply_jacobian, checkpoints).

- the matrix-free Jacobian product against central differences of the
  internal force computed by the oracle on the CPU, beside the reference's
  analytical stiffness derivative (both variants) on the same state;
- gradients of a reaction force with respect to the bond constants and to
  (E, nu) against central differences of whole forward runs, within the
  1e-5 relative bound the adjoint is held to;
- a response summed over a load history, replayed from checkpoints.
"""
import numpy as np
import pytest

from lpm_cases import cube, dense_from_bsr, gpu_bcs, lat, make_gpu, make_oracle, oracle, pkg, plate, tension_bcs

capi = pkg.capi
STEP = dict(solver=capi.SOLVER_FATIGUE_STATIC, tangent=capi.TANGENT_SYMMETRIC, precision=capi.PREC_FP64,
            max_iter=60, tol=1e-12, cg_tol=1e-13)
E0, NU0 = 69e3, 0.3


def strained_state(dim):
    if dim == 3:
        d, xyz, p1, p2, layer, Kn, Tv, cell = cube(4)
    else:
        d, xyz, p1, p2, layer, Kn, Tv, cell = plate(7, 7)
    rng = np.random.default_rng(7)
    x = xyz.copy()
    x[:, :dim] += rng.standard_normal((len(x), dim)) * 2e-3
    return (d, xyz, p1, p2, layer, Kn, Tv, cell), x


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
def test_jacobian_product_matches_central_differences(dim):
    args, x = strained_state(dim)
    g = make_gpu(*args)
    g.upload(capi.F_XYZ, x)
    g.update()
    o = make_oracle(*args)
    n = len(x)
    rng = np.random.default_rng(11)
    v = rng.standard_normal(n * dim)
    u = rng.standard_normal(n * dim)
    Hv = g.apply_jacobian(v)
    Hu = g.apply_jacobian(u)

    def pin(xx):
        o.set(oracle.XYZ, xx)
        o.update()
        return o.get(oracle.PIN)[:, :dim].ravel().copy()

    h = 1e-6
    V = np.zeros((n, 3))
    V[:, :dim] = v.reshape(n, dim)
    fd = (pin(x + h * V) - pin(x - h * V)) / (2 * h)
    assert np.abs(Hv - fd).max() <= 1e-6 * np.abs(fd).max()
    # the internal force is the gradient of the lattice energy: H is symmetric
    assert abs(u @ Hv - v @ Hu) <= 1e-12 * np.abs(u).sum() * np.abs(Hv).max()
    # the reference's stiffness derivative (derivative.h, the same file as
    # benchmark/Stiffness_derivative/derivative.h) is not this Jacobian: it
    # leaves out the change of the bond directions, and as written its
    # K_ii[1][0] entries are zero.  Its products differ from the central
    # differences by orders of magnitude more than the exact Jacobian's.
    cptr, cidx = g.pattern()
    err = {"exact Jacobian": np.abs(Hv - fd).max() / np.abs(fd).max()}
    for name, tangent in (("symmetric tangent", capi.TANGENT_SYMMETRIC), ("tangent as written", capi.TANGENT_AS_WRITTEN)):
        g.assemble(tangent, capi.BC_NONE)
        K = dense_from_bsr(cptr, cidx, g.K_bsr(), n, dim)
        err[name] = np.abs(K @ v - fd).max() / np.abs(fd).max()
    print("[jacobian] %d-D, random strain of 2e-3: max|product - central difference| / max|central difference|: %s" % (
        dim, ", ".join("%s %.2e" % kv for kv in err.items())))
    assert min(err["symmetric tangent"], err["tangent as written"]) >= 100 * err["exact Jacobian"]
    g.close()


def hex_case(ncol=13):
    d, xyz, p1, p2, layer, Kn, Tv, cell = plate(ncol, ncol, E=E0, nu=NU0)
    groups, _, _ = tension_bcs(xyz, d, 0.0)
    return d, xyz, p1, p2, layer, cell, groups


def forward(case, Kn, Tv, du=0.002, nsteps=3):
    """Displacement-controlled tension; J = reaction on the top row along y."""
    d, xyz, p1, p2, layer, cell, groups = case
    g = capi.Lattice(d, xyz, p1, p2, layer, Kn, Tv, cell.particle_volume, cell.nneighbors)
    bcs = gpu_bcs(g, groups, d, du)
    g.update()
    for _ in range(nsteps):
        r = g.load_step(bcs, **STEP)
        assert r["status"] == 0, r
    c = np.zeros((g.n, d))
    c[groups["top"], 1] = 1.0
    J = float((g.download(capi.F_PIN)[:, :d] * c).sum())
    return g, J, c.ravel()


def material(case, E, nu):
    d, xyz, p1, p2, layer, cell, groups = case
    return lat.bond_constants(cell, layer, cell.elastic_constants(E, nu, plane_stress=True, layout="row"))


@pytest.mark.gpu
def test_adjoint_gradient_matches_central_differences():
    case = hex_case()
    layer = case[4]
    Kn, Tv = material(case, E0, NU0)
    g, J, c = forward(case, Kn, Tv)
    gk_s, gt_s, iters, relres = g.backward_step(dJdpin=c, cg_tol=1e-13)
    assert relres <= 1e-13 and iters > 0
    perm = g.bond_perm
    gk = np.zeros_like(gk_s)
    gt = np.zeros_like(gt_s)
    gk[perm] = gk_s
    gt[perm] = gt_s
    g.close()
    # a random direction in the space of per-bond constants
    rng = np.random.default_rng(3)
    dKn = rng.uniform(-1, 1, Kn.shape) * Kn
    dTv = rng.uniform(-1, 1, Tv.shape) * np.abs(Tv)
    h = 1e-5
    gp = forward(case, Kn + h * dKn, Tv + h * dTv)
    gm = forward(case, Kn - h * dKn, Tv - h * dTv)
    fd = (gp[1] - gm[1]) / (2 * h)
    gp[0].close()
    gm[0].close()
    ad = float(gk @ dKn + gt @ dTv)
    assert abs(ad - fd) <= 1e-5 * abs(fd), (ad, fd)
    # (E, nu) through the constants' derivatives
    cell = case[5]
    dm = cell.elastic_constants_grad(E0, NU0, plane_stress=True, layout="row")  # rows d/dE, d/dnu of (Kn0, Kn1, Tv)
    dKn_dm = np.where(layer[None, :] == 0, dm[:, :1], dm[:, 1:2])
    grad_E = float(gk @ dKn_dm[0] + gt.sum() * dm[0, 2])
    grad_nu = float(gk @ dKn_dm[1] + gt.sum() * dm[1, 2])
    for k, (E, nu, hh) in enumerate([(E0, NU0, 1e-3 * E0), (E0, NU0, 1e-5)]):
        if k == 0:
            jp = forward(case, *material(case, E + hh, nu))
            jm = forward(case, *material(case, E - hh, nu))
        else:
            jp = forward(case, *material(case, E, nu + hh))
            jm = forward(case, *material(case, E, nu - hh))
        fdm = (jp[1] - jm[1]) / (2 * hh)
        jp[0].close()
        jm[0].close()
        ad = grad_E if k == 0 else grad_nu
        assert abs(ad - fdm) <= 1e-5 * abs(fdm), (k, ad, fdm)
    # displacement control with zero external force: J scales with E
    assert abs(grad_E * E0 - J) <= 1e-8 * abs(J)


@pytest.mark.gpu
def test_adjoint_over_load_history_with_checkpoints():
    case = hex_case(11)
    d, xyz, p1, p2, layer, cell, groups = case
    Kn, Tv = material(case, E0, NU0)
    target = np.array([2.0, 3.5, 6.0, 7.5, 9.0])

    def run(Kn, Tv, every, want_grad):
        g = capi.Lattice(d, xyz, p1, p2, layer, Kn, Tv, cell.particle_volume, cell.nneighbors)
        bcs = gpu_bcs(g, groups, d, 0.002)
        g.update()
        c = np.zeros((g.n, d))
        c[groups["top"], 1] = 1.0
        hist = pkg.adjoint.LoadHistory(g, [bcs] * len(target), every=every, **STEP)
        F = hist.forward(lambda n: (None, c.ravel()))
        J = float(((F - target) ** 2).sum())
        out = None
        if want_grad:
            gk, gt, _ = hist.backward(2.0 * (F - target), cg_tol=1e-13)
            out = (np.zeros_like(gk), np.zeros_like(gt))
            out[0][g.bond_perm] = gk
            out[1][g.bond_perm] = gt
        hist.close()
        g.close()
        return J, out

    J, (gk, gt) = run(Kn, Tv, 2, True)
    J1, (gk1, gt1) = run(Kn, Tv, 1, True)
    assert abs(J - J1) <= 1e-12 * abs(J)
    assert np.abs(gk - gk1).max() <= 1e-9 * np.abs(gk1).max()
    rng = np.random.default_rng(5)
    dKn = rng.uniform(-1, 1, Kn.shape) * Kn
    dTv = np.zeros_like(Tv)
    h = 1e-5
    fd = (run(Kn + h * dKn, Tv, 5, False)[0] - run(Kn - h * dKn, Tv, 5, False)[0]) / (2 * h)
    ad = float(gk @ dKn + gt @ dTv)
    assert abs(ad - fd) <= 1e-5 * abs(fd), (ad, fd)
