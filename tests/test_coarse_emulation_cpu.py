"""The coarse-space preconditioner's algebra, restated on the CPU over the
oracle's eliminated symmetric tangent: P from the library's own aggregates
(lpm_coarse_boxes) and the rigid-body modes (translations, then the
rotation about z in 2-D or about x, y, z in 3-D, omega x (x0 - centroid)),
zero on eliminated DOFs; A_c = P^T K P; M = D^-1 + P A_c^-1 P^T.  PCG with it
reaches the Jacobi solution in a fraction of the iterations, A_c is
symmetric positive definite on the modes with stiffness, and M is
symmetric.  (The GPU path applies the same M: tests/test_gpu_coarse.py.)"""
import numpy as np
import pytest
import scipy.linalg as sla
import scipy.sparse as sp

from lpm_cases import cube, make_oracle, pkg, plate, tension_bcs

capi = pkg.capi


def _system(maker, args, du):
    dim, xyz, p1, p2, layer, Kn, Tv, cell = maker(*args)
    groups, apply, dd = tension_bcs(xyz, dim, du)
    o = make_oracle(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    o.update()
    o.apply_disp_bc(apply, dd)
    o.update()
    o.assemble(sym=1, bc=1)
    t = o.topology()
    n = len(xyz)
    K = sp.bsr_matrix((o.K_bsr(), t["cidx"], t["cptr"]), shape=(n * dim, n * dim)).tocsr()
    r, _, _ = o.residual()
    fixed = apply[:, :dim].ravel().astype(bool)
    return dim, xyz, K, r, fixed


def _prolongation(dim, xyz, fixed, box):
    agg, nagg, _ = capi.coarse_boxes(dim, xyz, box)
    nm = 6 if dim == 3 else 3
    cen = np.zeros((nagg, 3))
    np.add.at(cen, agg, xyz)
    cen /= np.bincount(agg, minlength=nagg)[:, None]
    d = (xyz - cen[agg]).astype(np.float32).astype(np.float64)  # the library keeps the offsets in FP32
    n = len(xyz)
    rows, cols, vals = [], [], []
    for k in range(dim):
        q = dim * np.arange(n) + k
        rows.append(q)
        cols.append(nm * agg + k)
        vals.append(np.ones(n))
        if dim == 2:
            rot = [(2, -d[:, 1] if k == 0 else d[:, 0])]
        else:
            rot = {0: [(4, d[:, 2]), (5, -d[:, 1])], 1: [(3, -d[:, 2]), (5, d[:, 0])],
                   2: [(3, d[:, 1]), (4, -d[:, 0])]}[k]
        for m, v in rot:
            rows.append(q)
            cols.append(nm * agg + m)
            vals.append(v)
    P = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n * dim, nm * nagg))
    return sp.diags((~fixed).astype(float)) @ P


def _pcg(K, b, M, tol=1e-10, maxit=20000):
    x = np.zeros_like(b)
    r = b.copy()
    z = M(r)
    p = z.copy()
    rz = r @ z
    nb = np.linalg.norm(b)
    for it in range(1, maxit + 1):
        q = K @ p
        a = rz / (p @ q)
        x += a * p
        r -= a * q
        if np.linalg.norm(r) < tol * nb:
            return x, it
        z = M(r)
        rz, rz_old = r @ z, rz
        p = z + (rz / rz_old) * p
    return x, maxit


@pytest.mark.parametrize("maker,args,du,box,frac", [(plate, (61, 61), 1e-3, 3.0, 0.3), (cube, (15,), 2e-3, 0.8, 0.7)])
def test_coarse_preconditioner_algebra(maker, args, du, box, frac):
    dim, xyz, K, r, fixed = _system(maker, args, du)
    Dinv = 1.0 / K.diagonal()
    x0, it0 = _pcg(K, r, lambda v: Dinv * v)
    P = _prolongation(dim, xyz, fixed, box)
    Ac = (P.T @ K @ P).toarray()
    assert np.abs(Ac - Ac.T).max() <= 1e-12 * np.abs(Ac).max()
    active = np.abs(np.diag(Ac)) > 1e-12 * np.abs(np.diag(Ac)).max()
    Ak = Ac[np.ix_(active, active)]
    assert np.linalg.eigvalsh(Ak).min() > 0.0
    Pk = P[:, active]
    cf = sla.cho_factor(Ak)
    M = lambda v: Dinv * v + Pk @ sla.cho_solve(cf, Pk.T @ v)
    u, w = np.random.default_rng(1).standard_normal((2, K.shape[0]))
    assert abs(u @ M(w) - w @ M(u)) <= 1e-10 * np.linalg.norm(u) * np.linalg.norm(M(w))
    x1, it1 = _pcg(K, r, M)
    print("[coarse emulation] %s%s box %.2f: %d coarse modes, Jacobi %d, coarse %d iterations; solutions %.1e apart" % (
        maker.__name__, args, box, int(active.sum()), it0, it1, np.abs(x1 - x0).max() / np.abs(x0).max()))
    assert it1 <= frac * it0
    assert np.abs(x1 - x0).max() <= 1e-8 * np.abs(x0).max()
