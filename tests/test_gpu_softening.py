"""Configuration-3 form on the GPU: single-edge-notched hexagonal plate,
softening bond law with Weibull critical stretches, damage rounds on the
BC-eliminated tangent, against the oracle step by step."""
import math

import numpy as np
import pytest

from lpm_cases import lat, make_gpu, make_oracle, oracle, pkg

capi = pkg.capi


def setup(ncol=21, nrow=31, a=0.1, seed=20261203):
    xyz, p1, p2, layer, cell = lat.sent_plate(ncol, nrow, a)
    Kn, Tv = lat.bond_constants(cell, layer, cell.elastic_constants(69e3, 0.3, plane_stress=True, layout="row"))
    sc = lat.weibull_draws(p1, p2, 10.0, 1.2e-3, seed)[np.lexsort((layer, p1))]
    return (2, xyz, p1, p2, layer, Kn, Tv, cell), sc


@pytest.mark.gpu
@pytest.mark.parametrize("operator", [capi.OPERATOR_ASSEMBLED, capi.OPERATOR_MATRIX_FREE])
@pytest.mark.parametrize("precision", [capi.PREC_FP64, capi.PREC_MIXED])
def test_sent_softening_steps_match_oracle(precision, operator):
    """Both operator forms: the matrix-free one applies the same A = K^T,
    whose partially damaged bonds make it non-symmetric."""
    args, sc = setup()
    xyz = args[1]
    n = len(xyz)
    o = make_oracle(*args)
    g = make_gpu(*args)
    g.set_operator(operator)
    for s in (o, g):
        s.set_law(capi.LAW_SOFTENING, [3.0, 1.0e-3])
    o.set_bond(oracle.SCRIT, sc)
    g.upload(capi.B_SCRIT, sc)
    o.update()
    g.update()
    c = xyz[:, 1]
    bottom, top = np.where(c < c.min() + 1e-9)[0], np.where(c > c.max() - 1e-9)[0]
    du = 2.5e-4  # damage grows from step 3; the ligament bursts at step 7
    apply = np.zeros((n, 3), np.int32)
    dd = np.zeros((n, 3))
    apply[bottom, 1] = 1
    apply[bottom[0], 0] = 1
    apply[top, 1] = 1
    dd[top, 1] = du
    gb, gc, gt = g.add_group(bottom), g.add_group(bottom[:1]), g.add_group(top)
    bcs = [("disp", gb, 1, 0.0), ("disp", gc, 0, 0.0), ("disp", gt, 1, du)]
    # FP64 follows the oracle's arithmetic; the mixed form converges to the
    # same equilibrium within the Newton tolerance
    tol_u, tol_d = (1e-8, 1e-7) if precision == capi.PREC_FP64 else (1e-5, 1e-4)
    damaged_steps = 0
    for step in range(7):
        ro = o.load_step(apply, dd, sym=1, bc_elim=2, max_iter=60, tol=1e-9, cg_tol=1e-12)
        rg = g.load_step(bcs, solver=capi.SOLVER_STATIC_ELIMINATE, tangent=capi.TANGENT_SYMMETRIC,
                         precision=precision, max_iter=60, tol=1e-9, cg_tol=1e-12)
        assert ro >= 0 and rg["status"] == 0, (step, ro, rg)
        u_o = o.get(oracle.XYZ) - xyz
        u_g = g.download(capi.F_XYZ) - xyz
        d_o, d_g = o.get_bond(oracle.BDAMAGE), g.download(capi.B_BDAMAGE)
        print("[parity] softening prec %d step %d: displacement %.3e, bond damage %.3e (abs)" % (
            precision, step, np.abs(u_g - u_o).max() / np.abs(u_o).max(), np.abs(d_g - d_o).max()))
        assert np.abs(u_g - u_o).max() <= tol_u * np.abs(u_o).max(), step
        assert np.abs(d_g - d_o).max() <= tol_d, step
        assert np.array_equal(d_g > 0, d_o > 0), step
        k_o, k_g = o.get_bond(oracle.KAPPA), g.download(capi.B_KAPPA)
        assert np.abs(k_g - k_o).max() <= tol_u * max(np.abs(k_o).max(), 1e-12), step
        damaged_steps += bool((d_o > 0).any())
        # reaction on the pulled edge
        R_o = o.get(oracle.PIN)[top, 1].sum()
        R_g = g.download(capi.F_PIN)[top, 1].sum()
        assert abs(R_g - R_o) <= tol_u * abs(R_o)
    assert damaged_steps >= 2
    g.close()
