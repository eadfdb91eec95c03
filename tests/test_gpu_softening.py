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


def _sent_run(args, sc, scale_k, scale_sc, steps, tangents=False, precond=None):
    """The notched plate pulled `steps` times with the constants and the
    critical stretches scaled; per step the top reaction, the damage rounds
    and the damaged-bond pattern, and with `tangents` the reaction's
    derivatives along d/d(log E) and d/d(log lambda)."""
    dim, xyz, p1, p2, layer, Kn, Tv, cell = args
    g = make_gpu(dim, xyz, p1, p2, layer, Kn * scale_k, Tv * scale_k, cell)
    g.set_law(capi.LAW_SOFTENING, [3.0, 1.0e-3])
    g.upload(capi.B_SCRIT, sc * scale_sc)
    if precond is not None:
        g.set_preconditioner(precond, 0.0)
    g.update()
    c = xyz[:, 1]
    bottom, top = np.where(c < c.min() + 1e-9)[0], np.where(c > c.max() - 1e-9)[0]
    gb, gc, gt = g.add_group(bottom), g.add_group(bottom[:1]), g.add_group(top)
    bcs = [("disp", gb, 1, 0.0), ("disp", gc, 0, 0.0), ("disp", gt, 1, 2.5e-4)]
    if tangents:
        kn = g.download(capi.B_KN)
        tv = g.download(capi.B_TV)
        g.tangent_begin_softening([{"dKn": kn, "dTv": tv}, {"dscrit": g.download(capi.B_SCRIT)}], tol=1e-12)
    out = []
    for _ in range(steps):
        r = g.load_step(bcs, solver=capi.SOLVER_STATIC_ELIMINATE, tangent=capi.TANGENT_SYMMETRIC,
                        precision=capi.PREC_FP64, max_iter=400, tol=1e-10, cg_tol=1e-13, max_cuts=0)
        assert r["status"] == 0 and r["cuts"] == 0, r
        R = g.download(capi.F_PIN)[top, 1].sum()
        rec = dict(R=R, rounds=r["damage_rounds"], damaged=g.download(capi.B_BDAMAGE) > 0)
        if tangents:
            rec["dR"] = [g.tangent_get(k, capi.T_PIN)[top, 1].sum() for k in range(2)]
        out.append(rec)
    if tangents:
        g.tangent_end()
    g.close()
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("precond", ["jacobi", "coarse"])
def test_softening_reaction_tangents_match_central_differences(precond):
    """Configuration-3 sensitivities: the top reaction of each load step of
    the notched plate, differentiated along log E (all bond constants) and
    along log lambda (the scale of the Weibull critical stretches), by the
    forward-mode tangents that follow the damage rounds, against central
    differences of whole forward runs (h = 1e-4 relative, Newton to 1e-10).  Compared over
    the steps before any change of the discrete path (the damage rounds and
    the set of damaged bonds are the same in the base and both perturbed
    runs); at least one compared step must have softened bonds.  The peak
    reaction's derivative is that of the step where it peaks.  With the
    coarse-space preconditioner chosen, the tangents' BiCGSTAB solves use it
    too (the FP64 forward solves keep Jacobi), to the same bar."""
    args, sc = setup()
    steps, h = 6, 1e-4
    pre = capi.PRECOND_COARSE if precond == "coarse" else None
    base = _sent_run(args, sc, 1.0, 1.0, steps, tangents=True, precond=pre)
    runs = {(k, sgn): _sent_run(args, sc, *((1 + sgn * h, 1.0) if k == 0 else (1.0, 1 + sgn * h)), steps)
            for k in range(2) for sgn in (1, -1)}
    compared, softened = 0, 0
    for t in range(steps):
        same = all(runs[k, s][t]["rounds"] == base[t]["rounds"] and
                   np.array_equal(runs[k, s][t]["damaged"], base[t]["damaged"]) for k in range(2) for s in (1, -1))
        if not same:
            break
        for k in range(2):
            fd = (runs[k, 1][t]["R"] - runs[k, -1][t]["R"]) / (2 * h)
            tg = base[t]["dR"][k]
            err = abs(tg - fd) / max(abs(fd), 1e-12 * abs(base[t]["R"]))
            print("[softening tangent, %s] step %d dir %d: tangent %.9e FD %.9e rel %.2e rounds %d damaged %d" % (
                precond, t, k, tg, fd, err, base[t]["rounds"], int(base[t]["damaged"].sum())))
            assert err <= 1e-5, (t, k)
        compared += 1
        softened += bool(base[t]["damaged"].any())
    assert compared >= 3 and softened >= 1, (compared, softened)
    t_peak = int(np.argmax([b["R"] for b in base[:compared]]))
    assert base[t_peak]["dR"][0] != 0.0
