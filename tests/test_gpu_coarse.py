"""The coarse-space preconditioner of the mixed solve (lpm_set_preconditioner):
Jacobi plus a correction on the rigid-body modes of boxes of particles.
Load steps reach the same solution as with Jacobi (within the solve
tolerance, and within 1e-8 of the oracle's FP64 steps) in far fewer CG
iterations; the iterates repeat bit for bit; the cases it does not serve
are refused."""
import numpy as np
import pytest

from lpm_cases import cube, gpu_bcs, make_gpu, make_oracle, oracle, pkg, plate, rel, tension_bcs

capi = pkg.capi
pytestmark = pytest.mark.gpu


def _run(case, precond, box=0.0, nsteps=2, loop=capi.CG_LOOP_AUTO):
    maker, args, du = case
    dim, xyz, p1, p2, layer, Kn, Tv, cell = maker(*args)
    groups, _, _ = tension_bcs(xyz, dim, du)
    g = make_gpu(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    g.set_preconditioner(precond, box)
    g.set_cg_loop(loop)
    bcs = gpu_bcs(g, groups, dim, du)
    g.update()
    g.reset_stats()
    its = []
    for _ in range(nsteps):
        r = g.load_step(bcs, tangent=capi.TANGENT_SYMMETRIC, precision=capi.PREC_MIXED, cg_tol=1e-10)
        assert r["status"] == capi.OK, r
        its.append(r["cg_iters"])
    u = g.download(capi.F_XYZ) - xyz
    st = g.stats()
    g.close()
    return u, its, st


def _oracle(case, nsteps=2):
    maker, args, du = case
    dim, xyz, p1, p2, layer, Kn, Tv, cell = maker(*args)
    _, apply, dd = tension_bcs(xyz, dim, du)
    o = make_oracle(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    o.update()
    for _ in range(nsteps):
        o.load_step(apply, dd, sym=1, bc_elim=1, cg_tol=1e-10)
    return o.get(oracle.XYZ) - xyz


CASES = {"plate101": ((plate, (101, 101), 1e-3), 4.0, 0.35),
         "cube21": ((cube, (21,), 2e-3), 1.0, 0.6)}


@pytest.mark.parametrize("name", list(CASES))
def test_coarse_preconditioner_matches_jacobi_in_fewer_iterations(name):
    """Two mixed load steps with Jacobi and with the coarse correction
    (boxes of 8 x 8 particles on the plate, 5 x 5 x 5 on the cube): both
    within 1e-8 of the oracle's FP64 steps, and the coarse one in at most
    the stated fraction of Jacobi's CG iterations (a CPU emulation of the
    same preconditioner on these tangents gave 68 against 576 iterations on
    the plate and 50 against 170 on a 31^3 cube)."""
    case, box, frac = CASES[name]
    uj, itj, sj = _run(case, capi.PRECOND_JACOBI)
    uc, itc, sc = _run(case, capi.PRECOND_COARSE, box)
    ua, ita, sa = _run(case, capi.PRECOND_COARSE, 0.0)
    uo = _oracle(case)
    print("[coarse] %s: Jacobi %s, coarse (box %.2f) %s, coarse (automatic box) %s; vs oracle %.2e, %.2e, %.2e" % (
        name, itj, box, itc, ita, rel(uj, uo), rel(uc, uo), rel(ua, uo)))
    assert rel(uj, uo) <= 1e-8 and rel(uc, uo) <= 1e-8 and rel(ua, uo) <= 1e-8
    assert sum(itc) <= frac * sum(itj)
    assert sc["persistent_solves"] > 0


def test_coarse_preconditioner_repeats_and_refusals():
    """The same bits on a repeated coarse-preconditioned solve (forced even
    under the graph loop setting); LPM_ERR_STATE with the tangent as written
    or the matrix-free operator; LPM_ERR_ARG for boxes that give more than
    1,024 coarse DOFs or a negative edge."""
    dim, xyz, p1, p2, layer, Kn, Tv, cell = plate(61, 61)
    groups, _, _ = tension_bcs(xyz, dim, 1e-3)
    g = make_gpu(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    bcs = gpu_bcs(g, groups, dim, 1e-3)
    g.update()
    assert g.load_step(bcs, tangent=capi.TANGENT_SYMMETRIC, precision=capi.PREC_FP64)["status"] == capi.OK
    g.assemble(capi.TANGENT_SYMMETRIC, capi.BC_ELIMINATE)
    b = np.random.default_rng(3).standard_normal(g.ndof)
    g.set_preconditioner(capi.PRECOND_COARSE, 3.0)
    g.set_cg_loop(capi.CG_LOOP_GRAPH)
    out = []
    for _ in range(2):
        g.upload(capi.F_RESIDUAL, b)
        it, rr, st = g.solve(capi.PREC_MIXED, 1e-10)
        assert st == capi.OK and rr <= 1e-10
        out.append((it, g.download(capi.F_DISP)))
    assert out[0][0] == out[1][0] and np.array_equal(out[0][1], out[1][1])
    g.set_preconditioner(capi.PRECOND_JACOBI)
    g.upload(capi.F_RESIDUAL, b)
    it_j, rr_j, _ = g.solve(capi.PREC_MIXED, 1e-10)
    print("[coarse] plate 61x61 random right-hand side: Jacobi %d, coarse %d iterations; solutions %.2e apart" % (
        it_j, out[0][0], rel(out[0][1], g.download(capi.F_DISP))))
    assert rel(out[0][1], g.download(capi.F_DISP)) <= 1e-8 and out[0][0] < it_j
    g.set_preconditioner(capi.PRECOND_COARSE, 0.3)  # about 3,700 boxes
    g.upload(capi.F_RESIDUAL, b)
    with pytest.raises(capi.LpmError) as e:
        g.solve(capi.PREC_MIXED, 1e-10)
    assert e.value.code == capi.ERR_ARG
    with pytest.raises(capi.LpmError) as e:
        g.set_preconditioner(capi.PRECOND_COARSE, -1.0)
    assert e.value.code == capi.ERR_ARG
    g.set_preconditioner(capi.PRECOND_COARSE, 0.0)
    g.assemble(capi.TANGENT_AS_WRITTEN, capi.BC_ELIMINATE)
    with pytest.raises(capi.LpmError) as e:
        g.solve(capi.PREC_MIXED, 1e-10)
    assert e.value.code == capi.ERR_STATE
    g.set_operator(capi.OPERATOR_MATRIX_FREE)
    g.assemble(capi.TANGENT_SYMMETRIC, capi.BC_ELIMINATE)
    with pytest.raises(capi.LpmError) as e:
        g.solve(capi.PREC_MIXED, 1e-10)
    assert e.value.code == capi.ERR_STATE
    g.close()
