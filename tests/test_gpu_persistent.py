"""The persistent solve loops (lpm_set_cg_loop) against the graph loops: the
same recurrences (and, mixed, the same reliable updates) and stopping rule
run as one cooperative kernel whose blocks meet at grid barriers.  Load steps agree
to the solve tolerance and iteration counts within a few percent (the sums
are folded over another number of blocks, so the last bits differ), on 2-D
and 3-D lattices, with one row per thread and, forced on a lattice larger
than one resident wave, with several."""
import numpy as np
import pytest

from lpm_cases import cube, gpu_bcs, make_gpu, pkg, plate, rel, tension_bcs

capi = pkg.capi
pytestmark = pytest.mark.gpu


def _steps(case, loop, nsteps=2, precision=capi.PREC_MIXED):
    maker, args, du = case
    dim, xyz, p1, p2, layer, Kn, Tv, cell = maker(*args)
    groups, _, _ = tension_bcs(xyz, dim, du)
    g = make_gpu(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    g.set_cg_loop(loop)
    bcs = gpu_bcs(g, groups, dim, du)
    g.update()
    g.reset_stats()
    its, newton = [], 0
    for _ in range(nsteps):
        res = g.load_step(bcs, tangent=capi.TANGENT_SYMMETRIC, precision=precision, cg_tol=1e-10)
        assert res["status"] == capi.OK
        its.append(res["cg_iters"])
        newton += res["newton_iters"]
    u = g.download(capi.F_XYZ) - xyz
    st = g.stats()
    g.close()
    return u, its, st, newton


CASES = {"plate41": (plate, (41, 41), 1e-3), "cube21": (cube, (21,), 2e-3), "cube49": (cube, (49,), 2e-3)}


@pytest.mark.parametrize("name", list(CASES))
def test_persistent_loop_matches_graph_loop(name):
    """Two load steps: the forced persistent loop within 1e-8 of the graph
    loop (both solve to 1e-10) with iteration counts within 5 %; the
    automatic choice takes the persistent loop for the plate and the 21^3
    cube (one resident wave) and the graph for the 49^3 cube (more rows
    than resident threads, and an operator larger than half of L2)."""
    ug, itg, sg, _ = _steps(CASES[name], capi.CG_LOOP_GRAPH)
    up, itp, sp, newton = _steps(CASES[name], capi.CG_LOOP_PERSISTENT)
    ua, ita, sa, _ = _steps(CASES[name], capi.CG_LOOP_AUTO)
    print("[persistent] %s: graph %s, persistent %s (%d solves), auto %s (%d persistent); persistent vs graph %.2e" % (
        name, itg, itp, sp["persistent_solves"], ita, sa["persistent_solves"], rel(up, ug)))
    assert sg["persistent_solves"] == 0
    assert sp["persistent_solves"] >= newton > 0
    assert rel(up, ug) <= 1e-8
    assert abs(sum(itp) - sum(itg)) <= 0.05 * sum(itg) + 4
    if name == "cube49":
        assert sa["persistent_solves"] == 0 and ita == itg
    else:
        assert sa["persistent_solves"] == sp["persistent_solves"] and ita == itp
        assert np.array_equal(ua, up)  # the same grid: the same bits


def test_persistent_loop_iteration_cap_and_repeatability():
    """A solve capped at 7 iterations stops there with LPM_NOT_CONVERGED in
    both loops, from the same state; an uncapped persistent solve repeated
    on the same right-hand side gives the same bits and iteration count."""
    dim, xyz, p1, p2, layer, Kn, Tv, cell = plate(31, 31)
    groups, _, _ = tension_bcs(xyz, dim, 1e-3)
    g = make_gpu(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    bcs = gpu_bcs(g, groups, dim, 1e-3)
    g.update()
    assert g.load_step(bcs, tangent=capi.TANGENT_SYMMETRIC, precision=capi.PREC_FP64)["status"] == capi.OK
    g.assemble(capi.TANGENT_SYMMETRIC, capi.BC_ELIMINATE)
    rng = np.random.default_rng(11)
    b = rng.standard_normal(g.ndof)
    for loop in (capi.CG_LOOP_GRAPH, capi.CG_LOOP_PERSISTENT):
        g.set_cg_loop(loop)
        g.upload(capi.F_RESIDUAL, b)
        it, rr, st = g.solve(capi.PREC_MIXED, 1e-12, maxit=7)
        assert st == capi.NOT_CONVERGED and it == 7 and rr > 1e-12
    out = []
    for _ in range(2):
        g.upload(capi.F_RESIDUAL, b)
        it, rr, st = g.solve(capi.PREC_MIXED, 1e-10)
        assert st == capi.OK and rr <= 1e-10
        out.append((it, g.download(capi.F_DISP)))
    assert out[0][0] == out[1][0] and np.array_equal(out[0][1], out[1][1])
    with pytest.raises(capi.LpmError) as e:
        g.set_cg_loop(7)
    assert e.value.code == capi.ERR_ARG
    g.close()


@pytest.mark.parametrize("name", ["plate41", "cube21"])
def test_persistent_fp64_loop_matches_graph_and_oracle(name):
    """FP64 load steps: the persistent loop within 1e-10 of the graph loop
    and of the oracle (the plain FP64 form's bar), with the CG iteration
    counts within two per solve of the graph's."""
    from lpm_cases import make_oracle, oracle
    ug, itg, sg, _ = _steps(CASES[name], capi.CG_LOOP_GRAPH, precision=capi.PREC_FP64)
    up, itp, sp, newton = _steps(CASES[name], capi.CG_LOOP_PERSISTENT, precision=capi.PREC_FP64)
    maker, args, du = CASES[name]
    dim, xyz, p1, p2, layer, Kn, Tv, cell = maker(*args)
    _, apply, dd = tension_bcs(xyz, dim, du)
    o = make_oracle(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    o.update()
    for _ in range(2):
        o.load_step(apply, dd, sym=1, bc_elim=1, cg_tol=1e-10)
    uo = o.get(oracle.XYZ) - xyz
    print("[persistent fp64] %s: graph %s, persistent %s; persistent vs graph %.2e, vs oracle %.2e" % (
        name, itg, itp, rel(up, ug), rel(up, uo)))
    assert sg["persistent_solves"] == 0 and sp["persistent_solves"] >= newton > 0
    assert rel(up, ug) <= 1e-10 and rel(up, uo) <= 1e-10
    assert abs(sum(itp) - sum(itg)) <= 2 * newton
