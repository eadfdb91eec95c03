"""GPU path (through the C ABI) against the reference goldens and the oracle.

Bars: integer work (bond order, opposite bonds, pattern) bit-exact; FP64
force state and tangent within 1e-12 relative to the largest entry; FP64
solves and load steps within the tolerances written at each assert.
"""
import numpy as np
import pytest

from lpm_cases import (cube, dense_from_bsr, dense_from_csc, golden, golden_meta, gpu_bcs, inputs_from_golden, lat,
                       make_gpu, make_oracle, mask3, oracle, pkg, plate, rel, tension_bcs)

capi = pkg.capi
pytestmark = pytest.mark.gpu

KERNEL_CASES = ["kernels_hex", "kernels_sc", "kernels_hex_refmap", "kernels_sc_undamaged"]
FP_TOL = 1e-12  # force state and tangent (FP64, different summation/FMA order)


def _gpu_at_golden_state(d):
    dim, xyz0, p1, p2, layer, Kn, Tv, cell = inputs_from_golden(d)
    g = make_gpu(dim, xyz0, p1, p2, layer, Kn, Tv, cell)
    g.upload(capi.F_XYZ, d["s_xyz"])
    g.upload(capi.B_BDAMAGE, d["s_bdamage"])
    g.set_mask(mask3(d, len(xyz0), dim))
    g.update()
    return g, dim, len(xyz0)


@pytest.mark.parametrize("name", KERNEL_CASES)
def test_topology_pattern_bit_exact(name):
    d = golden(name)
    dim, xyz0, p1, p2, layer, Kn, Tv, cell = inputs_from_golden(d)
    g = make_gpu(dim, xyz0, p1, p2, layer, Kn, Tv, cell)
    o = make_oracle(dim, xyz0, p1, p2, layer, Kn, Tv, cell)
    b = g.bonds()
    t = o.topology()
    assert np.array_equal(b["bptr"], t["bptr"])
    assert np.array_equal(b["bp2"], d["bond_p2"])
    assert np.array_equal(b["blayer"], d["bond_layer"])
    assert np.array_equal(b["opp"], t["opp"])
    cptr, cidx = g.pattern()
    assert np.array_equal(cptr, d["conn_ptr"])
    assert np.array_equal(cidx, d["conn_idx"])
    g.close()


@pytest.mark.parametrize("name", KERNEL_CASES)
def test_force_state(name):
    d = golden(name)
    g, dim, n = _gpu_at_golden_state(d)
    for key, fld in [("dLe_total", capi.F_DLE_TOT), ("TdLe_total", capi.F_TDLE_TOT), ("cs_sum", capi.F_CS_SUM),
                     ("Pin", capi.F_PIN), ("stress", capi.F_STRESS), ("damage_visual", capi.F_DVIS)]:
        assert rel(g.download(fld).ravel(), d["s_" + key]) <= FP_TOL, key
    for key, fld in [("bforce", capi.B_BFORCE), ("dLe", capi.B_DLE)]:
        assert rel(g.download(fld), d["s_" + key]) <= FP_TOL, key
    nr, nR = g.residual()
    assert rel(g.download(capi.F_RESIDUAL), d["residual"]) <= FP_TOL
    assert nR == pytest.approx(np.linalg.norm(d["reaction"]), rel=1e-12)
    g.close()


@pytest.mark.parametrize("name", KERNEL_CASES)
def test_tangent_as_written_and_eliminated(name):
    d = golden(name)
    g, dim, n = _gpu_at_golden_state(d)
    cptr, cidx = g.pattern()
    nd = n * dim
    g.assemble(capi.TANGENT_AS_WRITTEN, capi.BC_NONE)
    K = dense_from_bsr(cptr, cidx, g.K_bsr(), n, dim)
    assert rel(K, dense_from_csc(d["K_csc_outer"], d["K_csc_inner"], d["K_csc_values"], nd)) <= FP_TOL
    g.assemble(capi.TANGENT_AS_WRITTEN, capi.BC_ELIMINATE)
    K = dense_from_bsr(cptr, cidx, g.K_bsr(), n, dim)
    assert rel(K, dense_from_csc(d["Kbc_csc_outer"], d["Kbc_csc_inner"], d["Kbc_csc_values"], nd)) <= FP_TOL
    g.close()


@pytest.mark.parametrize("name", ["kernels_sc_undamaged", "kernels_hex"])
def test_symmetric_tangent_matches_oracle(name):
    d = golden(name)
    g, dim, n = _gpu_at_golden_state(d)
    o = make_oracle(*inputs_from_golden(d))
    o.set(oracle.XYZ, d["s_xyz"])
    o.set_bond(oracle.BDAMAGE, d["s_bdamage"])
    o.set_mask(mask3(d, n, dim))
    o.update()
    for bc in (0, 1):
        g.assemble(capi.TANGENT_SYMMETRIC, bc)
        o.assemble(sym=1, bc=bc)
        assert rel(g.K_bsr(), o.K_bsr()) <= FP_TOL
    g.close()


def test_cg_fp64_matches_oracle():
    """Symmetric, eliminated tangent of the undamaged cube: CG to 1e-10."""
    d = golden("kernels_sc_undamaged")
    g, dim, n = _gpu_at_golden_state(d)
    o = make_oracle(*inputs_from_golden(d))
    o.set(oracle.XYZ, d["s_xyz"])
    o.set_mask(mask3(d, n, dim))
    o.update()
    g.assemble(capi.TANGENT_SYMMETRIC, capi.BC_ELIMINATE)
    o.assemble(sym=1, bc=1)
    r, _, _ = o.residual()
    g.residual()
    it, rr, st = g.solve(capi.PREC_FP64, 1e-10)
    x, it_o, err_o, st_o = o.cg(r, 1e-10)
    assert st == 0 and st_o == 0
    assert abs(it - it_o) <= 2
    assert rr < 1e-10
    assert rel(g.download(capi.F_DISP), x) <= 1e-8
    g.close()


def test_cg_zero_rhs_and_maxit():
    dim, xyz, p1, p2, layer, Kn, Tv, cell = cube(4)
    g = make_gpu(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    g.update()
    g.residual()  # zero: undeformed, no loads
    g.assemble(capi.TANGENT_SYMMETRIC, capi.BC_NONE)
    it, rr, st = g.solve(capi.PREC_FP64, 1e-10)
    assert it == 0 and st == 0 and not np.any(g.download(capi.F_DISP))
    g.close()


def test_mixed_solve_graph_matches_host_launched_loop():
    """The mixed solve's graph (device-set loop and reliable-update
    conditions) runs the same kernels in the same order as the host-launched
    loop that kernel timing selects: identical iterates, bit for bit, on a
    relaunch too; the iteration cap and a zero right-hand side end it.  (The
    persistent loop, which this small system would take by default, folds
    its sums over other blocks: within the solve tolerance of the graph.)"""
    d = golden("kernels_sc_undamaged")
    g, dim, n = _gpu_at_golden_state(d)
    g.assemble(capi.TANGENT_SYMMETRIC, capi.BC_ELIMINATE)
    g.residual()
    g.set_cg_loop(capi.CG_LOOP_GRAPH)
    runs = []
    for timing in (False, True, False):
        g.set_kernel_timing(timing)
        g.reset_stats()
        it, rr, st = g.solve(capi.PREC_MIXED, 1e-10)
        s = g.stats()
        assert st == 0 and rr <= 1e-10 and it > 0
        runs.append((it, g.download(capi.F_DISP).copy(), s))
    g.set_kernel_timing(False)
    for it, x, _ in runs[1:]:
        assert it == runs[0][0]
        assert np.array_equal(x, runs[0][1])
    g.set_cg_loop(capi.CG_LOOP_PERSISTENT)
    it_p, rr_p, st_p = g.solve(capi.PREC_MIXED, 1e-10)
    assert st_p == 0 and rr_p <= 1e-10 and abs(it_p - runs[0][0]) <= 2
    assert rel(g.download(capi.F_DISP), runs[0][1]) <= 1e-8
    g.set_cg_loop(capi.CG_LOOP_AUTO)
    assert runs[0][2]["refine_sweeps"] == runs[1][2]["refine_sweeps"] > 0
    # the graph launches the product, the update and the direction update per
    # iteration, and the two reliable-update kernels only when one is due
    assert runs[0][2]["kernel_launches"] < runs[1][2]["kernel_launches"]
    it, rr, st = g.solve(capi.PREC_MIXED, 1e-10, maxit=5)
    assert st == capi.NOT_CONVERGED and it == 5
    g.close()
    dim, xyz, p1, p2, layer, Kn, Tv, cell = cube(4)
    g = make_gpu(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    g.update()
    g.residual()  # zero: undeformed, no loads
    g.assemble(capi.TANGENT_SYMMETRIC, capi.BC_NONE)
    it, rr, st = g.solve(capi.PREC_MIXED, 1e-10)
    assert it == 0 and st == 0 and not np.any(g.download(capi.F_DISP))
    g.close()


def test_fp64_solve_graph_matches_host_launched_loop():
    """The FP64 solve's graph and its host-launched loop give the same
    iterates, bit for bit; the iteration cap ends the graph too.  The
    persistent loop (this small system's default) agrees to the solve
    tolerance, within two iterations, and stops at the cap too."""
    d = golden("kernels_sc_undamaged")
    g, dim, n = _gpu_at_golden_state(d)
    g.assemble(capi.TANGENT_SYMMETRIC, capi.BC_ELIMINATE)
    g.residual()
    g.set_cg_loop(capi.CG_LOOP_GRAPH)
    runs = []
    for timing in (False, True, False):
        g.set_kernel_timing(timing)
        it, rr, st = g.solve(capi.PREC_FP64, 1e-10)
        assert st == 0 and rr <= 1e-10 and it > 0
        runs.append((it, g.download(capi.F_DISP).copy()))
    g.set_kernel_timing(False)
    for it, x in runs[1:]:
        assert it == runs[0][0] and np.array_equal(x, runs[0][1])
    it, rr, st = g.solve(capi.PREC_FP64, 1e-10, maxit=7)
    assert st == capi.NOT_CONVERGED and it == 7
    g.set_cg_loop(capi.CG_LOOP_PERSISTENT)
    g.reset_stats()
    it, rr, st = g.solve(capi.PREC_FP64, 1e-10)
    assert st == 0 and rr <= 1e-10 and abs(it - runs[0][0]) <= 2
    assert rel(g.download(capi.F_DISP), runs[0][1]) <= 1e-9
    assert g.stats()["persistent_solves"] == 1
    it, rr, st = g.solve(capi.PREC_FP64, 1e-10, maxit=7)
    assert st == capi.NOT_CONVERGED and it == 7
    g.close()


# FP64 load steps against the reference: the plain FP64 form's bar, 1e-10
# relative (displacements over their largest entry, and the top reaction).
# Measured on a GB300: 3e-13 to 9e-13 (hexagonal plates), 6e-14 (SC cube).
FP64_STEP_TOL = 1e-10


@pytest.mark.parametrize("name", ["steps_hex_fatigue", "steps_sc_fatigue", "config1_hex"])
def test_load_steps_as_written_match_reference(name):
    """SolverFatigue static steps (as-written tangent, BC elimination, FP64
    CG at 1e-10) against the reference's positions and reactions, within
    1e-10.  The SC case runs a CG that stalls near 1e-6 (the as-written
    tangent is not symmetric); both sides stall on the same iterates."""
    rtol = FP64_STEP_TOL
    d = golden(name)
    meta = golden_meta(d)
    dim, xyz0, p1, p2, layer, Kn, Tv, cell = inputs_from_golden(d)
    g = make_gpu(dim, xyz0, p1, p2, layer, Kn, Tv, cell)
    steps, du = int(meta["steps"]), float(meta["du"])
    groups, _, _ = tension_bcs(xyz0, dim, du)
    bcs = gpu_bcs(g, groups, dim, du)
    g.update()
    n = len(xyz0)
    xs = d["xyz_steps"].reshape(-1, n, 3)
    react = d["reaction_top_bottom"].reshape(-1, 2)
    all_xyz = meta.get("all_xyz", "0") == "1"
    ax = 1 if dim == 2 else 2
    for s in range(steps):
        res = g.load_step(bcs, solver=capi.SOLVER_FATIGUE_STATIC, tangent=capi.TANGENT_AS_WRITTEN,
                          precision=capi.PREC_FP64, max_iter=30, tol=1e-5, cg_tol=1e-10)
        assert res["status"] == 0
        x = g.download(capi.F_XYZ)
        if all_xyz or s == steps - 1:
            ref = xs[s if all_xyz else 0]
            err = rel(x - xyz0, ref - xyz0)
            print("[parity] %s step %d: displacement %.3e" % (name, s, err))
            assert err <= rtol, "step %d" % s
        pin = g.download(capi.F_PIN)
        rerr = abs(pin[groups["top"], ax].sum() - react[s, 0]) / abs(react[s, 0])
        print("[parity] %s step %d: top reaction %.3e" % (name, s, rerr))
        assert rerr <= rtol
    g.close()


@pytest.mark.parametrize("maker,args,du", [(plate, (21, 21), 1e-3), (cube, (9,), 2e-3)])
def test_symmetric_steps_fp64_and_mixed_match_oracle(maker, args, du):
    """Benchmark semantics (symmetric tangent, BC elimination): FP64 GPU vs
    oracle within 1e-10, mixed precision vs FP64 GPU within 1e-8."""
    dim, xyz, p1, p2, layer, Kn, Tv, cell = maker(*args)
    groups, apply, dd = tension_bcs(xyz, dim, du)
    o = make_oracle(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    o.update()
    outs = {}
    for prec in (capi.PREC_FP64, capi.PREC_MIXED):
        g = make_gpu(dim, xyz, p1, p2, layer, Kn, Tv, cell)
        bcs = gpu_bcs(g, groups, dim, du)
        g.update()
        for s in range(2):
            res = g.load_step(bcs, tangent=capi.TANGENT_SYMMETRIC, precision=prec, cg_tol=1e-10)
            assert res["status"] == 0
        outs[prec] = g.download(capi.F_XYZ) - xyz
        g.close()
    for s in range(2):
        o.load_step(apply, dd, sym=1, bc_elim=1, cg_tol=1e-10)
    uo = o.get(oracle.XYZ) - xyz
    e64, emx = rel(outs[capi.PREC_FP64], uo), rel(outs[capi.PREC_MIXED], outs[capi.PREC_FP64])
    print("[parity] %s%s: FP64 vs oracle %.3e, mixed vs FP64 %.3e" % (maker.__name__, args, e64, emx))
    assert e64 <= FP64_STEP_TOL
    assert emx <= 1e-8


def test_broken_bonds_carry_no_force():
    dim, xyz, p1, p2, layer, Kn, Tv, cell = plate(9, 9)
    g = make_gpu(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    rng = np.random.default_rng(3)
    g.upload(capi.F_XYZ, xyz + 0.01 * rng.standard_normal(xyz.shape) * np.array([1, 1, 0]))
    bd = np.zeros(g.nb)
    bd[::5] = 1.0
    g.upload(capi.B_BDAMAGE, bd)
    g.update()
    f = g.download(capi.B_BFORCE)
    assert np.all(f[bd == 1.0] == 0.0)
    assert np.all(g.download(capi.B_CS)[bd == 1.0] == 0.0)
    g.close()


def test_static_damage_breaks_bonds_like_oracle():
    dim, xyz, p1, p2, layer, Kn, Tv, cell = plate(9, 9)
    g = make_gpu(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    o = make_oracle(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    x = xyz.copy()
    x[:, 1] *= 1.002
    for s in (g, o):
        s.set_law(0, [1.2e-3])
    g.upload(capi.F_XYZ, x)
    o.set(oracle.XYZ, x)
    g.update()
    o.update()
    assert g.update_damage()
    # oracle: particle_elastic.h:52-68 through its own SolverStatic path
    bstrain = o.get_bond(oracle.BSTRAIN)
    expect = (bstrain >= 1.2e-3).astype(float)
    assert np.array_equal(g.download(capi.B_BDAMAGE), expect)
    g.close()


def test_errors_are_reported():
    dim, xyz, p1, p2, layer, Kn, Tv, cell = plate(5, 5)
    g = make_gpu(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    with pytest.raises(capi.LpmError) as e:
        g.K_bsr()
    assert e.value.code == capi.ERR_STATE
    with pytest.raises(capi.LpmError):
        g.add_group([0, 10 ** 6])
    g.close()


def test_isolated_particle():
    """A particle with no bonds has an empty pattern row (conns is empty)."""
    dim, xyz, p1, p2, layer, Kn, Tv, cell = plate(5, 5)
    xyz2 = np.vstack([xyz, [[100.0, 100.0, 0.0]]])
    g = make_gpu(dim, xyz2, p1, p2, layer, Kn, Tv, cell)
    o = make_oracle(dim, xyz2, p1, p2, layer, Kn, Tv, cell)
    cptr, cidx = g.pattern()
    t = o.topology()
    assert np.array_equal(cptr, t["cptr"]) and np.array_equal(cidx, t["cidx"])
    assert cptr[-1] == cptr[-2]
    g.close()


def test_short_rows_stored_past_the_groups():
    """Slices whose rows all hold fewer than four blocks keep every block in
    the one-per-slot tail of the sliced operator, and a slice can mix such
    rows with full plate rows: a 9x9 plate plus 40 two-particle chains, each
    chain held at one end and pulled by a force at the other.  FP64 load
    steps match the oracle within 1e-10, mixed ones the FP64 ones within
    1e-8."""
    dim, xyz, _, _, _, _, _, cell = plate(9, 9)
    n0, a = len(xyz), 0.5
    x0 = xyz[:, 0].max() + 4 * a
    ym = 0.5 * (xyz[:, 1].min() + xyz[:, 1].max())
    pairs = np.array([[x0 + 4 * a * k + a * e, ym, 0.0] for k in range(40) for e in (0, 1)])
    xyz = np.vstack([xyz, pairs])
    p1, p2, layer = lat.find_bonds(xyz, cell)
    Kn, Tv = lat.bond_constants(cell, layer, cell.elastic_constants(69e3, 0.3, plane_stress=True, layout="row"))
    left, right = n0 + 2 * np.arange(40), n0 + 2 * np.arange(40) + 1
    du = 1e-3
    groups, apply, dd = tension_bcs(xyz[:n0], dim, du)
    apply = np.vstack([apply, np.zeros((80, 3), np.int32)])
    dd = np.vstack([dd, np.zeros((80, 3))])
    apply[left, 0] = apply[left, 1] = apply[right, 1] = 1
    F = 1e-3 * a * Kn[(p1 == left[0]) & (p2 == right[0])][0]
    f = np.zeros((len(xyz), 3))
    f[right, 0] = F
    outs = {}
    for prec in (capi.PREC_FP64, capi.PREC_MIXED):
        g = make_gpu(dim, xyz, p1, p2, layer, Kn, Tv, cell)
        cptr, _ = g.pattern()
        rowlen = np.diff(cptr)
        assert rowlen[96:160].max() < 4 and rowlen[64:96].max() >= 4
        gl, gr = g.add_group(left), g.add_group(right)
        bcs = gpu_bcs(g, groups, dim, du) + [("disp", gl, 0, 0.0), ("disp", gl, 1, 0.0), ("disp", gr, 1, 0.0),
                                             ("force", gr, 40 * F, 0.0, 0.0)]  # a total, split over the group
        g.update()
        for _ in range(2):
            res = g.load_step(bcs, tangent=capi.TANGENT_SYMMETRIC, precision=prec, cg_tol=1e-10)
            assert res["status"] == 0
        outs[prec] = g.download(capi.F_XYZ) - xyz
        g.close()
    o = make_oracle(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    o.update()
    for _ in range(2):
        o.load_step(apply, dd, f, sym=1, bc_elim=1, cg_tol=1e-10)
    uo = o.get(oracle.XYZ) - xyz
    assert np.abs(uo[right, 0]).min() > 0
    assert rel(outs[capi.PREC_FP64], uo) <= FP64_STEP_TOL
    assert rel(outs[capi.PREC_MIXED], outs[capi.PREC_FP64]) <= 1e-8


def test_mixed_solve_with_wide_pattern_uses_32bit_columns():
    """A particle numbering whose column offsets do not fit 16 bits (a
    randomly permuted 33^3 cube, 35,937 particles) runs the FP32 product on
    32-bit column indices; its load step matches the FP64 one within 1e-8."""
    dim, xyz, p1, p2, layer, Kn, Tv, cell = cube(33)
    n = len(xyz)
    xyz = xyz[np.random.default_rng(4).permutation(n)]
    q1, q2, ql = lat.find_bonds(xyz, cell)
    Kn, Tv = lat.bond_constants(cell, ql, cell.elastic_constants(200e3, 0.3, layout="row"))
    groups, _, _ = tension_bcs(xyz, dim, 2e-3)
    outs = {}
    for prec in (capi.PREC_FP64, capi.PREC_MIXED):
        g = make_gpu(dim, xyz, q1, q2, ql, Kn, Tv, cell)
        cptr, cidx = g.pattern()
        rows = np.repeat(np.arange(n), np.diff(cptr))
        assert np.abs(cidx - rows).max() > 32767
        bcs = gpu_bcs(g, groups, dim, 2e-3)
        g.update()
        res = g.load_step(bcs, tangent=capi.TANGENT_SYMMETRIC, precision=prec, cg_tol=1e-10)
        assert res["status"] == 0
        outs[prec] = g.download(capi.F_XYZ) - xyz
        g.close()
    assert rel(outs[capi.PREC_MIXED], outs[capi.PREC_FP64]) <= 1e-8
