"""Failure branches of the load step, made on the host (no GPU fault).

- A load step whose modified Newton cannot converge in `max_iter`
  iterations is halved and re-inserted (solver_static.h:79-87), after
  resetting the state to the last converged one (assembly.h:140-166).
- lpm_reset_state restores positions, damage, plastic stretch and the bond
  state from the stored copy.
- A non-finite right-hand side or position ends the solve or the Newton
  iteration with LPM_ERR_NONFINITE; the mixed solve first falls back to
  FP64 and counts it.
- Brittle bond break (particle_elastic.h:52-68) with critical strains set
  exactly at, and one ulp either side of, bond strains: the GPU's strains
  are the reference's quotient dL/dis bit for bit, so the broken flags are
  identical.
"""
import numpy as np
import pytest

from lpm_cases import gpu_bcs, make_gpu, make_oracle, oracle, pkg, plate, rel, tension_bcs

capi = pkg.capi
pytestmark = pytest.mark.gpu

J2 = [69e3, 0.3, 100.0, 0.0, 1e3, 0.0, 0.0]  # E, nu, yield, xi, H, A, (unused)


def test_cut_back_halves_the_step_like_the_oracle():
    """A 15x15 hexagonal plate with the J2 law pulled by 0.2 mm (3 % strain)
    in one step with at most 4 Newton iterations: the step fails, is cut,
    and its halves (and quarters) are solved from the reset state.  The GPU
    takes at least one cut and ends where the oracle, running the same
    cut-back, ends: positions and plastic stretch within 1e-10."""
    dim, xyz, p1, p2, layer, Kn, Tv, cell = plate(15, 15)
    du = 0.2
    groups, apply, dd = tension_bcs(xyz, dim, du)
    o = make_oracle(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    o.set_law(capi.LAW_J2, J2)
    o.update()
    o.clear_log()
    assert o.load_step(apply, dd, sym=1, bc_elim=1, max_iter=4, cg_tol=1e-10, max_cuts=8) >= 0
    g = make_gpu(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    g.set_law(capi.LAW_J2, J2)
    bcs = gpu_bcs(g, groups, dim, du)
    g.update()
    res = g.load_step(bcs, tangent=capi.TANGENT_SYMMETRIC, precision=capi.PREC_FP64, max_iter=4, cg_tol=1e-10,
                      max_cuts=8)
    print("[cut-back] GPU", res, "oracle Newton solves", len(o.log()))
    assert res["status"] == capi.OK and res["cuts"] >= 1
    err = rel(g.download(capi.F_XYZ) - xyz, o.get(oracle.XYZ) - xyz)
    derr = rel(g.download(capi.B_DLP), o.get_bond(oracle.DLP))
    print("[cut-back] displacement %.3e, plastic stretch %.3e" % (err, derr))
    assert np.abs(o.get_bond(oracle.DLP)).max() > 0
    assert err <= 1e-10 and derr <= 1e-10
    # one cut too many: the step reports non-convergence after max_cuts
    g2 = make_gpu(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    g2.set_law(capi.LAW_J2, J2)
    bcs2 = gpu_bcs(g2, groups, dim, du)
    g2.update()
    res2 = g2.load_step(bcs2, tangent=capi.TANGENT_SYMMETRIC, precision=capi.PREC_FP64, max_iter=4, cg_tol=1e-10,
                        max_cuts=0)
    assert res2["status"] == capi.NOT_CONVERGED and res2["cuts"] == 1
    g.close()
    g2.close()


def test_reset_state_restores_the_stored_step():
    """lpm_reset_state(h, 0) restores damage, bond damage and plastic
    stretch and keeps the positions; lpm_reset_state(h, 1) also restores the
    positions (Assembly::resetStateVar, assembly.h:154-166)."""
    dim, xyz, p1, p2, layer, Kn, Tv, cell = plate(9, 9)
    groups, _, _ = tension_bcs(xyz, dim, 0.05)
    g = make_gpu(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    g.set_law(capi.LAW_J2, J2)
    bcs = gpu_bcs(g, groups, dim, 0.05)
    g.update()
    assert g.load_step(bcs, tangent=capi.TANGENT_SYMMETRIC, precision=capi.PREC_FP64)["status"] == capi.OK
    keep = {f: g.download(f).copy() for f in (capi.F_XYZ, capi.F_DAMAGE, capi.B_DLP, capi.B_BDAMAGE,
                                               capi.B_BFORCE, capi.B_DIS)}
    state = g.state().copy()
    assert np.abs(keep[capi.B_DLP]).max() > 0
    rng = np.random.default_rng(5)
    g.upload(capi.F_XYZ, keep[capi.F_XYZ] + 0.01 * rng.standard_normal(keep[capi.F_XYZ].shape))
    g.upload(capi.F_DAMAGE, np.full(g.n, 0.5))
    g.upload(capi.B_DLP, 2.0 * keep[capi.B_DLP] + 1e-4)
    g.upload(capi.B_BDAMAGE, np.full(g.nb, 0.25))
    g.update()  # bond force and length of the disturbed state
    moved = g.download(capi.F_XYZ).copy()
    g.reset_state(reset_xyz=False)
    for f in (capi.F_DAMAGE, capi.B_DLP, capi.B_BDAMAGE, capi.B_BFORCE, capi.B_DIS):
        assert np.array_equal(g.download(f), keep[f]), f
    assert np.array_equal(g.state(), state)
    assert np.array_equal(g.download(capi.F_XYZ), moved)
    g.reset_state(reset_xyz=True)
    assert np.array_equal(g.download(capi.F_XYZ), keep[capi.F_XYZ])
    g.close()


def test_nonfinite_right_hand_side_and_positions():
    """A NaN in the right-hand side: the FP64 solve returns
    LPM_ERR_NONFINITE; the mixed solve breaks down, is redone in FP64
    (counted in mixed_fallbacks) and returns the same.  A NaN position: the
    Newton iteration returns LPM_ERR_NONFINITE instead of taking the NaN
    residual as converged."""
    dim, xyz, p1, p2, layer, Kn, Tv, cell = plate(9, 9)
    groups, _, _ = tension_bcs(xyz, dim, 1e-3)
    g = make_gpu(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    bcs = gpu_bcs(g, groups, dim, 1e-3)
    g.update()
    assert g.load_step(bcs, tangent=capi.TANGENT_SYMMETRIC, precision=capi.PREC_FP64)["status"] == capi.OK
    g.assemble(capi.TANGENT_SYMMETRIC, capi.BC_ELIMINATE)
    r = np.ones(g.ndof)
    r[7] = np.nan
    for prec in (capi.PREC_FP64, capi.PREC_MIXED):
        g.upload(capi.F_RESIDUAL, r)
        g.reset_stats()
        with pytest.raises(capi.LpmError) as e:
            g.solve(prec, 1e-10)
        assert e.value.code == capi.ERR_NONFINITE
        assert g.stats()["mixed_fallbacks"] == (1 if prec == capi.PREC_MIXED else 0)
    # a finite right-hand side afterwards solves normally (no state left behind)
    g.upload(capi.F_RESIDUAL, np.ones(g.ndof))
    for prec in (capi.PREC_FP64, capi.PREC_MIXED):
        it, rr, st = g.solve(prec, 1e-10)
        assert st == capi.OK and rr <= 1e-10
    x = g.download(capi.F_XYZ)
    x[3, 0] = np.nan
    g.upload(capi.F_XYZ, x)
    with pytest.raises(capi.LpmError) as e:
        g.newton(precision=capi.PREC_FP64)
    assert e.value.code == capi.ERR_NONFINITE
    g.close()


def test_brittle_flags_at_the_threshold_bit_exact():
    """Each particle's critical strain is set to the largest strain among its
    bonds, exactly and one ulp above and below.  Bond lengths and strains on
    the GPU equal the oracle's (the reference's arithmetic) bit for bit, so
    the flags of bstrain >= critical agree in all three cases, and the three
    cases break different bond sets."""
    dim, xyz, p1, p2, layer, Kn, Tv, cell = plate(11, 11)
    rng = np.random.default_rng(7)
    x = xyz.copy()
    x[:, :2] += 0.004 * rng.standard_normal((len(x), 2))
    g = make_gpu(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    o = make_oracle(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    g.upload(capi.F_XYZ, x)
    o.set(oracle.XYZ, x)
    g.update()
    o.update()
    assert np.array_equal(g.download(capi.B_DIS), o.get_bond(oracle.DIS))
    so = o.get_bond(oracle.BSTRAIN)
    assert np.array_equal(g.download(capi.B_BSTRAIN), so)
    bptr = g.bonds()["bptr"]
    smax = np.maximum.reduceat(so, bptr[:-1])
    broken = []
    for crit in (smax, np.nextafter(smax, np.inf), np.nextafter(smax, -np.inf)):
        zero = np.zeros(g.nb)
        g.upload(capi.B_BDAMAGE, zero)
        o.set_bond(oracle.BDAMAGE, zero)
        g.set_law(capi.LAW_ELASTIC, crit[:, None])
        o.set_law(capi.LAW_ELASTIC, crit[:, None])
        g.update()
        o.update()
        g.update_damage()
        o.static_damage()
        bg, bo = g.download(capi.B_BDAMAGE), o.get_bond(oracle.BDAMAGE)
        assert np.array_equal(bg, bo)
        broken.append(int((bg == 1.0).sum()))
    print("[brittle] bonds broken at, above and below the threshold:", broken)
    assert broken[0] > 0 and broken[1] == 0 and broken[2] >= broken[0]
    g.close()
