"""The CPU oracle against golden vectors produced by the reference headers.

The fixtures in tests/golden/ come from the reference's own code compiled
unmodified (tests/golden/make_golden.py); the oracle restatement must agree
with them bit for bit: topology, pattern, force state, tangent, CG solves and
whole load steps.
"""
import numpy as np
import pytest

from lpm_cases import golden, inputs_from_golden, make_oracle, mask3, oracle, dense_from_csc

KERNEL_CASES = ["kernels_hex", "kernels_sc", "kernels_hex_refmap", "kernels_sc_undamaged"]


@pytest.mark.parametrize("name", KERNEL_CASES)
def test_topology_and_pattern(name):
    d = golden(name)
    o = make_oracle(*inputs_from_golden(d))
    t = o.topology()
    assert np.array_equal(t["bp2"], d["bond_p2"])
    assert np.array_equal(t["blayer"], d["bond_layer"])
    assert np.array_equal(t["cptr"], d["conn_ptr"])
    assert np.array_equal(t["cidx"], d["conn_idx"])
    nb = np.diff(t["bptr"])
    assert np.array_equal(nb, d["nb"])


@pytest.mark.parametrize("name", KERNEL_CASES)
def test_force_state_tangent_cg(name):
    d = golden(name)
    dim, xyz0, p1, p2, layer, Kn, Tv, cell = inputs_from_golden(d)
    o = make_oracle(dim, xyz0, p1, p2, layer, Kn, Tv, cell)
    n = len(xyz0)
    o.set(oracle.XYZ, d["s_xyz"])
    o.set_bond(oracle.BDAMAGE, d["s_bdamage"])
    o.set_mask(mask3(d, n, dim))
    o.update()
    for key, fld in [("dLe_total", oracle.DLE_TOT), ("TdLe_total", oracle.TDLE_TOT), ("cs_sum", oracle.CS_SUM),
                     ("Pin", oracle.PIN), ("stress", oracle.STRESS), ("damage_visual", oracle.DVIS)]:
        assert np.array_equal(o.get(fld).ravel(), d["s_" + key]), key
    for key, fld in [("bforce", oracle.BFORCE), ("dLe", oracle.DLE)]:
        assert np.array_equal(o.get_bond(fld), d["s_" + key]), key
    r, nr, nR = o.residual()
    assert np.array_equal(r, d["residual"])
    assert nR == pytest.approx(np.linalg.norm(d["reaction"]), rel=1e-14)
    nd = n * dim
    o.assemble(sym=0, bc=0)
    assert np.array_equal(o.K_dense(), dense_from_csc(d["K_csc_outer"], d["K_csc_inner"], d["K_csc_values"], nd))
    x, it, err, st = o.cg(r, 1e-10)
    assert it == int(d["cg_iters"][0])
    assert np.array_equal(x, d["cg_disp"])
    o.assemble(sym=0, bc=1)
    assert np.array_equal(o.K_dense(), dense_from_csc(d["Kbc_csc_outer"], d["Kbc_csc_inner"], d["Kbc_csc_values"],
                                                      nd))
    x, it, err, st = o.cg(r, 1e-10)
    assert it == int(d["cgbc_iters"][0])
    assert np.array_equal(x, d["cgbc_disp"])


def test_symmetric_tangent_differs_only_in_diagonal_10():
    """The symmetric variant changes exactly the [1][0] entries of diagonal
    blocks, and with symmetric bond damage it makes K symmetric."""
    d = golden("kernels_sc_undamaged")
    dim, xyz0, p1, p2, layer, Kn, Tv, cell = inputs_from_golden(d)
    o = make_oracle(dim, xyz0, p1, p2, layer, Kn, Tv, cell)
    o.set(oracle.XYZ, d["s_xyz"])
    o.set_bond(oracle.BDAMAGE, d["s_bdamage"])
    o.update()
    o.assemble(sym=0, bc=0)
    K0 = o.K_dense()
    o.assemble(sym=1, bc=0)
    K1 = o.K_dense()
    diff = np.argwhere(K0 != K1)
    n = len(xyz0)
    for r, c in diff:
        assert r // dim == c // dim and r % dim == 1 and c % dim == 0
    for i in range(n):
        assert K1[dim * i + 1, dim * i] == K1[dim * i, dim * i + 1]
    assert np.abs(K1 - K1.T).max() <= 1e-12 * np.abs(K1).max()


@pytest.mark.parametrize("name", ["steps_hex_fatigue", "steps_sc_fatigue", "config1_hex"])
def test_load_steps_match_reference(name):
    from lpm_cases import golden_meta, tension_bcs
    d = golden(name)
    meta = golden_meta(d)
    dim, xyz0, p1, p2, layer, Kn, Tv, cell = inputs_from_golden(d)
    o = make_oracle(dim, xyz0, p1, p2, layer, Kn, Tv, cell)
    steps = int(meta["steps"])
    du = float(meta["du"])
    groups, apply, dd = tension_bcs(xyz0, dim, du)
    o.update()
    ax = 1 if dim == 2 else 2
    all_xyz = meta.get("all_xyz", "0") == "1"
    n = len(xyz0)
    xs = d["xyz_steps"].reshape(-1, n, 3)
    react = d["reaction_top_bottom"].reshape(-1, 2)
    for s in range(steps):
        o.load_step(apply, dd, sym=0, bc_elim=1, max_iter=30, tol=1e-5, cg_tol=1e-10)
        x = o.get(oracle.XYZ)
        if all_xyz or s == steps - 1:
            assert np.array_equal(x, xs[s if all_xyz else 0]), "step %d" % s
        pin = o.get(oracle.PIN)
        # sequential sums, as the driver adds them (cumsum is sequential;
        # Python's sum() is compensated since 3.12)
        assert np.cumsum(pin[groups["top"], ax])[-1] == react[s, 0]
        assert np.cumsum(pin[groups["bottom"], ax])[-1] == react[s, 1]
    assert np.array_equal(o.log()[:, 0].astype(np.int64), d["cg_iters"])
