"""The softening bond law (configuration-3 form), on the oracle, and the
SENT set-up helpers.  The law has no reference class: the oracle states it
from its definition and these tests pin that statement to the formula."""
import math

import numpy as np

from lpm_cases import lat, make_oracle, oracle


def sent(ncol=21, nrow=31, a=0.1):
    xyz, p1, p2, layer, cell = lat.sent_plate(ncol, nrow, a)
    Kn, Tv = lat.bond_constants(cell, layer, cell.elastic_constants(69e3, 0.3, plane_stress=True, layout="row"))
    return xyz, p1, p2, layer, Kn, Tv, cell


def softening_d(kappa, sc, alpha):
    k = np.where(kappa > sc, kappa, sc)
    d = np.where(kappa > sc, 1.0 - (sc / k) * (alpha * sc - k) / ((alpha - 1.0) * sc), 0.0)
    return np.where(kappa >= alpha * sc, 1.0, d)


def test_precrack_removes_exactly_the_crossing_bonds():
    a, ncol, nrow = 0.1, 21, 31
    xyz = lat.hex_plate(ncol, nrow, a)
    cell = lat.UnitCell(lat.HEXAGON2D, a / 2)
    p1, p2, layer = lat.find_bonds(xyz, cell)
    k1, k2, kl = lat.sent_plate(ncol, nrow, a)[1:4]
    kept = set(zip(k1.tolist(), k2.tolist()))
    assert all((j, i) in kept for i, j in kept)  # both directed copies kept or removed together
    y0 = (nrow // 2 - 0.5) * a * math.sqrt(3.0) / 2.0
    x_tip = xyz[:, 0].min() + 0.3 * (xyz[:, 0].max() - xyz[:, 0].min())
    removed = 0
    for i, j in zip(p1.tolist(), p2.tolist()):
        yi, yj = xyz[i, 1], xyz[j, 1]
        crosses = (yi - y0) * (yj - y0) < 0 and xyz[i, 0] + (y0 - yi) / (yj - yi) * (xyz[j, 0] - xyz[i, 0]) < x_tip
        assert ((i, j) in kept) != crosses
        removed += crosses
    assert removed > 0 and len(k1) == len(p1) - removed


def test_weibull_draws_shared_by_directed_copies_and_distributed():
    xyz, p1, p2, layer, Kn, Tv, cell = sent(41, 61)
    s = lat.weibull_draws(p1, p2, 10.0, 1.2e-3, 20261203)
    d = dict(zip(zip(p1.tolist(), p2.tolist()), s.tolist()))
    assert all(d[(j, i)] == v for (i, j), v in d.items())
    mean = 1.2e-3 * math.gamma(1.0 + 1.0 / 10.0)
    assert abs(s.mean() - mean) < 0.02 * mean
    assert np.array_equal(s, lat.weibull_draws(p1, p2, 10.0, 1.2e-3, 20261203))


def test_oracle_softening_damage_matches_the_formula():
    xyz, p1, p2, layer, Kn, Tv, cell = sent()
    o = make_oracle(2, xyz, p1, p2, layer, Kn, Tv, cell)
    alpha = 3.0
    o.set_law(4, [alpha, 1.0e-3])
    perm = np.lexsort((layer, p1))
    sc = lat.weibull_draws(p1, p2, 10.0, 1.2e-3, 7)[perm]
    o.set_bond(oracle.SCRIT, sc)
    x = xyz.copy()
    x[:, 1] *= 1.0 + 2.0e-3  # uniaxial stretch: bonds see 0 .. 2e-3
    o.set(oracle.XYZ, x)
    o.update()
    new = o.static_damage()
    dis, dis0 = o.get_bond(oracle.DIS), o.get_bond(oracle.DIS0)
    kappa = (dis - dis0) / dis0
    d = o.get_bond(oracle.BDAMAGE)
    assert new
    assert np.array_equal(o.get_bond(oracle.KAPPA), np.maximum(kappa, 0.0))
    assert np.abs(d - softening_d(np.maximum(kappa, 0.0), sc, alpha)).max() <= 1e-15
    assert (d > 0).any() and (d < 1).any()
    # history: unloading keeps kappa and d; the law never heals
    o.set(oracle.XYZ, xyz)
    o.update()
    assert not o.static_damage()
    assert np.array_equal(o.get_bond(oracle.BDAMAGE), d)


def test_oracle_sent_steps_damage_the_crack_tip_first():
    xyz, p1, p2, layer, Kn, Tv, cell = sent()
    o = make_oracle(2, xyz, p1, p2, layer, Kn, Tv, cell)
    o.set_law(4, [3.0, 1.0e-3])
    perm = np.lexsort((layer, p1))
    o.set_bond(oracle.SCRIT, lat.weibull_draws(p1, p2, 10.0, 1.2e-3, 20261203)[perm])
    o.update()
    c = xyz[:, 1]
    n = len(xyz)
    apply = np.zeros((n, 3), np.int32)
    dd = np.zeros((n, 3))
    bottom, top = np.where(c < c.min() + 1e-9)[0], np.where(c > c.max() - 1e-9)[0]
    apply[bottom, 1] = 1
    apply[bottom[0], 0] = 1
    apply[top, 1] = 1
    dd[top, 1] = 2.5e-4
    for _ in range(40):
        r = o.load_step(apply, dd, sym=1, bc_elim=2, max_iter=60, tol=1e-9, cg_tol=1e-12)
        assert r >= 0
        d = o.get_bond(oracle.BDAMAGE)
        if (d > 0).any():
            break
    assert (d > 0).any()
    # damage starts at the crack tip
    b = int(np.argmax(d))
    bp1 = np.repeat(np.arange(n), np.diff(o.topology()["bptr"]))
    x_tip = xyz[:, 0].min() + 0.3 * (xyz[:, 0].max() - xyz[:, 0].min())
    y_crack = (31 // 2 - 0.5) * 0.1 * math.sqrt(3.0) / 2.0
    assert abs(xyz[bp1[b], 0] - x_tip) < 0.3 and abs(xyz[bp1[b], 1] - y_crack) < 0.2
