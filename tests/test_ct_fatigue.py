"""Configuration-5 form: compact-tension plate, HCF fatigue law with seeded
parameters, cyclic pin loading through lpm_fatigue_cycle against the same
cycle composed from the oracle's primitives (SolverFatigue::
solveProblemOneCycle, solver_fatigue.h:212-233)."""
import math

import numpy as np
import pytest

from lpm_cases import lat, make_gpu, make_oracle, oracle, pkg

capi = pkg.capi
W, A0, SP = 10.0, 0.4, 0.4
E, NU = 110e3, 0.34
F_MAX, R_RATIO = 100.0, 0.1
OPTS = dict(max_iter=30, tol=1e-9, cg_tol=1e-12)


def ct_case(seed=20261203):
    xyz, p1, p2, layer, cell, info = lat.ct_specimen(W, A0, SP)
    Kn, Tv = lat.bond_constants(cell, layer, cell.elastic_constants(E, NU, plane_stress=True, layout="row"))
    groups = lat.ct_groups(xyz, info, SP)
    n = len(xyz)
    rng = np.random.default_rng(seed)
    # HCF {A, B, d, threshold}: A and B drawn per particle, d fixed at the CT example's value
    params = np.stack([rng.uniform(1.5e-4, 2.5e-4, n), rng.uniform(0.50, 0.65, n), np.full(n, 1.079),
                       np.ones(n)], axis=1)
    (cx, cy_b), (_, cy_t) = info["holes"]
    r = info["radius"]
    types = np.zeros(n, np.int32)
    near_pins = (np.abs(xyz[:, 0] - cx) <= r) & ((xyz[:, 1] >= cy_t) | (xyz[:, 1] <= cy_b))
    types[near_pins] = 4
    L = 2.0 * SP
    nl_ptr, nl_idx = lat.nonlocal_neighbors(xyz, 1.5 * L)
    return (2, xyz, p1, p2, layer, Kn, Tv, cell), info, groups, params, types, (nl_ptr, nl_idx, L)


def test_ct_geometry():
    xyz, p1, p2, layer, cell, info = lat.ct_specimen(W, A0, SP)
    (cx, cy_b), (_, cy_t) = info["holes"]
    r = info["radius"]
    for cy in (cy_b, cy_t):
        assert (np.hypot(xyz[:, 0] - cx, xyz[:, 1] - cy) > r).all()
    tip = info["tip"]
    assert not lat._in_notch(xyz[:, 0], xyz[:, 1], tip, 0.026 * W).any()
    kept = set(zip(p1.tolist(), p2.tolist()))
    assert all((j, i) in kept for i, j in kept)
    # no bond bridges the notch: bonds joining the two faces end left of the tip
    x1, y1, x2, y2 = xyz[p1, 0], xyz[p1, 1], xyz[p2, 0], xyz[p2, 1]
    across = (y1 - info["crack_y"]) * (y2 - info["crack_y"]) < 0
    assert (np.minimum(x1, x2)[across] < tip[0] + SP).all()
    g = lat.ct_groups(xyz, info, SP)
    assert min(len(v) for v in g.values()) >= 2
    # the particle count of the full-size specimen (W = 40 mm, 0.15 mm spacing) is about 113k
    assert abs(1.25 * 40 * 1.2 * 40 / (0.15 ** 2 * math.sqrt(3) / 2) - 120e3) < 15e3


def oracle_cycle(o, apply, f_unit, f0, f1, f2, n_interval, dNdt):
    for inc in [(f1 - f0) / n_interval] * n_interval + [(f2 - f1) / n_interval] * n_interval:
        o.add_pex(f_unit * inc)
        o.apply_disp_bc(apply, np.zeros_like(f_unit))
        o.assemble(sym=1, bc=1)
        o.newton(OPTS["max_iter"], OPTS["tol"], OPTS["cg_tol"])
        o.update_state()
    new = o.fatigue_damage(dNdt)
    o.store_state()
    o.update()
    return new


def bc_arrays(n, groups):
    apply = np.zeros((n, 3), np.int32)
    apply[groups["mid"], 1] = 1
    apply[groups["top"], 0] = 1
    apply[groups["bottom"], 0] = 1
    f = np.zeros((n, 3))
    f[groups["top"], 1] = 1.0 / len(groups["top"])
    f[groups["bottom"], 1] = -1.0 / len(groups["bottom"])
    return apply, f


def test_oracle_ct_cycles_damage_the_notch_tip():
    args, info, groups, params, types, (nl_ptr, nl_idx, L) = ct_case()
    xyz = args[1]
    o = make_oracle(*args)
    o.set_law(3, params)
    o.set_types(types, 4)
    o.set_nonlocal(nl_ptr, nl_idx, np.full(len(xyz), L))
    o.update()
    apply, f = bc_arrays(len(xyz), groups)
    f_min = R_RATIO * F_MAX
    # static step to f_min (solveProblemStatic of the CT example), then cycles
    o.load_step(apply, np.zeros((len(xyz), 3)), f * f_min, sym=1, bc_elim=1, max_iter=30, tol=1e-9, cg_tol=1e-12)
    for _ in range(3):
        oracle_cycle(o, apply, f, f_min, F_MAX, f_min, 1, 1000)
    dmg = o.get(oracle.DAMAGE)
    assert dmg.max() > 0
    i = int(np.argmax(dmg))
    assert abs(xyz[i, 0] - info["tip"][0]) < 2.0 and abs(xyz[i, 1] - info["crack_y"]) < 1.0


@pytest.mark.gpu
def test_ct_fatigue_cycles_match_oracle():
    args, info, groups, params, types, (nl_ptr, nl_idx, L) = ct_case()
    xyz = args[1]
    n = len(xyz)
    o = make_oracle(*args)
    g = make_gpu(*args)
    o.set_law(3, params)
    g.set_law(capi.LAW_FATIGUE_HCF, params)
    o.set_types(types, 4)
    g.set_types(types, 4)
    o.set_nonlocal(nl_ptr, nl_idx, np.full(n, L))
    g.set_nonlocal(nl_ptr, nl_idx, L)
    o.update()
    g.update()
    apply, f = bc_arrays(n, groups)
    f_min = R_RATIO * F_MAX
    gm, gt, gb = g.add_group(groups["mid"]), g.add_group(groups["top"]), g.add_group(groups["bottom"])
    unit = [("disp", gm, 1, 0.0), ("disp", gt, 0, 0.0), ("disp", gb, 0, 0.0), ("force", gt, 0.0, 1.0, 0.0),
            ("force", gb, 0.0, -1.0, 0.0)]
    o.load_step(apply, np.zeros((n, 3)), f * f_min, sym=1, bc_elim=1, max_iter=30, tol=1e-9, cg_tol=1e-12)
    static = [("disp", gm, 1, 0.0), ("disp", gt, 0, 0.0), ("disp", gb, 0, 0.0), ("force", gt, 0.0, f_min, 0.0),
              ("force", gb, 0.0, -f_min, 0.0)]
    r = g.load_step(static, solver=capi.SOLVER_FATIGUE_STATIC, tangent=capi.TANGENT_SYMMETRIC, **OPTS)
    assert r["status"] == 0
    spectrum = pkg.fatigue.ca_spectrum(F_MAX, R_RATIO, 3000)
    recs = pkg.fatigue.run_cycles(g, unit, spectrum, 1, 0.001, max_calls=3, tangent=capi.TANGENT_SYMMETRIC, **OPTS)
    assert [rc["N"] for rc in recs] == [1000, 2000, 3000]
    for rc in recs:
        new_o = oracle_cycle(o, apply, f, f_min, F_MAX, f_min, 1, 1000)
        assert rc["status"] == 0 and rc["new_damage"] == new_o
    scale = np.abs(o.get(oracle.XYZ) - xyz).max()
    eu = np.abs((g.download(capi.F_XYZ) - xyz) - (o.get(oracle.XYZ) - xyz)).max() / scale
    print("[parity] CT fatigue: displacement %.3e, damage %.3e" % (
        eu, np.abs(g.download(capi.F_DAMAGE) - o.get(oracle.DAMAGE)).max() / o.get(oracle.DAMAGE).max()))
    assert eu <= 1e-10
    d_o, d_g = o.get(oracle.DAMAGE), g.download(capi.F_DAMAGE)
    assert d_o.max() > 0
    assert np.abs(d_g - d_o).max() <= 1e-10 * d_o.max()
    s_o, s_g = o.state(), g.state()
    assert np.abs(s_g - s_o).max() <= 1e-10 * np.abs(s_o).max()
    # the mean strain energy solveProblemCyclic prints (solver_fatigue.h:201-212)
    mean_o = s_o[types != 4, 0].mean()
    assert abs(recs[-1]["mean_energy"] - mean_o) <= 1e-10 * abs(mean_o)
    g.close()


def _ct_gpu():
    args, info, groups, params, types, (nl_ptr, nl_idx, L) = ct_case()
    g = make_gpu(*args)
    g.set_law(capi.LAW_FATIGUE_HCF, params)
    g.set_types(types, 4)
    g.set_nonlocal(nl_ptr, nl_idx, L)
    g.update()
    gm, gt, gb = g.add_group(groups["mid"]), g.add_group(groups["top"]), g.add_group(groups["bottom"])
    fixed = [("disp", gm, 1, 0.0), ("disp", gt, 0, 0.0), ("disp", gb, 0, 0.0)]
    f_min = R_RATIO * F_MAX
    r = g.load_step(fixed + [("force", gt, 0.0, f_min, 0.0), ("force", gb, 0.0, -f_min, 0.0)],
                    solver=capi.SOLVER_FATIGUE_STATIC, tangent=capi.TANGENT_SYMMETRIC, **OPTS)
    assert r["status"] == 0
    return g, fixed + [("force", gt, 0.0, 1.0, 0.0), ("force", gb, 0.0, -1.0, 0.0)]


@pytest.mark.gpu
@pytest.mark.parametrize("mode,tau", [(pkg.fatigue.LINEAR, 0.001), (pkg.fatigue.EXPONENTIAL, 0.5)])
def test_cyclic_driver_in_library_matches_per_cycle_calls(mode, tau):
    """lpm_fatigue_run (the spectrum on the device, the cycle loop inside
    the library) against the same loop driven from Python with one
    lpm_fatigue_cycle call per cycle: identical records and identical
    positions, damage and state, bit for bit, for the linear time map
    (dN/dt = 1000) and the exponential one (dN/dt = int(exp(t/tau)/tau) =
    2, 14, 109 for tau = 0.5)."""
    spectrum = pkg.fatigue.ca_spectrum(F_MAX, R_RATIO, 3000)
    # a spectrum whose amplitude varies, so the per-cycle loads differ
    spectrum = [v * (1.0 + 0.1 * math.sin(0.37 * k)) for k, v in enumerate(spectrum)]
    ga, unit_a = _ct_gpu()
    gb, unit_b = _ct_gpu()
    ra = pkg.fatigue.run_cycles(ga, unit_a, spectrum, 2, tau, mode=mode, max_calls=3, tangent=capi.TANGENT_SYMMETRIC,
                                **OPTS)
    rb = pkg.fatigue.run_cycles_per_call(gb, unit_b, spectrum, 2, tau, mode=mode, max_calls=3,
                                         tangent=capi.TANGENT_SYMMETRIC, **OPTS)
    assert len(ra) == len(rb) == 3
    for a, b in zip(ra, rb):
        for k in ("N", "dNdt", "newton_iters", "cg_iters", "unconverged_steps", "new_damage"):
            assert a[k] == b[k], k
    for fld in (capi.F_XYZ, capi.F_DAMAGE, capi.F_PEX):
        assert np.array_equal(ga.download(fld), gb.download(fld)), fld
    assert np.array_equal(ga.state(), gb.state())
    with pytest.raises(capi.LpmError) as e:
        ga.fatigue_run(unit_a, spectrum[:-1], 1, tau)  # an even count of spectrum values
    assert e.value.code == capi.ERR_ARG
    ga.close()
    gb.close()


def _ct_run(scale_a, shift_b, cycles, tangents=False):
    """The CT plate at test size: a static step to f_min, then `cycles`
    fatigue cycles (cycle jump 1000) through lpm_fatigue_run, with A scaled
    and B shifted; returns the particle damage, and with `tangents` its
    tangents along d/d(log A) and d/dB."""
    args, info, groups, params, types, (nl_ptr, nl_idx, L) = ct_case()
    p = params.copy()
    p[:, 0] *= scale_a
    p[:, 1] += shift_b
    g = make_gpu(*args)
    g.set_law(capi.LAW_FATIGUE_HCF, p)
    g.set_types(types, 4)
    g.set_nonlocal(nl_ptr, nl_idx, L)
    g.update()
    gm, gt, gb = g.add_group(groups["mid"]), g.add_group(groups["top"]), g.add_group(groups["bottom"])
    fixed = [("disp", gm, 1, 0.0), ("disp", gt, 0, 0.0), ("disp", gb, 0, 0.0)]
    opts = dict(tangent=capi.TANGENT_SYMMETRIC, precision=capi.PREC_FP64, **OPTS)
    f_min = R_RATIO * F_MAX
    r = g.load_step(fixed + [("force", gt, 0.0, f_min, 0.0), ("force", gb, 0.0, -f_min, 0.0)],
                    solver=capi.SOLVER_FATIGUE_STATIC, **opts)
    assert r["status"] == 0, r
    if tangents:
        da = np.zeros_like(p)
        da[:, 0] = p[:, 0]
        db = np.zeros_like(p)
        db[:, 1] = 1.0
        g.tangent_begin([da, db], tol=1e-12)
    unit = fixed + [("force", gt, 0.0, 1.0, 0.0), ("force", gb, 0.0, -1.0, 0.0)]
    spectrum = pkg.fatigue.ca_spectrum(F_MAX, R_RATIO, 1000 * cycles)
    recs = pkg.fatigue.run_cycles(g, unit, spectrum, 1, 0.001, **opts)
    assert len(recs) == cycles and all(rc["status"] == 0 for rc in recs), recs
    out = dict(D=g.download(capi.F_DAMAGE), info=info, xyz=args[1])
    if tangents:
        out["dD"] = [g.tangent_get(k, capi.T_DAMAGE) for k in range(2)]
        g.tangent_end()
    g.close()
    return out


@pytest.mark.gpu
def test_crack_length_tangents_match_central_differences():
    """Configuration-5 sensitivities: a crack-length measure after three
    fatigue cycles, the damage summed along the ligament ahead of the notch
    times the spacing, differentiated along log A and B (the two drawn HCF
    parameters, all particles at once) by the forward-mode tangents that
    follow the cycles, against central differences of whole runs
    (h = 1e-3; Newton to 1e-9), within 1e-5.  The particle damage tangents
    are checked too where the damage is above 1 % of its largest value."""
    base = _ct_run(1.0, 0.0, 3, tangents=True)
    xyz, info = base["xyz"], base["info"]
    lig = (np.abs(xyz[:, 1] - info["crack_y"]) < SP) & (xyz[:, 0] > info["tip"][0])
    crack = lambda D: SP * D[lig].sum()
    assert crack(base["D"]) > 0
    h = 1e-3
    for k, (dA, dB) in enumerate([((1 + h, 0.0), (1 - h, 0.0)), ((1.0, h), (1.0, -h))]):
        plus, minus = _ct_run(*dA, 3), _ct_run(*dB, 3)
        fd = (crack(plus["D"]) - crack(minus["D"])) / (2 * h)
        tg = SP * base["dD"][k][lig].sum()
        err = abs(tg - fd) / abs(fd)
        big = base["D"] > 0.01 * base["D"].max()
        fdD = (plus["D"] - minus["D"]) / (2 * h)
        errD = np.abs(base["dD"][k][big] - fdD[big]).max() / np.abs(fdD[big]).max()
        print("[crack-length tangent] dir %d: tangent %.9e FD %.9e rel %.2e; damage field rel %.2e" % (
            k, tg, fd, err, errD))
        assert err <= 1e-5 and errD <= 1e-4, (k, err, errD)
