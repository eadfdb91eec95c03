"""The oracle's material laws against the reference (goldens from
tests/golden/make_golden.py, case "laws"): state variables, local and
nonlocal damage rates, particle damage, plastic bond stretch, and the damage
carried into the bond forces.  Bit-exact."""
import numpy as np
import pytest

from lpm_cases import golden, golden_meta, make_oracle, oracle, lat

PARAMS = {
    # ParticleElasticDamage {k0, k1, damage_threshold}
    "damage": lambda m: [float(m.get("k0", 0.1936)), float(m.get("k1", 1.0)), float(m.get("dthr", 0.99))],
    # ParticleJ2Plasticity {E, mu, sigmay, xi, H, A, damage_threshold}; the
    # reference never sets damage_threshold for this class (stays 0)
    "j2": lambda m: [float(m.get("E", 110e3)), float(m.get("nu", 0.34)), float(m.get("sigmay", 900.0)),
                     float(m.get("xi", 0.3)), float(m.get("H", 1e3)), float(m.get("A", 0.5)), 0.0],
    # ParticleFatigueHCF {A, B, d, damage_threshold}
    "hcf": lambda m: [float(m.get("fA", 1.94e-4)), float(m.get("fB", 0.581)), float(m.get("fd", 1.079)),
                      float(m.get("dthr", 1.0))],
}
LAW_ID = {"damage": 1, "j2": 2, "hcf": 3}


def oracle_for_law_golden(d):
    m = golden_meta(d)
    kind = str(d["_meta"][0])
    a = float(m["a"])
    cell = lat.UnitCell(lat.HEXAGON2D if kind.endswith("hex") else lat.SIMPLECUBIC3D, a / 2)
    xyz0 = d["xyz0"].reshape(-1, 3)
    o = make_oracle(cell.dim, xyz0, d["bond_p1"].astype(np.int32), d["bond_p2"].astype(np.int32),
                    d["bond_layer"].astype(np.int32), d["Kn"], d["Tv"], cell)
    law = m["law"]
    o.set_law(LAW_ID[law], PARAMS[law](m))
    o.set_types(d["types"], int(m.get("undamaged", 4)))
    o.set_nonlocal(d["nl_ptr"], d["nl_idx"], float(m["nonlocal_L"]))
    return o, law, m


def check_state(o, d, pfx):
    for key, fld in [("Pin", oracle.PIN), ("stress", oracle.STRESS), ("damage_visual", oracle.DVIS),
                     ("dLe_total", oracle.DLE_TOT)]:
        assert np.array_equal(o.get(fld).ravel(), d[pfx + key], equal_nan=True), pfx + key
    for key, fld in [("bforce", oracle.BFORCE), ("bdamage", oracle.BDAMAGE), ("dLe", oracle.DLE)]:
        assert np.array_equal(o.get_bond(fld), d[pfx + key], equal_nan=True), pfx + key


def check_laws(o, d, pfx):
    assert np.array_equal(o.state().ravel(), d[pfx + "state_var"], equal_nan=True), pfx + "state_var"
    loc, nl = o.ddot()
    assert np.array_equal(loc, d[pfx + "ddot_local"], equal_nan=True), pfx + "ddot_local"
    assert np.array_equal(nl, d[pfx + "ddot_nonlocal"], equal_nan=True), pfx + "ddot_nonlocal"
    assert np.array_equal(o.get(oracle.DAMAGE), d[pfx + "damage"], equal_nan=True), pfx + "damage"
    assert np.array_equal(o.get_bond(oracle.DLP), d[pfx + "dLp"], equal_nan=True), pfx + "dLp"


@pytest.mark.parametrize("name", ["law_damage_hex", "law_j2_sc", "law_j2_hex", "law_hcf_hex"])
def test_material_law_update_matches_reference(name):
    d = golden(name)
    o, law, m = oracle_for_law_golden(d)
    o.set(oracle.XYZ, d["a_xyz"])
    o.update()
    check_state(o, d, "a_")
    o.update_state()
    check_laws(o, d, "a_")
    if law == "hcf":
        o.set(oracle.XYZ, d["b_xyz"])
        o.update()
        check_state(o, d, "b_")
        o.update_state()
        check_laws(o, d, "b_")
        any_new = o.fatigue_damage(float(m["dNdt"]))
    else:
        any_new = o.static_damage()
    assert any_new == bool(d["any_damaged"][0])
    check_laws(o, d, "c_")
    o.update()
    check_state(o, d, "c_")


def test_laws_do_something():
    """The fixtures exercise the interesting branches: yielding, damage growth,
    fatigue damage and damage carried into bonds."""
    d = golden("law_j2_sc")
    assert np.any(d["a_dLp"] != 0) and np.any(d["a_state_var"].reshape(-1, 7)[:, 0] > 0)
    d = golden("law_damage_hex")
    assert np.any(d["a_ddot_local"] > 0) and np.any(d["c_damage"] > 0) and np.any(d["c_bdamage"] > 0)
    d = golden("law_hcf_hex")
    assert np.any(d["c_damage"] > 0)
