"""Material laws on the GPU (C ABI) against the reference goldens: J2 return
map, elastic-damage rate, HCF energy range, nonlocal averaging, static and
fatigue damage, and damage carried into the bond forces.  FP64 within 1e-12
relative to the largest entry of each field."""
import numpy as np
import pytest

from lpm_cases import golden, golden_meta, lat, make_gpu, pkg, rel
from test_oracle_laws import LAW_ID, PARAMS

capi = pkg.capi
pytestmark = pytest.mark.gpu
TOL = 1e-12


def gpu_for_law_golden(d):
    m = golden_meta(d)
    kind = str(d["_meta"][0])
    a = float(m["a"])
    cell = lat.UnitCell(lat.HEXAGON2D if kind.endswith("hex") else lat.SIMPLECUBIC3D, a / 2)
    xyz0 = d["xyz0"].reshape(-1, 3)
    g = make_gpu(cell.dim, xyz0, d["bond_p1"].astype(np.int32), d["bond_p2"].astype(np.int32),
                 d["bond_layer"].astype(np.int32), d["Kn"], d["Tv"], cell)
    law = m["law"]
    g.set_law(LAW_ID[law], PARAMS[law](m))
    g.set_types(d["types"], int(m.get("undamaged", 4)))
    g.set_nonlocal(d["nl_ptr"], d["nl_idx"], float(m["nonlocal_L"]))
    return g, law, m


def close(a, b, what):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    nan_a, nan_b = np.isnan(a), np.isnan(b)
    assert np.array_equal(nan_a, nan_b), what + " (NaN pattern)"
    assert rel(a[~nan_a], b[~nan_b]) <= TOL, what


def check_state(g, d, pfx):
    for key, fld in [("Pin", capi.F_PIN), ("stress", capi.F_STRESS), ("damage_visual", capi.F_DVIS)]:
        close(g.download(fld), d[pfx + key], pfx + key)
    for key, fld in [("bforce", capi.B_BFORCE), ("bdamage", capi.B_BDAMAGE)]:
        close(g.download(fld), d[pfx + key], pfx + key)


def check_laws(g, d, pfx):
    close(g.state(), d[pfx + "state_var"], pfx + "state_var")
    close(g.download(capi.F_DDOT_LOCAL), d[pfx + "ddot_local"], pfx + "ddot_local")
    close(g.download(capi.F_DDOT_NONLOCAL), d[pfx + "ddot_nonlocal"], pfx + "ddot_nonlocal")
    close(g.download(capi.F_DAMAGE), d[pfx + "damage"], pfx + "damage")
    close(g.download(capi.B_DLP), d[pfx + "dLp"], pfx + "dLp")


@pytest.mark.parametrize("name", ["law_damage_hex", "law_j2_sc", "law_j2_hex", "law_hcf_hex"])
def test_material_law_update_on_gpu(name):
    d = golden(name)
    g, law, m = gpu_for_law_golden(d)
    g.upload(capi.F_XYZ, d["a_xyz"])
    g.update()
    check_state(g, d, "a_")
    g.update_state()
    check_laws(g, d, "a_")
    if law == "hcf":
        g.upload(capi.F_XYZ, d["b_xyz"])
        g.update()
        check_state(g, d, "b_")
        g.update_state()
        check_laws(g, d, "b_")
        any_new = g.fatigue_damage(float(m["dNdt"]))
    else:
        any_new = g.update_damage()
    assert any_new == bool(d["any_damaged"][0])
    check_laws(g, d, "c_")
    g.update()
    check_state(g, d, "c_")
    g.close()
