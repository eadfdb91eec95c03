"""Lattice generators and the createBonds rule (assembly.h:212-234)."""
import numpy as np
import pytest

from lpm_cases import golden, lat, make_oracle, plate


@pytest.mark.parametrize("name,kind,args,a", [("kernels_hex", "hex", (9, 9), 0.5), ("kernels_sc", "sc", (5, 5, 5), 0.2)])
def test_bonds_match_reference(name, kind, args, a):
    d = golden(name)
    if kind == "hex":
        cell = lat.UnitCell(lat.HEXAGON2D, a / 2)
        xyz = lat.hex_plate(*args, a)
    else:
        cell = lat.UnitCell(lat.SIMPLECUBIC3D, a / 2)
        xyz = lat.sc_cuboid(*args, a)
    assert np.array_equal(xyz.ravel(), d["xyz0"])
    p1, p2, layer = lat.find_bonds(xyz, cell)
    o = np.lexsort((p2, layer, p1))
    assert np.array_equal(p1[o], d["bond_p1"])
    assert np.array_equal(layer[o], d["bond_layer"])
    assert np.array_equal(p2[o], d["bond_p2"])


def test_reference_constants_layout():
    """Kn/Tv as the reference computes them (column-major Map of el_mapping)."""
    d = golden("kernels_hex_refmap")
    cell = lat.UnitCell(lat.HEXAGON2D, 0.25)
    kn0, kn1, tv = cell.elastic_constants(69e3, 0.3, plane_stress=True, layout="reference")
    assert np.all(d["Kn"] == kn0) and np.all(d["Tv"] == tv)
    d2 = golden("kernels_hex")
    kn0, kn1, tv = cell.elastic_constants(69e3, 0.3, plane_stress=True, layout="row")
    assert np.allclose(d2["Kn"], kn0, rtol=1e-15) and np.allclose(d2["Tv"], tv, rtol=1e-15)


def test_sc_row_constants_are_physical():
    cell = lat.UnitCell(lat.SIMPLECUBIC3D, 0.1)
    E, nu = 200e3, 0.3
    kn0, kn1, tv = cell.elastic_constants(E, nu, layout="row")
    G = E / 2 / (1 + nu)
    assert kn1 == pytest.approx(0.1 * G, rel=1e-14)
    assert tv == pytest.approx(0.1 * E * (4 * nu - 1) / (36 * (1 + nu) * (1 - 2 * nu)), rel=1e-12)


def test_configuration1_counts():
    dim, xyz, p1, p2, layer, Kn, Tv, cell = plate(41, 41)
    assert len(xyz) == 1661
    assert len(p1) == 19040
    o = make_oracle(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    assert o.nblk == 47877


@pytest.mark.slow
def test_configuration3_counts():
    dim, xyz, p1, p2, layer, Kn, Tv, cell = plate(201, 401, a=0.1)
    assert len(xyz) == 80401
    assert len(p1) == 958400
    o = make_oracle(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    assert o.nblk == 2466017


def test_interior_conns_counts():
    """Interior conns counts equal nneighbors_AFEM + 1 (unit_cell.h)."""
    from lpm_cases import cube
    for maker, args, nn in [(plate, (15, 15), 31), (cube, (9,), 61)]:
        dim, xyz, p1, p2, layer, Kn, Tv, cell = maker(*args)
        o = make_oracle(dim, xyz, p1, p2, layer, Kn, Tv, cell)
        counts = np.diff(o.topology()["cptr"])
        assert counts.max() == nn == cell.nneighbors_AFEM + 1


def test_nonlocal_neighbours_match_reference():
    d = golden("law_damage_hex")
    cell = lat.UnitCell(lat.HEXAGON2D, 0.25)
    xyz = d["xyz0"].reshape(-1, 3)
    ptr, idx = lat.nonlocal_neighbors(xyz, 1.5 * 0.6)
    assert np.array_equal(ptr, d["nl_ptr"]) and np.array_equal(idx, d["nl_idx"])


def test_elastic_constants_grad_matches_central_differences():
    for kind in (lat.HEXAGON2D, lat.SIMPLECUBIC3D, lat.FCC3D):
        c = lat.UnitCell(kind, 0.25)
        for ps in (False, True):
            E, nu, h = 69e3, 0.3, 1e-6
            g = c.elastic_constants_grad(E, nu, ps, "row")
            f = lambda E_, nu_: np.array(c.elastic_constants(E_, nu_, ps, layout="row"))  # noqa: E731
            fE = (f(E * (1 + h), nu) - f(E * (1 - h), nu)) / (2 * h * E)
            fn = (f(E, nu + h) - f(E, nu - h)) / (2 * h)
            assert np.abs(g[0] - fE).max() <= 1e-8 * np.abs(fE).max()
            assert np.abs(g[1] - fn).max() <= 1e-8 * np.abs(fn).max()
