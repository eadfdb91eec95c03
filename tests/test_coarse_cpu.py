"""The aggregates of the coarse-space preconditioner (lpm_coarse_boxes), on
the CPU: boxes of a given edge from the lowest corner of the particles'
bounding box, numbered by first particle, against a numpy restatement; the
automatic edge keeps the coarse DOFs near 480 and under the 1,024 cap on
the configurations' plates and cubes; bad arguments are refused."""
import numpy as np
import pytest

from lpm_cases import cube, pkg, plate

capi = pkg.capi


def _boxes(dim, x, edge):
    lo = x.min(axis=0)
    idx = np.floor((x[:, :dim] - lo[:dim]) / edge).astype(np.int64)
    _, first, inv = np.unique(idx, axis=0, return_index=True, return_inverse=True)
    order = np.argsort(first)                 # boxes in the order of their first particle
    rank = np.empty_like(order)
    rank[order] = np.arange(len(order))
    return rank[inv.ravel()], len(first)


@pytest.mark.parametrize("maker,args,box", [(plate, (41, 41), 2.0), (plate, (101, 101), 4.0), (cube, (21,), 1.0),
                                            (cube, (31,), 0.8)])
def test_boxes_match_restatement(maker, args, box):
    dim, xyz = maker(*args)[:2]
    agg, nagg, edge = capi.coarse_boxes(dim, xyz, box)
    ref, nref = _boxes(dim, xyz, box)
    assert edge == box and nagg == nref and np.array_equal(agg, ref)
    counts = np.bincount(agg, minlength=nagg)
    assert counts.min() >= 1 and counts.sum() == len(xyz)


@pytest.mark.parametrize("maker,args", [(plate, (101, 101)), (plate, (201, 401)), (cube, (41,)), (cube, (101,))])
def test_automatic_edge_stays_under_the_cap(maker, args):
    dim, xyz = maker(*args)[:2]
    agg, nagg, edge = capi.coarse_boxes(dim, xyz, 0.0)
    nm = 6 if dim == 3 else 3
    ext = np.prod(xyz.max(axis=0)[:dim] - xyz.min(axis=0)[:dim])
    assert edge == pytest.approx((ext / (480 // nm)) ** (1.0 / dim), rel=1e-12)
    assert nagg * nm <= 1024
    ref, nref = _boxes(dim, xyz, edge)
    assert nagg == nref and np.array_equal(agg, ref)
    print("[coarse boxes] %s%s: edge %.3f, %d boxes, %d coarse DOFs" % (maker.__name__, args, edge, nagg, nm * nagg))


def test_bad_arguments_refused():
    x = np.zeros((4, 3))
    for dim, box in ((4, 0.0), (2, -1.0), (2, float("nan"))):
        with pytest.raises(capi.LpmError) as e:
            capi.coarse_boxes(dim, x, box)
        assert e.value.code == capi.ERR_ARG


def test_empty_and_single_particle_inputs():
    agg, nagg, edge = capi.coarse_boxes(2, np.zeros((0, 3)), 1.0)
    assert nagg == 0 and len(agg) == 0 and edge == 1.0
    agg, nagg, edge = capi.coarse_boxes(3, np.array([[0.5, -1.0, 2.0]]), 0.0)
    assert nagg == 1 and agg.tolist() == [0] and edge > 0.0
