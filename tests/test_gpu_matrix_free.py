"""The matrix-free tangent apply (lpm_set_operator) against the assembled
operator: the same products up to rounding on damaged and undamaged states,
for both tangent variants and both BC modes, and the same load steps."""
import numpy as np
import pytest

from lpm_cases import cube, golden, gpu_bcs, inputs_from_golden, make_gpu, make_oracle, mask3, oracle, pkg, plate, rel, \
    tension_bcs

capi = pkg.capi
pytestmark = pytest.mark.gpu


def _at_golden_state(name):
    d = golden(name)
    dim, xyz0, p1, p2, layer, Kn, Tv, cell = inputs_from_golden(d)
    g = make_gpu(dim, xyz0, p1, p2, layer, Kn, Tv, cell)
    g.upload(capi.F_XYZ, d["s_xyz"])
    g.upload(capi.B_BDAMAGE, d["s_bdamage"])
    g.set_mask(mask3(d, len(xyz0), dim))
    g.update()
    return g


@pytest.mark.parametrize("name", ["kernels_hex", "kernels_sc", "kernels_sc_undamaged"])
def test_products_match_assembled_operator(name):
    """FP64 products within 1e-12 of the assembled operator's, relative to
    the largest entry, on states with partial bond damage (where K is not
    symmetric and the product must be the one with A = K^T).  The FP32
    products of the mixed solve are as close to the FP64 product as the
    assembled FP32 operator's (within twice its error plus 1e-7), on a
    random vector and on a smooth one (a translation plus a small random
    part, whose product nearly cancels), where the difference form
    matters."""
    g = _at_golden_state(name)
    rng = np.random.default_rng(3)
    vr = rng.standard_normal(g.ndof)
    vs = np.tile(np.array([1.0, -0.5, 0.25])[:g.dim], g.n) + 1e-3 * rng.standard_normal(g.ndof)
    for tangent in (capi.TANGENT_AS_WRITTEN, capi.TANGENT_SYMMETRIC):
        for bc in (capi.BC_NONE, capi.BC_ELIMINATE):
            g.set_operator(capi.OPERATOR_ASSEMBLED)
            g.assemble(tangent, bc)
            ref = [g.apply_operator(v) for v in (vr, vs)]
            ref32 = [g.apply_operator(v, capi.PREC_MIXED) for v in (vr, vs)]
            g.set_operator(capi.OPERATOR_MATRIX_FREE)
            with pytest.raises(capi.LpmError):
                g.apply_operator(vr)  # not assembled after the switch
            g.assemble(tangent, bc)
            for v, y_ref, y32_ref in zip((vr, vs), ref, ref32):
                e64 = rel(g.apply_operator(v), y_ref)
                e32 = rel(g.apply_operator(v, capi.PREC_MIXED), y_ref)
                e32a = rel(y32_ref, y_ref)
                print("[matrix-free] %s tangent %d bc %d: FP64 %.2e, FP32 %.2e (assembled FP32 %.2e)" % (
                    name, tangent, bc, e64, e32, e32a))
                assert e64 <= 1e-12 and e32 <= 2 * e32a + 1e-7
            with pytest.raises(capi.LpmError) as e:
                g.K_bsr()
            assert e.value.code == capi.ERR_STATE
    g.close()


@pytest.mark.parametrize("maker,args,du", [(plate, (21, 21), 1e-3), (cube, (9,), 2e-3), (cube, (21,), 2e-3)])
def test_load_steps_match_assembled_and_oracle(maker, args, du):
    """Two load steps (symmetric tangent, BC elimination) with the
    matrix-free operator: FP64 within 1e-10 of the oracle, mixed within
    1e-8 of FP64; CG iteration counts printed beside the assembled ones."""
    dim, xyz, p1, p2, layer, Kn, Tv, cell = maker(*args)
    groups, apply, dd = tension_bcs(xyz, dim, du)
    o = make_oracle(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    o.update()
    for _ in range(2):
        o.load_step(apply, dd, sym=1, bc_elim=1, cg_tol=1e-10)
    uo = o.get(oracle.XYZ) - xyz
    out = {}
    for op in (capi.OPERATOR_ASSEMBLED, capi.OPERATOR_MATRIX_FREE):
        for prec in (capi.PREC_FP64, capi.PREC_MIXED):
            g = make_gpu(dim, xyz, p1, p2, layer, Kn, Tv, cell)
            g.set_operator(op)
            bcs = gpu_bcs(g, groups, dim, du)
            g.update()
            its = []
            for _ in range(2):
                res = g.load_step(bcs, tangent=capi.TANGENT_SYMMETRIC, precision=prec, cg_tol=1e-10)
                assert res["status"] == 0
                its.append(res["cg_iters"])
            out[op, prec] = (g.download(capi.F_XYZ) - xyz, its)
            g.close()
    mf64, mfmx = out[capi.OPERATOR_MATRIX_FREE, capi.PREC_FP64][0], out[capi.OPERATOR_MATRIX_FREE, capi.PREC_MIXED][0]
    print("[matrix-free] %s%s: FP64 vs oracle %.2e, mixed vs FP64 %.2e; CG iterations %s" % (
        maker.__name__, args, rel(mf64, uo), rel(mfmx, mf64), {k: v[1] for k, v in out.items()}))
    assert rel(mf64, uo) <= 1e-10
    assert rel(mfmx, mf64) <= 1e-8
