"""The allocation-free CG entry point, lpm_cg_solve_noalloc.

It serves callers that cannot allocate device memory while they solve: a
real-time loop that reserved its memory up front, or a host framework whose
allocator owns the device.  They
pass their own device buffers; the solver's scratch is a fixed device array
inside the library.  This test calls it through the C ABI twice in a row on
the same device and compares each result with lpm_solve on the same system.
The file is named to run last: if it fails, a run that stops at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from lpm_cases import cube, gpu_bcs, make_gpu, pkg, rel, tension_bcs

capi = pkg.capi
pytestmark = pytest.mark.gpu


def _operator_from_handle(g):
    """Block-CSR of the operator lpm_solve applies (A = K^T) on the host."""
    cptr, cidx = g.pattern()
    K = g.K_bsr()
    n, d = g.n, g.dim
    pos = {}
    for i in range(n):
        for q in range(cptr[i], cptr[i + 1]):
            pos[(i, int(cidx[q]))] = q
    vals = np.zeros_like(K)
    for j in range(n):  # row j of A holds K_ij^T for i in conns(j)
        for q in range(cptr[j], cptr[j + 1]):
            i = int(cidx[q])
            vals[q] = K[pos[(i, j)]].T
    return cptr, cidx, vals


def test_noalloc_solve_matches_lpm_solve_twice():
    import torch
    torch.cuda.init()
    dim, xyz, p1, p2, layer, Kn, Tv, cell = cube(7)
    groups, _, _ = tension_bcs(xyz, dim, 2e-3)
    g = make_gpu(dim, xyz, p1, p2, layer, Kn, Tv, cell)
    bcs = gpu_bcs(g, groups, dim, 2e-3)
    g.update()
    for b in bcs:
        g.apply_disp_bc(b[1], b[2], b[3])
    g.update()
    g.residual()
    g.assemble(capi.TANGENT_SYMMETRIC, capi.BC_ELIMINATE)
    it_ref, rr_ref, st = g.solve(capi.PREC_FP64, 1e-10)
    assert st == capi.OK
    x_ref = g.download(capi.F_DISP)
    rhs = g.download(capi.F_RESIDUAL)
    cptr, cidx, vals = _operator_from_handle(g)

    dev = torch.device("cuda:0")
    t_ptr = torch.from_numpy(cptr.astype(np.int64)).to(dev)
    t_col = torch.from_numpy(cidx.astype(np.int32)).to(dev)
    t_vals = torch.from_numpy(vals.ravel().copy()).to(dev)
    L = capi.load()
    f = L.lpm_cg_solve_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_double, ctypes.c_int64, ctypes.c_void_p,
                  ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double)]
    for call, scale in enumerate((1.0, -0.5)):  # two calls in a row, the second on another right-hand side
        t_b = torch.from_numpy(rhs * scale).to(dev)
        t_x = torch.full_like(t_b, float("nan"))  # the entry point must overwrite every entry
        torch.cuda.synchronize()
        it = ctypes.c_int64()
        rr = ctypes.c_double()
        st = f(dim, g.n, t_ptr.data_ptr(), t_col.data_ptr(), t_vals.data_ptr(), t_b.data_ptr(), t_x.data_ptr(),
               1e-10, -1, None, ctypes.byref(it), ctypes.byref(rr))
        assert st == capi.OK, L.lpm_last_error(None)
        torch.cuda.synchronize()
        x = t_x.cpu().numpy()
        assert rr.value <= 1e-10
        assert abs(it.value - it_ref) <= 2, (call, it.value, it_ref)
        assert rel(x, scale * x_ref) <= 1e-8, call
    # sizes beyond the fixed scratch are refused with a clear error
    st = f(3, (1 << 20) // 3 + 1, t_ptr.data_ptr(), t_col.data_ptr(), t_vals.data_ptr(), t_b.data_ptr(),
           t_x.data_ptr(), 1e-10, -1, None, None, None)
    assert st == capi.ERR_ARG and b"LPM_NOALLOC_MAX_DOF" in L.lpm_last_error(None)
    g.close()
