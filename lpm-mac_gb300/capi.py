"""ctypes binding of liblpmgpu (include/lpm_gpu.h).

The library is the only implementation: if it is missing or fails to load
the calls raise, there is no fallback.
"""
import ctypes
import os

import numpy as np

from . import build as _build

# status codes
OK, NOT_CONVERGED = 0, 1
ERR_ARG, ERR_TOPOLOGY, ERR_CUDA, ERR_NOMEM, ERR_STATE, ERR_NONFINITE = -1, -2, -3, -4, -5, -6
# particle fields
F_XYZ, F_XYZ0, F_PIN, F_PEX, F_STRESS, F_DVIS, F_DLE_TOT, F_TDLE_TOT, F_CS_SUM, F_DAMAGE, F_XYZ_LAST, F_DISP, \
    F_RESIDUAL, F_STATE, F_DDOT_LOCAL, F_DDOT_NONLOCAL, F_DAMAGE_LAST = range(17)
# bond fields
B_BFORCE, B_BDAMAGE, B_DLE, B_DIS, B_BSTRAIN, B_CS, B_KN, B_TV, B_DIS0, B_DLP, B_SCRIT, B_KAPPA = range(100, 112)
TANGENT_AS_WRITTEN, TANGENT_SYMMETRIC = 0, 1
BC_NONE, BC_ELIMINATE = 0, 1
PREC_FP64, PREC_MIXED = 0, 1
BC_DISP, BC_FORCE = 0, 1
SOLVER_STATIC, SOLVER_FATIGUE_STATIC, SOLVER_STATIC_ELIMINATE = 0, 1, 2
LAW_ELASTIC, LAW_DAMAGE, LAW_J2, LAW_FATIGUE_HCF, LAW_SOFTENING = 0, 1, 2, 3, 4
T_PIN, T_XYZ, T_DAMAGE = 1, 2, 3  # tangent fields (lpm_tangent_get)
OPERATOR_ASSEMBLED, OPERATOR_MATRIX_FREE = 0, 1
CG_LOOP_AUTO, CG_LOOP_GRAPH, CG_LOOP_PERSISTENT = 0, 1, 2
PRECOND_JACOBI, PRECOND_COARSE = 0, 1
_NSTATE = {LAW_ELASTIC: 1, LAW_DAMAGE: 1, LAW_J2: 7, LAW_FATIGUE_HCF: 3, LAW_SOFTENING: 1}


class LpmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("liblpmgpu error %d: %s" % (code, msg))
        self.code = code


class Stats(ctypes.Structure):
    _fields_ = [("cg_iters_total", ctypes.c_int64), ("refine_sweeps", ctypes.c_int64),
                ("spmv_launches", ctypes.c_int64), ("spmv_ms", ctypes.c_double),
                ("spmv32_launches", ctypes.c_int64), ("spmv32_ms", ctypes.c_double),
                ("kernel_launches", ctypes.c_int64), ("mixed_fallbacks", ctypes.c_int64),
                ("tangent_cg_iters", ctypes.c_int64), ("persistent_solves", ctypes.c_int64)]


class BC(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("group", ctypes.c_int), ("mode", ctypes.c_int), ("axis", ctypes.c_int),
                ("value", ctypes.c_double), ("fx", ctypes.c_double), ("fy", ctypes.c_double),
                ("fz", ctypes.c_double)]


class StepOpts(ctypes.Structure):
    _fields_ = [("solver", ctypes.c_int), ("tangent", ctypes.c_int), ("precision", ctypes.c_int),
                ("max_iter", ctypes.c_int), ("tol", ctypes.c_double), ("cg_tol", ctypes.c_double),
                ("cg_maxit", ctypes.c_int64), ("max_cuts", ctypes.c_int)]


class CycleResult(ctypes.Structure):
    _fields_ = [("newton_iters", ctypes.c_int), ("unconverged_steps", ctypes.c_int), ("new_damage", ctypes.c_int),
                ("pad", ctypes.c_int), ("cg_iters", ctypes.c_int64)]


class FatigueRecord(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int64), ("dNdt", ctypes.c_int), ("newton_iters", ctypes.c_int),
                ("unconverged_steps", ctypes.c_int), ("new_damage", ctypes.c_int), ("cg_iters", ctypes.c_int64),
                ("mean_energy", ctypes.c_double)]


TIME_LINEAR, TIME_EXPONENTIAL = 0, 1


class AdjointResult(ctypes.Structure):
    _fields_ = [("cg_iters", ctypes.c_int64), ("relres", ctypes.c_double)]


class StepResult(ctypes.Structure):
    _fields_ = [("newton_iters", ctypes.c_int), ("cuts", ctypes.c_int), ("damage_rounds", ctypes.c_int),
                ("pad", ctypes.c_int), ("cg_iters", ctypes.c_int64)]


_lib = None


def library_path():
    return _build.LIB


def load(build_if_needed=True):
    """Loads liblpmgpu.so (building it first when sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_needed:
        _build.build()
    if not os.path.exists(_build.LIB):
        raise OSError("liblpmgpu.so is not built (%s)" % _build.LIB)
    L = ctypes.CDLL(_build.LIB)
    H = ctypes.c_void_p
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    i64p = ctypes.POINTER(ctypes.c_int64)
    i64 = ctypes.c_int64
    sigs = {
        "lpm_set_device": [ctypes.c_int],
        "lpm_create": [ctypes.c_int, ctypes.c_int, i64, dp, ip, ip, ip, dp, dp, ctypes.c_double, ctypes.c_int,
                       ctypes.POINTER(H)],
        "lpm_destroy": [H],
        "lpm_num_bonds": [H, i64p],
        "lpm_num_blocks": [H, i64p],
        "lpm_get_pattern": [H, i64p, ip],
        "lpm_get_bonds": [H, i64p, ip, ip, i64p],
        "lpm_upload": [H, ctypes.c_int, dp],
        "lpm_download": [H, ctypes.c_int, dp],
        "lpm_set_mask": [H, ip],
        "lpm_get_mask": [H, ip],
        "lpm_set_law": [H, ctypes.c_int, dp, ctypes.c_int, ctypes.c_int],
        "lpm_set_types": [H, ip, ctypes.c_int],
        "lpm_set_nonlocal": [H, i64p, ip, dp],
        "lpm_update_state": [H],
        "lpm_fatigue_damage": [H, ctypes.c_double, ip],
        "lpm_update_damage": [H, ip],
        "lpm_add_group": [H, ip, ctypes.c_int, ip],
        "lpm_apply_disp_bc": [H, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double],
        "lpm_apply_force_bc": [H, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double],
        "lpm_update_geometry_force": [H],
        "lpm_residual": [H, dp, dp],
        "lpm_assemble": [H, ctypes.c_int, ctypes.c_int],
        "lpm_get_K": [H, dp],
        "lpm_set_operator": [H, ctypes.c_int],
        "lpm_apply_operator": [H, ctypes.c_int, dp, dp],
        "lpm_solve": [H, ctypes.c_int, ctypes.c_double, i64, i64p, dp],
        "lpm_move_by_disp": [H],
        "lpm_newton": [H, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_double, i64, ip],
        "lpm_load_step": [H, ctypes.POINTER(BC), ctypes.c_int, ctypes.POINTER(StepOpts), ctypes.POINTER(StepResult)],
        "lpm_store_state": [H],
        "lpm_reset_state": [H, ctypes.c_int],
        "lpm_get_stats": [H, ctypes.POINTER(Stats)],
        "lpm_reset_stats": [H],
        "lpm_set_kernel_timing": [H, ctypes.c_int],
        "lpm_set_cg_loop": [H, ctypes.c_int],
        "lpm_set_preconditioner": [H, ctypes.c_int, ctypes.c_double],
        "lpm_coarse_boxes": [ctypes.c_int, ctypes.c_int, dp, ctypes.c_double, ip, ip, dp],
        "lpm_get_stream": [H, ctypes.POINTER(ctypes.c_void_p)],
        "lpm_synchronize": [H],
        "lpm_find_bonds": [ctypes.c_int, dp, ctypes.c_double, ctypes.c_double, i64, ip, ip, ip, i64p],
        "lpm_find_neighbors": [ctypes.c_int, dp, dp, i64, i64p, ip, i64p],
        "lpm_fatigue_cycle": [H, ctypes.POINTER(BC), ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                              ctypes.c_int, ctypes.c_double, ctypes.POINTER(StepOpts), ctypes.POINTER(CycleResult)],
        "lpm_fatigue_run": [H, ctypes.POINTER(BC), ctypes.c_int, dp, i64, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                            i64, ctypes.POINTER(StepOpts), ctypes.POINTER(FatigueRecord), i64, i64p],
        "lpm_backward_step": [H, dp, dp, ctypes.c_double, i64, ctypes.c_int, dp, dp, ctypes.POINTER(AdjointResult)],
        "lpm_apply_jacobian": [H, dp, dp],
        "lpm_tangent_begin": [H, ctypes.c_int, dp, ctypes.c_double],
        "lpm_tangent_bond_constants": [H, ctypes.c_int, dp, dp],
        "lpm_tangent_get": [H, ctypes.c_int, ctypes.c_int, dp],
        "lpm_tangent_bond_scrit": [H, ctypes.c_int, dp],
        "lpm_tangent_end": [H],
        "lpm_checkpoint_save": [H, ip],
        "lpm_checkpoint_restore": [H, ctypes.c_int],
        "lpm_checkpoint_drop": [H, ctypes.c_int],
    }
    for name, args in sigs.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    L.lpm_last_error.argtypes = [H]
    L.lpm_last_error.restype = ctypes.c_char_p
    _lib = L
    return L


def exported_symbols():
    """Names of the C-ABI entry points this binding uses."""
    return ["lpm_set_device", "lpm_create", "lpm_destroy", "lpm_last_error", "lpm_num_bonds", "lpm_num_blocks", "lpm_get_pattern",
            "lpm_get_bonds", "lpm_upload", "lpm_download", "lpm_set_mask", "lpm_get_mask", "lpm_set_law",
            "lpm_update_damage", "lpm_set_types", "lpm_set_nonlocal", "lpm_update_state", "lpm_fatigue_damage",
            "lpm_add_group", "lpm_apply_disp_bc", "lpm_apply_force_bc",
            "lpm_update_geometry_force", "lpm_residual", "lpm_assemble", "lpm_get_K", "lpm_set_operator",
            "lpm_apply_operator", "lpm_solve",
            "lpm_move_by_disp", "lpm_newton", "lpm_load_step", "lpm_store_state", "lpm_reset_state",
            "lpm_get_stats", "lpm_reset_stats", "lpm_set_kernel_timing", "lpm_set_cg_loop", "lpm_set_preconditioner", "lpm_coarse_boxes", "lpm_get_stream", "lpm_synchronize",
            "lpm_find_bonds", "lpm_find_neighbors", "lpm_fatigue_cycle", "lpm_fatigue_run", "lpm_backward_step", "lpm_apply_jacobian", "lpm_checkpoint_save", "lpm_checkpoint_restore",
            "lpm_checkpoint_drop", "lpm_tangent_begin", "lpm_tangent_bond_constants", "lpm_tangent_bond_scrit",
            "lpm_tangent_get",
            "lpm_tangent_end"]


def set_device(device):
    """Device for later Lattice() calls on this thread (the library's own CUDA runtime)."""
    L = load()
    st = L.lpm_set_device(int(device))
    if st != OK:
        raise LpmError(st, L.lpm_last_error(None).decode())


def find_bonds(xyz, cell):
    """Directed bonds (p1, p2, layer) of the createBonds rule, searched on
    the GPU (lpm_find_bonds); the same arrays as lattice.find_bonds."""
    L = load()
    x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    n = len(x)
    nb = ctypes.c_int64()
    null = ctypes.POINTER(ctypes.c_int)()
    st = L.lpm_find_bonds(n, _d(x), float(cell.neighbor_cutoff[0]), float(cell.neighbor_cutoff[1]), 0, null, null,
                          null, ctypes.byref(nb))
    if st != OK:
        raise LpmError(st, L.lpm_last_error(None).decode())
    p1 = np.zeros(nb.value, np.int32)
    p2 = np.zeros(nb.value, np.int32)
    layer = np.zeros(nb.value, np.int32)
    st = L.lpm_find_bonds(n, _d(x), float(cell.neighbor_cutoff[0]), float(cell.neighbor_cutoff[1]), nb.value, _i(p1),
                          _i(p2), _i(layer), ctypes.byref(nb))
    if st != OK:
        raise LpmError(st, L.lpm_last_error(None).decode())
    return p1, p2, layer


def find_neighbors(xyz, radius):
    """Nonlocal neighbour lists (searchNonlocalNeighbors) on the GPU: CSR
    (ptr, idx) of the ids closer than radius (scalar or per particle)."""
    L = load()
    x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    n = len(x)
    r = np.ascontiguousarray(np.broadcast_to(np.asarray(radius, dtype=np.float64), (n,)))
    tot = ctypes.c_int64()
    ptr = np.zeros(n + 1, np.int64)
    null = ctypes.POINTER(ctypes.c_int)()
    st = L.lpm_find_neighbors(n, _d(x), _d(r), 0, _l(ptr), null, ctypes.byref(tot))
    if st != OK:
        raise LpmError(st, L.lpm_last_error(None).decode())
    idx = np.zeros(tot.value, np.int32)
    st = L.lpm_find_neighbors(n, _d(x), _d(r), tot.value, _l(ptr), _i(idx), ctypes.byref(tot))
    if st != OK:
        raise LpmError(st, L.lpm_last_error(None).decode())
    return ptr, idx


def coarse_boxes(dim, xyz0, box=0.0):
    """The aggregates of the coarse-space preconditioner (lpm_coarse_boxes,
    host only): (aggregate id per particle, count, box edge used)."""
    L = load()
    x = np.ascontiguousarray(xyz0, dtype=np.float64).reshape(-1, 3)
    agg = np.zeros(len(x), np.int32)
    nagg = ctypes.c_int()
    edge = ctypes.c_double()
    st = L.lpm_coarse_boxes(int(dim), len(x), _d(x), float(box), _i(agg), ctypes.byref(nagg), ctypes.byref(edge))
    if st != OK:
        raise LpmError(st, L.lpm_last_error(None).decode())
    return agg, nagg.value, edge.value


def _d(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _i(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _l(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


_PWIDTH = {F_XYZ: 3, F_XYZ0: 3, F_PIN: 3, F_PEX: 3, F_STRESS: 6, F_DVIS: 1, F_DLE_TOT: 2, F_TDLE_TOT: 2,
           F_CS_SUM: 6, F_DAMAGE: 1, F_XYZ_LAST: 3, F_DDOT_LOCAL: 1, F_DDOT_NONLOCAL: 1, F_DAMAGE_LAST: 1}
_BWIDTH = {B_BFORCE: 1, B_BDAMAGE: 1, B_DLE: 1, B_DIS: 1, B_BSTRAIN: 1, B_CS: 3, B_KN: 1, B_TV: 1, B_DIS0: 1,
           B_DLP: 1, B_SCRIT: 1, B_KAPPA: 1}


class Lattice:
    """One lattice resident on the GPU (an lpm_handle)."""

    def __init__(self, dim, xyz, p1, p2, layer, Kn, Tv, particle_volume, nneighbors):
        L = load()
        self._L = L
        self.dim = int(dim)
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        self.n = xyz.shape[0]
        p1 = np.ascontiguousarray(p1, dtype=np.int32)
        p2 = np.ascontiguousarray(p2, dtype=np.int32)
        layer = np.ascontiguousarray(layer, dtype=np.int32)
        Kn = np.ascontiguousarray(Kn, dtype=np.float64)
        Tv = np.ascontiguousarray(Tv, dtype=np.float64)
        h = ctypes.c_void_p()
        st = L.lpm_create(self.dim, self.n, len(p1), _d(xyz), _i(p1), _i(p2), _i(layer), _d(Kn), _d(Tv),
                          float(particle_volume), int(nneighbors), ctypes.byref(h))
        if st != OK:
            raise LpmError(st, L.lpm_last_error(None).decode())
        self.h = h
        nb = ctypes.c_int64()
        L.lpm_num_bonds(h, ctypes.byref(nb))
        self.nb = nb.value
        nk = ctypes.c_int64()
        L.lpm_num_blocks(h, ctypes.byref(nk))
        self.nblk = nk.value
        self.ndof = self.dim * self.n
        # input index of each stored bond: stored order is by owner, then
        # layer, input order within (stable)
        self.bond_perm = np.lexsort((layer, p1))

    def close(self):
        if getattr(self, "h", None):
            self._L.lpm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, allow=(OK,)):
        if st not in allow:
            raise LpmError(st, self._L.lpm_last_error(self.h).decode())
        return st

    # -- transfers -------------------------------------------------------
    def download(self, field):
        if field == F_DISP or field == F_RESIDUAL:
            out = np.zeros(self.ndof)
        elif field >= 100:
            out = np.zeros(self.nb * _BWIDTH[field])
        else:
            out = np.zeros(self.n * _PWIDTH[field])
        self._check(self._L.lpm_download(self.h, field, _d(out)))
        if field >= 100:
            return out.reshape(self.nb, -1) if _BWIDTH[field] > 1 else out
        if field in (F_DISP, F_RESIDUAL):
            return out
        return out.reshape(self.n, -1) if _PWIDTH[field] > 1 else out

    def upload(self, field, values):
        v = np.ascontiguousarray(values, dtype=np.float64).ravel()
        self._check(self._L.lpm_upload(self.h, field, _d(v)))

    def set_mask(self, mask):
        m = np.ascontiguousarray(mask, dtype=np.int32).reshape(self.n, 3)
        self._check(self._L.lpm_set_mask(self.h, _i(m)))

    def get_mask(self):
        m = np.zeros((self.n, 3), np.int32)
        self._check(self._L.lpm_get_mask(self.h, _i(m)))
        return m

    def pattern(self):
        cptr = np.zeros(self.n + 1, np.int64)
        cidx = np.zeros(self.nblk, np.int32)
        self._check(self._L.lpm_get_pattern(self.h, _l(cptr), _i(cidx)))
        return cptr, cidx

    def bonds(self):
        bptr = np.zeros(self.n + 1, np.int64)
        bp2 = np.zeros(self.nb, np.int32)
        bl = np.zeros(self.nb, np.int32)
        opp = np.zeros(self.nb, np.int64)
        self._check(self._L.lpm_get_bonds(self.h, _l(bptr), _i(bp2), _i(bl), _l(opp)))
        return dict(bptr=bptr, bp2=bp2, blayer=bl, opp=opp)

    # -- physics -----------------------------------------------------------
    def set_law(self, law, params):
        """params: one row for all particles, or an (N, P) array per particle."""
        p = np.ascontiguousarray(params, dtype=np.float64)
        per = p.ndim == 2
        self._check(self._L.lpm_set_law(self.h, int(law), _d(p), p.shape[-1], int(per)))
        self.law = int(law)

    def set_types(self, types, undamaged):
        t = np.ascontiguousarray(types, dtype=np.int32)
        self._check(self._L.lpm_set_types(self.h, _i(t), int(undamaged)))

    def set_nonlocal(self, ptr, idx, L):
        ptr = np.ascontiguousarray(ptr, dtype=np.int64)
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        L = np.ascontiguousarray(np.broadcast_to(np.asarray(L, dtype=np.float64), (self.n,)))
        self._check(self._L.lpm_set_nonlocal(self.h, _l(ptr), _i(idx), _d(L)))

    def update_state(self):
        self._check(self._L.lpm_update_state(self.h))

    def fatigue_damage(self, dNdt):
        f = ctypes.c_int()
        self._check(self._L.lpm_fatigue_damage(self.h, float(dNdt), ctypes.byref(f)))
        return bool(f.value)

    def state(self):
        ns = _NSTATE[getattr(self, "law", LAW_ELASTIC)]
        out = np.zeros(self.n * ns)
        self._check(self._L.lpm_download(self.h, F_STATE, _d(out)))
        return out.reshape(self.n, ns)

    def update(self):
        self._check(self._L.lpm_update_geometry_force(self.h))

    def update_damage(self):
        f = ctypes.c_int()
        self._check(self._L.lpm_update_damage(self.h, ctypes.byref(f)))
        return bool(f.value)

    def residual(self):
        nr = ctypes.c_double()
        nR = ctypes.c_double()
        self._check(self._L.lpm_residual(self.h, ctypes.byref(nr), ctypes.byref(nR)))
        return nr.value, nR.value

    def assemble(self, tangent=TANGENT_SYMMETRIC, bc=BC_ELIMINATE):
        self._check(self._L.lpm_assemble(self.h, int(tangent), int(bc)))

    def set_operator(self, kind):
        """OPERATOR_ASSEMBLED (default) or OPERATOR_MATRIX_FREE; assemble again after a switch."""
        self._check(self._L.lpm_set_operator(self.h, int(kind)))

    def apply_operator(self, v, precision=PREC_FP64):
        """A' v with the operator the solves use (n*dim vectors)."""
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(self.ndof)
        y = np.zeros(self.ndof)
        self._check(self._L.lpm_apply_operator(self.h, int(precision), _d(v), _d(y)))
        return y

    def K_bsr(self):
        v = np.zeros(self.nblk * self.dim * self.dim)
        self._check(self._L.lpm_get_K(self.h, _d(v)))
        return v.reshape(self.nblk, self.dim, self.dim)

    def solve(self, precision=PREC_FP64, tol=1e-10, maxit=-1):
        it = ctypes.c_int64()
        rr = ctypes.c_double()
        st = self._check(self._L.lpm_solve(self.h, int(precision), float(tol), int(maxit), ctypes.byref(it),
                                           ctypes.byref(rr)), allow=(OK, NOT_CONVERGED))
        return it.value, rr.value, st

    def move_by_disp(self):
        self._check(self._L.lpm_move_by_disp(self.h))

    def newton(self, max_iter=30, tol=1e-5, precision=PREC_FP64, cg_tol=1e-10, cg_maxit=-1):
        ni = ctypes.c_int()
        st = self._check(self._L.lpm_newton(self.h, int(max_iter), float(tol), int(precision), float(cg_tol),
                                            int(cg_maxit), ctypes.byref(ni)), allow=(OK, NOT_CONVERGED))
        return ni.value, st

    def add_group(self, ids):
        a = np.ascontiguousarray(ids, dtype=np.int32)
        g = ctypes.c_int()
        self._check(self._L.lpm_add_group(self.h, _i(a), len(a), ctypes.byref(g)))
        return g.value

    def apply_disp_bc(self, group, axis, value, mode=0):
        self._check(self._L.lpm_apply_disp_bc(self.h, int(group), int(axis), int(mode), float(value)))

    def apply_force_bc(self, group, fx, fy, fz, mode=0):
        self._check(self._L.lpm_apply_force_bc(self.h, int(group), int(mode), float(fx), float(fy), float(fz)))

    @staticmethod
    def _bc_array(bcs):
        arr = (BC * max(len(bcs), 1))()
        for k, b in enumerate(bcs):
            if b[0] == "disp":
                arr[k] = BC(BC_DISP, int(b[1]), int(b[4]) if len(b) > 4 else 0, int(b[2]), float(b[3]), 0, 0, 0)
            else:
                arr[k] = BC(BC_FORCE, int(b[1]), int(b[5]) if len(b) > 5 else 0, 0, 0.0, float(b[2]), float(b[3]),
                            float(b[4]))
        return arr

    def fatigue_cycle(self, bcs_unit, f0, f1, f2, n_interval, dNdt, tangent=TANGENT_SYMMETRIC, precision=PREC_FP64,
                      max_iter=30, tol=1e-5, cg_tol=1e-10, cg_maxit=-1):
        """One cycle of lpm_fatigue_cycle; bcs_unit in load_step's form, for a
        unit load increment."""
        o = StepOpts(SOLVER_FATIGUE_STATIC, int(tangent), int(precision), int(max_iter), float(tol), float(cg_tol),
                     int(cg_maxit), 0)
        r = CycleResult()
        st = self._check(self._L.lpm_fatigue_cycle(self.h, self._bc_array(bcs_unit), len(bcs_unit), float(f0),
                                                   float(f1), float(f2), int(n_interval), float(dNdt),
                                                   ctypes.byref(o), ctypes.byref(r)), allow=(OK, NOT_CONVERGED))
        return dict(status=st, newton_iters=r.newton_iters, unconverged_steps=r.unconverged_steps,
                    new_damage=bool(r.new_damage), cg_iters=r.cg_iters)

    def fatigue_run(self, bcs_unit, spectrum, n_interval, tau, time_mode=TIME_LINEAR, max_cycles=0,
                    tangent=TANGENT_SYMMETRIC, precision=PREC_FP64, max_iter=30, tol=1e-5, cg_tol=1e-10, cg_maxit=-1):
        """lpm_fatigue_run: the whole cyclic loading inside the library, the
        spectrum on the device.  Returns (status, list of per-cycle records)."""
        sp = np.ascontiguousarray(spectrum, dtype=np.float64)
        o = StepOpts(SOLVER_FATIGUE_STATIC, int(tangent), int(precision), int(max_iter), float(tol), float(cg_tol),
                     int(cg_maxit), 0)
        nsim = int(max_cycles) if max_cycles > 0 else max(1, (len(sp) - 1) // 2)
        recs = (FatigueRecord * nsim)()
        n = ctypes.c_int64()
        st = self._check(self._L.lpm_fatigue_run(self.h, self._bc_array(bcs_unit), len(bcs_unit), _d(sp), len(sp),
                                                 int(n_interval), int(time_mode), float(tau), int(max_cycles),
                                                 ctypes.byref(o), recs, nsim, ctypes.byref(n)),
                         allow=(OK, NOT_CONVERGED))
        out = [{k: getattr(recs[i], k) for k, _ in FatigueRecord._fields_} for i in range(min(n.value, nsim))]
        return st, out

    def load_step(self, bcs, solver=SOLVER_FATIGUE_STATIC, tangent=TANGENT_SYMMETRIC, precision=PREC_FP64,
                  max_iter=30, tol=1e-5, cg_tol=1e-10, cg_maxit=-1, max_cuts=8):
        """bcs: list of ("disp", group, axis, value[, mode]) / ("force", group, fx, fy, fz[, mode])."""
        arr = (BC * max(len(bcs), 1))()
        for k, b in enumerate(bcs):
            if b[0] == "disp":
                arr[k] = BC(BC_DISP, int(b[1]), int(b[4]) if len(b) > 4 else 0, int(b[2]), float(b[3]), 0, 0, 0)
            else:
                arr[k] = BC(BC_FORCE, int(b[1]), int(b[5]) if len(b) > 5 else 0, 0, 0.0, float(b[2]), float(b[3]),
                            float(b[4]))
        o = StepOpts(int(solver), int(tangent), int(precision), int(max_iter), float(tol), float(cg_tol),
                     int(cg_maxit), int(max_cuts))
        r = StepResult()
        st = self._check(self._L.lpm_load_step(self.h, arr, len(bcs), ctypes.byref(o), ctypes.byref(r)),
                         allow=(OK, NOT_CONVERGED))
        return dict(status=st, newton_iters=r.newton_iters, cuts=r.cuts, damage_rounds=r.damage_rounds,
                    cg_iters=r.cg_iters)

    def store_state(self):
        self._check(self._L.lpm_store_state(self.h))

    def reset_state(self, reset_xyz=True):
        self._check(self._L.lpm_reset_state(self.h, int(bool(reset_xyz))))

    def stats(self):
        s = Stats()
        self._check(self._L.lpm_get_stats(self.h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def reset_stats(self):
        self._check(self._L.lpm_reset_stats(self.h))

    def set_cg_loop(self, mode):
        """CG_LOOP_AUTO (default), CG_LOOP_GRAPH or CG_LOOP_PERSISTENT: how the
        mixed solve runs its iteration loop."""
        self._check(self._L.lpm_set_cg_loop(self.h, int(mode)))

    def set_preconditioner(self, kind, box=0.0):
        """PRECOND_JACOBI (default) or PRECOND_COARSE (Jacobi plus the rigid-body
        modes of boxes of edge `box`, 0: automatic) for the mixed solve."""
        self._check(self._L.lpm_set_preconditioner(self.h, int(kind), float(box)))

    def set_kernel_timing(self, on):
        self._check(self._L.lpm_set_kernel_timing(self.h, int(bool(on))))

    def stream(self):
        p = ctypes.c_void_p()
        self._check(self._L.lpm_get_stream(self.h, ctypes.byref(p)))
        return p.value

    def synchronize(self):
        self._check(self._L.lpm_synchronize(self.h))

    # -- adjoint -----------------------------------------------------------
    def backward_step(self, dJdx=None, dJdpin=None, cg_tol=1e-10, cg_maxit=-1, accumulate=False):
        """Gradients of J = dJdx . x + dJdpin . Pin (arrays of N*dim, or None)
        with respect to every directed bond's Kn and Tv (stored bond order),
        at the current converged state.  Returns (dJ/dKn, dJ/dTv, cg_iters,
        relres)."""
        null = ctypes.POINTER(ctypes.c_double)()
        a = None if dJdx is None else np.ascontiguousarray(dJdx, dtype=np.float64).reshape(self.ndof)
        c = None if dJdpin is None else np.ascontiguousarray(dJdpin, dtype=np.float64).reshape(self.ndof)
        gk = np.zeros(self.nb)
        gt = np.zeros(self.nb)
        r = AdjointResult()
        self._check(self._L.lpm_backward_step(self.h, null if a is None else _d(a), null if c is None else _d(c),
                                              float(cg_tol), int(cg_maxit), int(bool(accumulate)), _d(gk), _d(gt),
                                              ctypes.byref(r)), allow=(OK, NOT_CONVERGED))
        return gk, gt, r.cg_iters, r.relres

    def apply_jacobian(self, v):
        """H v with H = dPin/dx at the current state (N*dim vectors)."""
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(self.ndof)
        y = np.zeros(self.ndof)
        self._check(self._L.lpm_apply_jacobian(self.h, _d(v), _d(y)))
        return y

    def tangent_begin(self, dparams, tol=1e-12, dbond=None):
        """Carries len(dparams) tangent directions through the following load
        steps (J2 law): each direction an (N, np) array, or one row of np
        values for all particles, of parameter changes.  dbond: per
        direction None or (dKn, dTv), the bond constants' changes in input
        bond order (for directions in E or nu)."""
        rows = []
        for d in dparams:
            d = np.asarray(d, dtype=np.float64)
            rows.append(np.broadcast_to(d, (self.n, d.shape[-1])))
        dp = np.ascontiguousarray(np.stack(rows)) if rows else np.zeros(1)
        self._check(self._L.lpm_tangent_begin(self.h, len(rows), _d(dp), float(tol)))
        for k, db in enumerate(dbond or []):
            if db is None:
                continue
            dkn = np.ascontiguousarray(np.asarray(db[0], dtype=np.float64)[self.bond_perm])
            dtv = np.ascontiguousarray(np.asarray(db[1], dtype=np.float64)[self.bond_perm])
            self._check(self._L.lpm_tangent_bond_constants(self.h, k, _d(dkn), _d(dtv)))

    def tangent_begin_softening(self, directions, tol=1e-12):
        """Tangents through the softening law's damage history (configuration
        3): one dict per direction with optional "dKn", "dTv" (changes of
        the bond constants) and "dscrit" (change of the critical stretch),
        each an array per directed bond in stored order (the order of
        download and of B_SCRIT uploads)."""
        null = ctypes.POINTER(ctypes.c_double)()
        self._check(self._L.lpm_tangent_begin(self.h, len(directions), null, float(tol)))
        for k, dr in enumerate(directions):
            if dr.get("dKn") is not None:
                dkn = np.ascontiguousarray(dr["dKn"], dtype=np.float64)
                dtv = np.ascontiguousarray(dr.get("dTv", np.zeros(self.nb)), dtype=np.float64)
                self._check(self._L.lpm_tangent_bond_constants(self.h, k, _d(dkn), _d(dtv)))
            if dr.get("dscrit") is not None:
                dsc = np.ascontiguousarray(dr["dscrit"], dtype=np.float64)
                self._check(self._L.lpm_tangent_bond_scrit(self.h, k, _d(dsc)))

    def tangent_get(self, direction, field=T_PIN):
        """The step's d Pin (T_PIN) or d x (T_XYZ) along one direction, (N, dim);
        T_DAMAGE: d damage per particle (N,)."""
        if field == T_DAMAGE:
            y = np.zeros(self.n)
            self._check(self._L.lpm_tangent_get(self.h, int(direction), int(field), _d(y)))
            return y
        y = np.zeros(self.ndof)
        self._check(self._L.lpm_tangent_get(self.h, int(direction), int(field), _d(y)))
        return y.reshape(self.n, self.dim)

    def tangent_end(self):
        self._check(self._L.lpm_tangent_end(self.h))

    def checkpoint_save(self):
        i = ctypes.c_int()
        self._check(self._L.lpm_checkpoint_save(self.h, ctypes.byref(i)))
        return i.value

    def checkpoint_restore(self, cid):
        self._check(self._L.lpm_checkpoint_restore(self.h, int(cid)))

    def checkpoint_drop(self, cid):
        self._check(self._L.lpm_checkpoint_drop(self.h, int(cid)))
