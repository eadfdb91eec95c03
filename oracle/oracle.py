"""ctypes binding of the CPU oracle (oracle/lpm_oracle.cpp).

TEST INFRASTRUCTURE: only tests/, ``__graft_entry__.smoke()`` and the CPU
baseline of bench.py import this module, and only as the checker.  The
product path (the package's CUDA library) never calls it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblpm_oracle.so")

_lib = None

# particle / bond field ids (lpm_oracle.h)
XYZ, XYZ0, PIN, PEX, STRESS, DVIS, DLE_TOT, TDLE_TOT, CS_SUM, DAMAGE, XYZ_LAST, STATE, DDOT_LOCAL = range(13)
BFORCE, BDAMAGE, DLE, DIS, BSTRAIN, CS, KN, TV, DIS0, DLP, SCRIT, KAPPA = range(12)

_PWIDTH = {XYZ: 3, XYZ0: 3, PIN: 3, PEX: 3, STRESS: 6, DVIS: 1, DLE_TOT: 2, TDLE_TOT: 2, CS_SUM: 6,
           DAMAGE: 1, XYZ_LAST: 3, DDOT_LOCAL: 1}
_BWIDTH = {BFORCE: 1, BDAMAGE: 1, DLE: 1, DIS: 1, BSTRAIN: 1, CS: 3, KN: 1, TV: 1, DIS0: 1, DLP: 1, SCRIT: 1,
           KAPPA: 1}


def build(force=False):
    """Compiles the oracle with oracle/Makefile (gcc, OpenMP)."""
    if force or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "lpm_oracle.cpp")):
        subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        lp = ctypes.POINTER(ctypes.c_long)
        L.lo_create.restype = P
        L.lo_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_long, dp, ip, ip, ip, dp, dp, ctypes.c_double,
                                ctypes.c_int, ip]
        L.lo_destroy.argtypes = [P]
        L.lo_set_threads.argtypes = [ctypes.c_int]
        L.lo_num_bonds.restype = ctypes.c_long
        L.lo_num_bonds.argtypes = [P]
        L.lo_num_blocks.restype = ctypes.c_long
        L.lo_num_blocks.argtypes = [P]
        L.lo_get_topology.argtypes = [P, lp, ip, ip, lp, lp, lp, ip]
        for f in ("lo_get_particle", "lo_set_particle", "lo_get_bond", "lo_set_bond"):
            getattr(L, f).argtypes = [P, ctypes.c_int, dp]
        L.lo_set_mask.argtypes = [P, ip]
        L.lo_set_law.argtypes = [P, ctypes.c_int, dp, ctypes.c_int, ctypes.c_int]
        L.lo_set_types.argtypes = [P, ip, ctypes.c_int]
        L.lo_set_nonlocal.argtypes = [P, lp, ip, dp]
        L.lo_update_state.argtypes = [P]
        L.lo_static_damage.argtypes = [P]
        L.lo_static_damage.restype = ctypes.c_int
        L.lo_fatigue_damage.argtypes = [P, ctypes.c_double]
        L.lo_fatigue_damage.restype = ctypes.c_int
        L.lo_get_ddot.argtypes = [P, dp, dp]
        L.lo_num_state.argtypes = [P]
        L.lo_num_state.restype = ctypes.c_int
        L.lo_update_geometry_force.argtypes = [P]
        L.lo_residual.argtypes = [P, dp, dp, dp]
        L.lo_assemble.argtypes = [P, ctypes.c_int, ctypes.c_int]
        L.lo_get_K.argtypes = [P, dp]
        L.lo_cg.restype = ctypes.c_int
        L.lo_cg.argtypes = [P, dp, dp, ctypes.c_double, ctypes.c_long, lp, dp]
        L.lo_newton.restype = ctypes.c_int
        L.lo_newton.argtypes = [P, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_long]
        L.lo_log_size.restype = ctypes.c_long
        L.lo_log_size.argtypes = [P]
        L.lo_get_log.argtypes = [P, dp]
        L.lo_clear_log.argtypes = [P]
        L.lo_apply_disp_bc.argtypes = [P, ip, dp]
        L.lo_add_pex.argtypes = [P, dp]
        L.lo_load_step.restype = ctypes.c_int
        L.lo_load_step.argtypes = [P, ip, dp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_long, ctypes.c_int]
        L.lo_store_state.argtypes = [P]
        L.lo_reset_state.argtypes = [P, ctypes.c_int]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _i(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _l(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_long))


class OracleSystem:
    """One lattice held by the CPU oracle (flat arrays, reference semantics)."""

    def __init__(self, dim, xyz, p1, p2, layer, Kn, Tv, particle_volume, nneighbors):
        L = lib()
        self.dim = int(dim)
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        self.n = self.xyz.shape[0]
        p1 = np.ascontiguousarray(p1, dtype=np.int32)
        p2 = np.ascontiguousarray(p2, dtype=np.int32)
        layer = np.ascontiguousarray(layer, dtype=np.int32)
        Kn = np.ascontiguousarray(Kn, dtype=np.float64)
        Tv = np.ascontiguousarray(Tv, dtype=np.float64)
        err = ctypes.c_int(0)
        h = L.lo_create(self.dim, self.n, len(p1), _d(self.xyz), _i(p1), _i(p2), _i(layer), _d(Kn), _d(Tv),
                        float(particle_volume), int(nneighbors), ctypes.byref(err))
        if not h:
            raise ValueError("oracle rejected the lattice (code %d)" % err.value)
        self.h = h
        self.nb = L.lo_num_bonds(h)
        self.nblk = L.lo_num_blocks(h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().lo_destroy(self.h)
            self.h = None

    def topology(self):
        bptr = np.zeros(self.n + 1, np.int64)
        bp2 = np.zeros(self.nb, np.int32)
        bl = np.zeros(self.nb, np.int32)
        bsrc = np.zeros(self.nb, np.int64)
        opp = np.zeros(self.nb, np.int64)
        cptr = np.zeros(self.n + 1, np.int64)
        cidx = np.zeros(self.nblk, np.int32)
        lib().lo_get_topology(self.h, _l(bptr), _i(bp2), _i(bl), _l(bsrc), _l(opp), _l(cptr), _i(cidx))
        return dict(bptr=bptr, bp2=bp2, blayer=bl, bsrc=bsrc, opp=opp, cptr=cptr, cidx=cidx)

    def get(self, field):
        out = np.zeros(self.n * _PWIDTH[field])
        lib().lo_get_particle(self.h, field, _d(out))
        return out.reshape(self.n, -1) if _PWIDTH[field] > 1 else out

    def set(self, field, values):
        v = np.ascontiguousarray(values, dtype=np.float64).ravel()
        assert v.size == self.n * _PWIDTH[field]
        lib().lo_set_particle(self.h, field, _d(v))

    def get_bond(self, field):
        out = np.zeros(self.nb * _BWIDTH[field])
        lib().lo_get_bond(self.h, field, _d(out))
        return out.reshape(self.nb, -1) if _BWIDTH[field] > 1 else out

    def set_bond(self, field, values):
        v = np.ascontiguousarray(values, dtype=np.float64).ravel()
        assert v.size == self.nb * _BWIDTH[field]
        lib().lo_set_bond(self.h, field, _d(v))

    def set_mask(self, mask):
        m = np.ascontiguousarray(mask, dtype=np.int32).reshape(self.n, 3)
        lib().lo_set_mask(self.h, _i(m))

    def set_law(self, law, params):
        """params: one row for all particles, or an (N, P) array per particle."""
        p = np.ascontiguousarray(params, dtype=np.float64)
        per = p.ndim == 2
        lib().lo_set_law(self.h, int(law), _d(p), p.shape[-1], int(per))

    def set_types(self, types, undamaged):
        t = np.ascontiguousarray(types, dtype=np.int32)
        lib().lo_set_types(self.h, _i(t), int(undamaged))

    def set_nonlocal(self, ptr, idx, L):
        ptr = np.ascontiguousarray(ptr, dtype=np.int64)
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        L = np.ascontiguousarray(np.broadcast_to(np.asarray(L, dtype=np.float64), (self.n,)))
        lib().lo_set_nonlocal(self.h, _l(ptr), _i(idx), _d(L))

    def update_state(self):
        lib().lo_update_state(self.h)

    def static_damage(self):
        return bool(lib().lo_static_damage(self.h))

    def fatigue_damage(self, dNdt):
        return bool(lib().lo_fatigue_damage(self.h, float(dNdt)))

    def ddot(self):
        a = np.zeros(self.n)
        b = np.zeros(self.n)
        lib().lo_get_ddot(self.h, _d(a), _d(b))
        return a, b

    def state(self):
        ns = lib().lo_num_state(self.h)
        out = np.zeros(self.n * ns)
        lib().lo_get_particle(self.h, STATE, _d(out))
        return out.reshape(self.n, ns)

    def update(self):
        lib().lo_update_geometry_force(self.h)

    def residual(self):
        r = np.zeros(self.n * self.dim)
        nr = ctypes.c_double()
        nR = ctypes.c_double()
        lib().lo_residual(self.h, _d(r), ctypes.byref(nr), ctypes.byref(nR))
        return r, nr.value, nR.value

    def assemble(self, sym=0, bc=0):
        lib().lo_assemble(self.h, int(sym), int(bc))

    def K_bsr(self):
        v = np.zeros(self.nblk * self.dim * self.dim)
        lib().lo_get_K(self.h, _d(v))
        return v.reshape(self.nblk, self.dim, self.dim)

    def K_dense(self):
        t = self.topology()
        d = self.dim
        K = np.zeros((self.n * d, self.n * d))
        B = self.K_bsr()
        for i in range(self.n):
            for q in range(t["cptr"][i], t["cptr"][i + 1]):
                j = t["cidx"][q]
                K[d * i:d * i + d, d * j:d * j + d] = B[q]
        return K

    def cg(self, b, tol, maxit=-1):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b)
        it = ctypes.c_long()
        err = ctypes.c_double()
        st = lib().lo_cg(self.h, _d(b), _d(x), float(tol), int(maxit), ctypes.byref(it), ctypes.byref(err))
        return x, it.value, err.value, st

    def newton(self, max_iter, tol, cg_tol, cg_maxit=-1):
        return lib().lo_newton(self.h, int(max_iter), float(tol), float(cg_tol), int(cg_maxit))

    def log(self):
        n = lib().lo_log_size(self.h)
        out = np.zeros(3 * n)
        lib().lo_get_log(self.h, _d(out))
        return out.reshape(n, 3)

    def clear_log(self):
        lib().lo_clear_log(self.h)

    def load_step(self, apply, d, f=None, sym=1, bc_elim=1, max_iter=30, tol=1e-5, cg_tol=1e-10, cg_maxit=-1,
                  max_cuts=8):
        a = np.ascontiguousarray(apply, dtype=np.int32).reshape(self.n, 3)
        dd = np.ascontiguousarray(d, dtype=np.float64).reshape(self.n, 3)
        ff = np.zeros((self.n, 3)) if f is None else np.ascontiguousarray(f, dtype=np.float64).reshape(self.n, 3)
        return lib().lo_load_step(self.h, _i(a), _d(dd), _d(ff), int(sym), int(bc_elim), int(max_iter), float(tol),
                                  float(cg_tol), int(cg_maxit), int(max_cuts))

    def apply_disp_bc(self, apply, d):
        """Relative DispBC: x += d where apply is set; sets the mask there."""
        a = np.ascontiguousarray(apply, dtype=np.int32).reshape(self.n, 3)
        dd = np.ascontiguousarray(d, dtype=np.float64).reshape(self.n, 3)
        lib().lo_apply_disp_bc(self.h, _i(a), _d(dd))

    def add_pex(self, f):
        """Relative ForceBC: Pex += f."""
        ff = np.ascontiguousarray(f, dtype=np.float64).reshape(self.n, 3)
        lib().lo_add_pex(self.h, _d(ff))

    def store_state(self):
        lib().lo_store_state(self.h)

    def reset_state(self, reset_xyz=True):
        lib().lo_reset_state(self.h, int(bool(reset_xyz)))
