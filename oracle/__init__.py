"""ctypes loader for the CPU oracle (oracle/falcon_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / --impl reference legs of bench.py, as the checker. The product
package never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

NVAR = 9   # variables of a block array (rho1 .. s1, psi), as FALCON_NVAR

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "liboracle.so")
# -O3 timing build of the same sources (the CPU baseline's clock), never used as the checker
FAST_LIB_PATH = os.path.join(HERE, "build", "liboracle_fast.so")
_lib = None
_fast = None


def build(force=False):
    """Compile both oracle builds with the Makefile (parity: -O2
    -ffp-contract=off; timing: -O3)."""
    srcs = [os.path.join(HERE, f) for f in ("falcon_oracle.cpp", "solver_oracle.cpp", "Makefile")]
    if force or any(not os.path.exists(p) or any(os.path.getmtime(p) < os.path.getmtime(f) for f in srcs)
                    for p in (LIB_PATH, FAST_LIB_PATH)):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib(timing=False):
    """The parity build, or with timing=True the -O3 timing build."""
    global _lib, _fast
    if timing:
        if _fast is None:
            build()
            _fast = _declare(C.CDLL(FAST_LIB_PATH))
        return _fast
    if _lib is None:
        build()
        _lib = _declare(C.CDLL(LIB_PATH))
    return _lib


def _declare(L):
    """Return types of the exported functions."""
    vp = C.c_void_p
    L.orc_create.restype = vp
    L.orc_create.argtypes = [vp]
    L.orc_destroy.argtypes = [vp]
    for name in ("orc_num_blocks", "orc_block_ranges", "orc_block_flags", "orc_get_background",
                 "orc_ghost_map", "orc_set_state", "orc_get_state", "orc_exchange",
                 "orc_timestep", "orc_step", "orc_block_rhs", "orc_block_diffusion",
                 "orc_block_grid", "orc_phase", "orc_get_stage_state", "orc_save_allcells",
                 "orc_set_background"):
        getattr(L, name).restype = C.c_int
    L.orc_ghost_count.restype = C.c_int64
    L.orc_ghost_count.argtypes = [vp]
    L.orc_uncovered_ghosts.restype = C.c_int64
    L.orc_uncovered_ghosts.argtypes = [vp]
    L.orc_num_threads.restype = C.c_int
    L.orc_dt.restype = C.c_double
    L.orc_dt.argtypes = [vp]
    L.orc_hc_halo.restype = C.c_int64
    for name in ("orc_pfss_operator", "orc_spmv", "orc_halo_fill", "orc_find_leaf", "orc_mg_restrict",
                 "orc_mg_prolong_add", "orc_mg_rbgs"):
        getattr(L, name).restype = C.c_int
    return L


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class Oracle:
    """The reference step restated on the CPU, one instance per grid."""

    def __init__(self, cfg, timing=False):
        self.L = lib(timing)
        self.cfg = cfg
        self.h = self.L.orc_create(C.byref(cfg))
        nb, ny = C.c_int32(), C.c_int32()
        self.L.orc_num_blocks(C.c_void_p(self.h), C.byref(nb), C.byref(ny))
        self.nblocks, self.nblocks_yin = nb.value, ny.value
        t = cfg.tree
        self.shape = (self.nblocks, NVAR, t.nk + 2 * t.ng, t.nj + 2 * t.ng, t.ni + 2 * t.ng)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(C.c_void_p(self.h))
            self.h = None

    @property
    def hp(self):
        return C.c_void_p(self.h)

    def block_ranges(self):
        out = np.zeros((self.nblocks, 3, 2))
        self.L.orc_block_ranges(self.hp, _ptr(out))
        return out

    def block_flags(self):
        out = np.zeros(self.nblocks, dtype=np.int32)
        self.L.orc_block_flags(self.hp, _ptr(out))
        return out

    def background(self):
        t = self.cfg.tree
        out = np.zeros((self.nblocks, 9, t.ni + 2 * t.ng))
        self.L.orc_get_background(self.hp, _ptr(out))
        return out

    def set_background(self, prof):
        """The driver's own radial profiles [b][9][ni+2ng] in place of the polytrope's."""
        prof = np.ascontiguousarray(prof, dtype=np.float64)
        assert prof.shape == self.background().shape
        self.L.orc_set_background(self.hp, _ptr(prof))

    def ghost_count(self):
        return int(self.L.orc_ghost_count(self.hp))

    # ---- a rank of a block-sharded run
    def set_owned(self, first, last):
        """Compute (phases, dt, exchange) only blocks [first, last)."""
        self.L.orc_set_owned(self.hp, C.c_int32(first), C.c_int32(last))

    def set_dt(self, dt):
        self.L.orc_set_dt(self.hp, C.c_double(dt))

    def dt(self):
        """The current step's dt (after phase 0 or a step)."""
        return float(self.L.orc_dt(self.hp))

    def interp_entries(self, rk, ent, x):
        """Values [n][9] of ghost entries ent[n][5] = (tblock, ti, tj, tk, sblock)
        with source-frame centres x[n][3], from the stage buffer (rk) or state."""
        ent = np.ascontiguousarray(ent, dtype=np.int32)
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros((len(ent), NVAR))
        self.L.orc_interp_entries(self.hp, C.c_int32(1 if rk else 0), _ptr(ent), _ptr(x), C.c_int64(len(ent)), _ptr(out))
        return out

    def write_ghosts(self, rk, ent, vals):
        ent = np.ascontiguousarray(ent, dtype=np.int32)
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        self.L.orc_write_ghosts(self.hp, C.c_int32(1 if rk else 0), _ptr(ent), C.c_int64(len(ent)), _ptr(vals))

    def uncovered_ghosts(self):
        return int(self.L.orc_uncovered_ghosts(self.hp))

    def ghost_map(self):
        from falcon_gb300.config import GhostEntry
        n = self.ghost_count()
        arr = (GhostEntry * n)()
        rc = self.L.orc_ghost_map(self.hp, arr, C.c_int64(n))
        assert rc == 0
        return ghost_entries_to_numpy(arr, n)

    def set_state(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        assert u.shape == self.shape
        self.L.orc_set_state(self.hp, _ptr(u))

    def get_state(self):
        u = np.zeros(self.shape)
        self.L.orc_get_state(self.hp, _ptr(u))
        return u

    def exchange(self):
        self.L.orc_exchange(self.hp)

    def timestep(self):
        dt = C.c_double()
        self.L.orc_timestep(self.hp, C.byref(dt))
        return dt.value

    def step(self):
        dt = C.c_double()
        self.L.orc_step(self.hp, C.byref(dt))
        return dt.value

    def phase(self, ph):
        self.L.orc_phase(self.hp, C.c_int32(ph))
        return self.L.orc_dt(self.hp)

    def save_allcells(self, directory, step):
        """ModSave_AllCells of the oracle's state: directory/AllCells_<step>/."""
        rc = self.L.orc_save_allcells(C.c_void_p(self.h), os.fsencode(directory), C.c_int32(step))
        if rc != 0:
            raise OSError("oracle could not write AllCells files under %s" % directory)
        return os.path.join(directory, "AllCells_" + str(int(step)).rjust(8).replace(" ", "0"))

    def get_stage_state(self):
        u = np.zeros(self.shape)
        self.L.orc_get_stage_state(self.hp, _ptr(u))
        return u

    def block_rhs(self, b, p):
        t = self.cfg.tree
        p = np.ascontiguousarray(p, dtype=np.float64)
        R = np.zeros((NVAR, t.nk, t.nj, t.ni))
        self.L.orc_block_rhs(self.hp, C.c_int32(b), _ptr(p), _ptr(R))
        return R

    def block_diffusion(self, b, p):
        t = self.cfg.tree
        p = np.ascontiguousarray(p, dtype=np.float64)
        R = np.zeros((NVAR, t.nk, t.nj, t.ni))
        self.L.orc_block_diffusion(self.hp, C.c_int32(b), _ptr(p), _ptr(R))
        return R

    def block_grid(self, b):
        t = self.cfg.tree
        xi = np.zeros(t.ni + 2 * t.ng)
        xj = np.zeros(t.nj + 2 * t.ng)
        xk = np.zeros(t.nk + 2 * t.ng)
        d = np.zeros(3)
        self.L.orc_block_grid(self.hp, C.c_int32(b), _ptr(xi), _ptr(xj), _ptr(xk), _ptr(d))
        return xi, xj, xk, d


def pfss_operator(o, m):
    """Level-1 PFSS operator of the oracle's tree (3_5/ModPFSS.f90:57-86)."""
    nb = o.nblocks
    Aii = np.zeros((nb, m, m, m)); Ai = np.zeros((nb, m, m, m + 1))
    Aj = np.zeros((nb, m, m + 1, m)); Ak = np.zeros((nb, m + 1, m, m))
    lib().orc_pfss_operator(o.hp, C.c_int32(m), _ptr(Aii), _ptr(Ai), _ptr(Aj), _ptr(Ak))
    return Aii, Ai, Aj, Ak


def hc_halo(o, m):
    """1-layer halo map in the reference's order: idx[n][8], wx[n][6], clamped[n]."""
    L = lib()
    n = L.orc_hc_halo(o.hp, C.c_int32(m), None, None, None, C.c_int64(1 << 40))
    idx = np.zeros((n, 8), dtype=np.int32)
    wx = np.zeros((n, 6))
    cl = np.zeros(n, dtype=np.int32)
    L.orc_hc_halo(o.hp, C.c_int32(m), _ptr(idx), _ptr(wx), _ptr(cl), C.c_int64(n))
    return idx, wx, cl


def spmv(m, A, xp):
    """y = A x (3_5/ModLinearSolver.f90:43-50) on a padded vector."""
    Aii, Ai, Aj, Ak = [np.ascontiguousarray(a, dtype=np.float64) for a in A]
    nb = Aii.shape[0]
    xp = np.ascontiguousarray(xp, dtype=np.float64)
    y = np.zeros_like(Aii)
    lib().orc_spmv(C.c_int32(nb), C.c_int32(m), _ptr(Aii), _ptr(Ai), _ptr(Aj), _ptr(Ak), _ptr(xp), _ptr(y))
    return y


def halo_fill(m, idx, wx, xp):
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    wx = np.ascontiguousarray(wx, dtype=np.float64)
    lib().orc_halo_fill(C.c_int32(m), _ptr(idx), _ptr(wx), C.c_int64(len(idx)), _ptr(xp))
    return xp


def mg_restrict(res):
    """Coarse right-hand side from a fine residual res[b][m][m][m] (FP32):
    the 8 children summed in ModMath_rebin_3D_factor2's order, no /8."""
    res = np.ascontiguousarray(res, dtype=np.float32)
    nb, m = res.shape[0], res.shape[1]
    out = np.zeros((nb, m // 2, m // 2, m // 2), dtype=np.float32)
    lib().orc_mg_restrict(C.c_int32(nb), C.c_int32(m), _ptr(res), _ptr(out))
    return out


def mg_prolong_add(zc, zf):
    """zf + injection of zc (FP32, interior arrays)."""
    zc = np.ascontiguousarray(zc, dtype=np.float32)
    out = np.array(zf, dtype=np.float32, copy=True)
    lib().orc_mg_prolong_add(C.c_int32(out.shape[0]), C.c_int32(out.shape[1]), _ptr(zc), _ptr(out))
    return out


def mg_rbgs(A, r, zp, colour):
    """One red-black half sweep (FP32) on the padded zp (halo filled)."""
    A32 = [np.ascontiguousarray(a, dtype=np.float32) for a in A]
    r = np.ascontiguousarray(r, dtype=np.float32)
    out = np.array(zp, dtype=np.float32, copy=True)
    nb, m = r.shape[0], r.shape[1]
    lib().orc_mg_rbgs(C.c_int32(nb), C.c_int32(m), *(_ptr(a) for a in A32), _ptr(r), _ptr(out), C.c_int32(colour))
    return out


def mg_solve(ops, halos, bprob, nproblems, b, x0, tol, max_iter, smoothing):
    """CPU FP64 MG-preconditioned flexible CG of a batch (see orc_mg_solve).
    ops[l] = (Aii, Ai, Aj, Ak), halos[l] = (idx, wx); returns (x, iterations,
    per-problem FP64 relative residuals)."""
    nl = len(ops)
    keep = []
    op_ptrs = (C.c_void_p * (4 * nl))()
    hi = (C.c_void_p * nl)()
    hw = (C.c_void_p * nl)()
    nh = (C.c_int64 * nl)()
    for l in range(nl):
        for a, arr in enumerate(ops[l]):
            arr = np.ascontiguousarray(arr, dtype=np.float64)
            keep.append(arr)
            op_ptrs[4 * l + a] = arr.ctypes.data
        idx = np.ascontiguousarray(halos[l][0], dtype=np.int32)
        wx = np.ascontiguousarray(halos[l][1], dtype=np.float64)
        keep += [idx, wx]
        hi[l], hw[l], nh[l] = idx.ctypes.data, wx.ctypes.data, len(idx)
    bprob = np.ascontiguousarray(bprob, dtype=np.int32)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.array(x0, dtype=np.float64, copy=True)
    rel = np.zeros(nproblems)
    m0 = ops[0][0].shape[1]
    L = lib()
    L.orc_mg_solve.restype = C.c_int
    it = L.orc_mg_solve(C.c_int32(b.shape[0]), C.c_int32(nproblems), _ptr(bprob), C.c_int32(nl), C.c_int32(m0),
                        op_ptrs, hi, hw, nh, C.c_int32(smoothing[0]), C.c_int32(smoothing[1]),
                        C.c_int32(smoothing[2]), _ptr(b), _ptr(x), C.c_double(tol), C.c_int32(max_iter), _ptr(rel))
    return x, it, rel


def ghost_entries_to_numpy(arr, n):
    """Structured array view of a ctypes GhostEntry array."""
    dt = np.dtype([("tblock", "<i4"), ("ti", "<i4"), ("tj", "<i4"), ("tk", "<i4"),
                   ("sblock", "<i4"), ("pad_", "<i4"), ("src_x", "<f8", (3,))])
    buf = np.frombuffer((C.c_char * (n * dt.itemsize)).from_address(C.addressof(arr)), dtype=dt, count=n)
    return buf.copy()


def coord_conv(rtp):
    out = np.zeros(3)
    rtp = np.ascontiguousarray(rtp, dtype=np.float64)
    lib().orc_coord_conv(_ptr(rtp), _ptr(out))
    return out


def vec_conv(rtp, v):
    out = np.zeros(3)
    rtp = np.ascontiguousarray(rtp, dtype=np.float64)
    v = np.ascontiguousarray(v, dtype=np.float64)
    lib().orc_vec_conv(_ptr(rtp), _ptr(v), _ptr(out))
    return out


def set_threads(n, timing=False):
    lib(timing).orc_set_threads(C.c_int(n))


def num_threads(timing=False):
    return int(lib(timing).orc_num_threads())
