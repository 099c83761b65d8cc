"""Python face of the implicit-solver C ABI (include/falcon_gb300.h).

    PFSS batch  : ModPFSS_setup + ModPFSS_solve (3_5/ModPFSS.f90:21-150)
    Conduction  : the implicit step ModHeatConduction leaves empty
                  (3_6/ModHeatConduction.f90), same operator format
    solve       : ModLinearSolver_Multigrid_CG (3_5/ModLinearSolver.f90:313-427)
                  as FP64 flexible CG with an FP32 V-cycle preconditioner
"""
import ctypes as C

import numpy as np

from . import lib as _lib, FalconError, OK

MAX_PROBLEMS = 256
PFSS = 0
CONDUCTION = 1
PRECOND_NONE = 0
PRECOND_MG = 1
PRECOND_MG_LCC = 2
VCYCLE_RESTRICT, VCYCLE_PROLONG_ADD, VCYCLE_SMOOTH_RED, VCYCLE_SMOOTH_BLACK, VCYCLE_RESIDUAL = range(5)


class SolverSpec(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("nproblems", C.c_int32), ("block", C.c_int32), ("nlevels", C.c_int32),
        ("device", C.c_int32), ("pad_", C.c_int32), ("seed", C.c_uint64),
        ("r_range_rsun", C.c_double * 2), ("dt_factor", C.c_double),
        ("nr", C.c_int32 * MAX_PROBLEMS), ("nt", C.c_int32 * MAX_PROBLEMS), ("np", C.c_int32 * MAX_PROBLEMS),
    ]


class SolveReport(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("converged", C.c_int32), ("vcycles", C.c_int32),
                ("refinements", C.c_int32), ("rel_residual", C.c_double), ("ms", C.c_double),
                ("fallbacks", C.c_int32), ("pad_", C.c_int32), ("floor_residual", C.c_double)]


_SYMS = ("falcon_solver_create", "falcon_solver_last_error", "falcon_solver_info", "falcon_solver_problem_blocks",
         "falcon_solver_rhs", "falcon_solver_operator", "falcon_solver_halo_count", "falcon_solver_halo_map",
         "falcon_solver_apply", "falcon_solver_solve", "falcon_solver_solution", "falcon_solver_timestep",
         "falcon_solver_set_rhs", "falcon_solver_coarse_shape", "falcon_solver_attach_lcc", "falcon_solver_record",
         "falcon_solver_set_smoothing", "falcon_solver_problem_residuals", "falcon_solver_set_operator",
         "falcon_solver_set_magnetogram", "falcon_solver_magnetogram", "falcon_solver_set_guess",
         "falcon_solver_block_ranges", "falcon_solver_block_flags", "falcon_solver_magnetogram_sources",
         "falcon_solver_vcycle_op", "falcon_solver_tuning", "falcon_solver_set_tile")


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def pfss_spec(sizes, seed=5000, block=8, nlevels=3, device=0, r_range=(1.0, 2.5)):
    """sizes: list of (nr, ntheta) per problem (nphi = 2 ntheta)."""
    s = SolverSpec()
    s.kind, s.nproblems, s.block, s.nlevels, s.device, s.seed = PFSS, len(sizes), block, nlevels, device, seed
    s.r_range_rsun[0], s.r_range_rsun[1] = r_range
    for q, (nr, nt) in enumerate(sizes):
        s.nr[q], s.nt[q] = nr, nt
    return s


def conduction_spec(nr=64, nt=128, np_=384, seed=3001, block=16, nlevels=3, device=0, dt_factor=50.0,
                    r_range=(0.7, 1.0)):
    s = SolverSpec()
    s.kind, s.nproblems, s.block, s.nlevels, s.device, s.seed = CONDUCTION, 1, block, nlevels, device, seed
    s.r_range_rsun[0], s.r_range_rsun[1] = r_range
    s.dt_factor = dt_factor
    s.nr[0], s.nt[0], s.np[0] = nr, nt, np_
    return s


def random_pfss_sizes(n=64, seed=5000):
    """nr ~ U{24..64}, ntheta ~ U{45..180} per problem."""
    rs = np.random.Generator(np.random.PCG64(seed))
    return [(int(rs.integers(24, 65)), int(rs.integers(45, 181))) for _ in range(n)]


class Solver:
    def __init__(self, spec):
        L = _lib()
        for n in _SYMS:
            getattr(L, n).restype = C.c_int
        L.falcon_solver_destroy.restype = None
        self.L = L
        self.spec = spec
        h = C.c_void_p()
        rc = L.falcon_solver_create(C.byref(h), C.byref(spec))
        self.h = h
        if rc != OK:
            msg = self.last_error()
            L.falcon_solver_destroy(h)
            self.h = None
            raise FalconError(rc, msg)
        info = (C.c_int32 * 6)()
        L.falcon_solver_info(self.h, info)
        self.nblocks, self.nproblems, self.nlevels = info[0], info[1], info[2]
        self.m = (info[3], info[4], info[5])
        self.nint = self.m[0] * self.m[1] * self.m[2]

    def close(self):
        if getattr(self, "h", None):
            self.L.falcon_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def last_error(self):
        buf = C.create_string_buffer(512)
        self.L.falcon_solver_last_error(self.h, buf, C.c_size_t(512))
        return buf.value.decode()

    def _ck(self, rc):
        if rc != OK:
            raise FalconError(rc, self.last_error())

    def problem_blocks(self):
        out = np.zeros(self.nproblems + 1, dtype=np.int32)
        self._ck(self.L.falcon_solver_problem_blocks(self.h, _ptr(out)))
        return out

    def rhs(self):
        out = np.zeros((self.nblocks, self.m[2], self.m[1], self.m[0]))
        self._ck(self.L.falcon_solver_rhs(self.h, _ptr(out)))
        return out

    def level_shape(self, level):
        return tuple(x >> level for x in self.m)

    def operator(self, level=0):
        mi, mj, mk = self.level_shape(level)
        nb = self.nblocks
        Aii = np.zeros((nb, mk, mj, mi)); Ai = np.zeros((nb, mk, mj, mi + 1))
        Aj = np.zeros((nb, mk, mj + 1, mi)); Ak = np.zeros((nb, mk + 1, mj, mi))
        self._ck(self.L.falcon_solver_operator(self.h, C.c_int32(level), _ptr(Aii), _ptr(Ai), _ptr(Aj), _ptr(Ak)))
        return Aii, Ai, Aj, Ak

    def halo_map(self, level=0):
        n = C.c_int64()
        self._ck(self.L.falcon_solver_halo_count(self.h, C.c_int32(level), C.byref(n)))
        idx = np.zeros((n.value, 8), dtype=np.int32)
        wx = np.zeros((n.value, 6))
        self._ck(self.L.falcon_solver_halo_map(self.h, C.c_int32(level), _ptr(idx), _ptr(wx)))
        return idx, wx

    def apply(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        self._ck(self.L.falcon_solver_apply(self.h, _ptr(x), _ptr(y)))
        return y

    def solve(self, tol=1e-8, max_iter=500, precond=PRECOND_MG, check=True):
        rep = SolveReport()
        rc = self.L.falcon_solver_solve(self.h, C.c_double(tol), C.c_int32(max_iter), C.c_int32(precond),
                                        C.byref(rep))
        if check:
            self._ck(rc)
        return {k: getattr(rep, k) for k, _ in SolveReport._fields_ if k != "pad_"}

    def set_smoothing(self, nu_pre=2, nu_post=2, nu_coarse=16):
        self._ck(self.L.falcon_solver_set_smoothing(self.h, C.c_int32(nu_pre), C.c_int32(nu_post),
                                                    C.c_int32(nu_coarse)))

    def problem_residuals(self):
        out = np.zeros(self.nproblems)
        self._ck(self.L.falcon_solver_problem_residuals(self.h, _ptr(out)))
        return out

    def set_rhs(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        assert b.size == self.nblocks * self.nint
        self._ck(self.L.falcon_solver_set_rhs(self.h, _ptr(b)))

    def set_operator(self, Aii, Ai, Aj, Ak):
        """The driver's level-0 face coefficients (the layout of operator(0))."""
        ref = self.operator(0)
        arrs = []
        for a, r in zip((Aii, Ai, Aj, Ak), ref):
            a = np.ascontiguousarray(a, dtype=np.float64)
            if a.shape != r.shape:
                raise ValueError("operator array shape %s != %s" % (a.shape, r.shape))
            arrs.append(a)
        self._ck(self.L.falcon_solver_set_operator(self.h, *(_ptr(a) for a in arrs)))

    def magnetogram(self):
        """PFSS: Br at the bottom faces, [block][k][j] (0 off the bottom blocks)."""
        out = np.zeros((self.nblocks, self.m[2], self.m[1]))
        self._ck(self.L.falcon_solver_magnetogram(self.h, _ptr(out)))
        return out

    def set_magnetogram(self, br):
        br = np.ascontiguousarray(br, dtype=np.float64)
        if br.shape != (self.nblocks, self.m[2], self.m[1]):
            raise ValueError("magnetogram shape %s" % (br.shape,))
        self._ck(self.L.falcon_solver_set_magnetogram(self.h, _ptr(br)))

    def vcycle_op(self, op, level, in0, in1=None):
        """One V-cycle kernel on host FP32 arrays (see falcon_solver_vcycle_op)."""
        shp = lambda l: (self.nblocks,) + self.level_shape(l)[::-1]
        a = np.ascontiguousarray(in0, dtype=np.float32)
        b = None if in1 is None else np.ascontiguousarray(in1, dtype=np.float32)
        out = np.zeros(shp(level + 1) if op == VCYCLE_RESTRICT else shp(level), dtype=np.float32)
        self._ck(self.L.falcon_solver_vcycle_op(self.h, C.c_int32(op), C.c_int32(level), _ptr(a),
                                                None if b is None else _ptr(b), _ptr(out)))
        return out

    def tuning(self):
        """The tile shape of the cell kernels: cells and threads per CTA, whether
        tuned (or set), and the tuner's time of one iteration with it."""
        t = (C.c_int32 * 3)()
        ms = C.c_double()
        self._ck(self.L.falcon_solver_tuning(self.h, t, C.byref(ms)))
        return {"cells_per_cta": t[0], "threads_per_cta": t[1], "tuned": bool(t[2]), "ms_per_iteration": ms.value}

    def set_tile(self, cells_per_cta, threads_per_cta):
        self._ck(self.L.falcon_solver_set_tile(self.h, C.c_int32(cells_per_cta), C.c_int32(threads_per_cta)))

    def block_ranges(self):
        out = np.zeros((self.nblocks, 3, 2))
        self._ck(self.L.falcon_solver_block_ranges(self.h, _ptr(out)))
        return out

    def block_flags(self):
        out = np.zeros(self.nblocks, dtype=np.int32)
        self._ck(self.L.falcon_solver_block_flags(self.h, _ptr(out)))
        return out

    def magnetogram_sources(self, problem):
        """[n][4] x, y, z (cm, Yin frame), q of problem's synthetic magnetogram."""
        n = C.c_int32()
        self._ck(self.L.falcon_solver_magnetogram_sources(self.h, C.c_int32(problem), None, C.c_int32(0), C.byref(n)))
        out = np.zeros((n.value, 4))
        self._ck(self.L.falcon_solver_magnetogram_sources(self.h, C.c_int32(problem), _ptr(out), C.c_int32(n.value),
                                                          C.byref(n)))
        return out

    def set_guess(self, x0):
        x0 = np.ascontiguousarray(x0, dtype=np.float64)
        assert x0.size == self.nblocks * self.nint
        self._ck(self.L.falcon_solver_set_guess(self.h, _ptr(x0)))

    def coarse_shape(self):
        s = (C.c_int32 * 4)()
        self._ck(self.L.falcon_solver_coarse_shape(self.h, s))
        return tuple(s)

    def attach_lcc(self, net, sweeps=2):
        self._ck(self.L.falcon_solver_attach_lcc(self.h, net.h, C.c_int32(sweeps)))
        self._net = net   # keep the network alive while attached

    def record(self, tol=1e-8, max_iter=100, max_records=16):
        n, D, H, W = self.coarse_shape()
        x = np.zeros((max_records * n, D, H, W, 8), dtype=np.float32)
        t = np.zeros((max_records * n, D, H, W), dtype=np.float32)
        nr = C.c_int32()
        self._ck(self.L.falcon_solver_record(self.h, C.c_double(tol), C.c_int32(max_iter), C.c_int32(max_records),
                                             _ptr(x), _ptr(t), C.byref(nr)))
        return x[:nr.value * n], t[:nr.value * n]

    def solution(self):
        out = np.zeros((self.nblocks, self.m[2], self.m[1], self.m[0]))
        self._ck(self.L.falcon_solver_solution(self.h, _ptr(out)))
        return out

    def timestep(self):
        d = C.c_double()
        self._ck(self.L.falcon_solver_timestep(self.h, C.byref(d)))
        return d.value


def _main(argv=None):
    """Command line: one heat-conduction or PFSS solve on a GPU, report printed.

    python -m falcon_gb300.solver conduction --size 64 128 384 --tol 1e-8
    python -m falcon_gb300.solver pfss --problems 4 --size 64 96 --tol 1e-10
    """
    import argparse
    import json
    ap = argparse.ArgumentParser(prog="python -m falcon_gb300.solver")
    ap.add_argument("kind", choices=["conduction", "pfss"])
    ap.add_argument("--size", type=int, nargs="+", default=None,
                    help="conduction: nr ntheta nphi per panel; pfss: nr ntheta")
    ap.add_argument("--problems", type=int, default=1)
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--max-iter", type=int, default=300)
    ap.add_argument("--precond", choices=["mg", "none"], default="mg")
    ap.add_argument("--solves", type=int, default=2, help="solves of the same system (the first warms up)")
    ap.add_argument("--smoothing", type=int, nargs=3, default=None, metavar=("PRE", "POST", "COARSE"),
                    help="red-black Gauss-Seidel sweeps before/after the coarse correction and on the coarsest level")
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    from . import build
    build()
    if a.kind == "conduction":
        nr, nt, np_ = a.size or (64, 128, 384)
        spec = conduction_spec(nr=nr, nt=nt, np_=np_, device=a.device)
    else:
        nr, nt = a.size or (64, 96)
        spec = pfss_spec([(nr, nt)] * a.problems, device=a.device)
    sv = Solver(spec)
    if a.smoothing:
        sv.set_smoothing(*a.smoothing)
    pc = PRECOND_MG if a.precond == "mg" else PRECOND_NONE
    for s in range(a.solves):
        rep = sv.solve(tol=a.tol, max_iter=a.max_iter, precond=pc, check=False)
        print(json.dumps({"solve": s, "cells": sv.nblocks * sv.nint, **rep}))
    sv.close()


if __name__ == "__main__":
    _main()
