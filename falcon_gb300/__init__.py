"""falcon_gb300 -- GB300-native per-step hot path of the Falcon solar MHD code.

Python face of the C ABI in include/falcon_gb300.h (ctypes). It mirrors the
reference's step interface:

    Falcon.timestep()      ModTimeStep_Dynamo + MPI MIN  (3_6/ModTimeStep.f90:10-30)
    Falcon.advance_rk4()   ModAdvance_rk4                (3_6/ModAdvance.f90:18-112)
    Falcon.exchange()      ModCommunication_SendRecvGC_new(Tree,.false.)
                                                         (3_6/ModCommunication.f90:655-795)

There is no CPU fallback: every call goes to the CUDA library, and a missing or
unloadable library raises.
"""
import ctypes as C
import os

import numpy as np

from . import config
from .config import (Config, GhostEntry, PREC_FP64, PREC_MIXED, NVAR, VAR_NAMES,
                     make_config, shell_fp64_cpu, shell_mixed_21m, tiny)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libfalcon_gb300.so")

OK = 0
ERR_INVALID_ARG = -1
ERR_CUDA = -2
ERR_NAN_DETECTED = -3
ERR_TIMEOUT = -4
ERR_NOT_CONVERGED = -5
ERR_BOUNDS = -6
ERR_UNCOVERED_GHOST = -7
ERR_NO_DEVICE = -8
SHARD_SEND = 0
SHARD_RECV = 1
STEP_GRAPH = 0        # falcon_set_step_mode: one captured graph per step
STEP_PERSISTENT = 1   # one persistent cooperative launch per step

def host_array(shape, dtype=np.float64, align=4096):
    """An uninitialised host array whose first element sits on an `align`-byte
    boundary. The core transfers (Falcon.upload_state_core/download_state_core)
    move runs of whole rows that start 64-byte aligned when the array does; a
    run that starts inside a 64-byte line leaves partial lines at both of its
    ends, which the host link writes back at a lower rate (the core download of
    the 21M-cell shell: 188 GB/s aligned, 175 GB/s at the 16-mod-64 address that
    a large malloc returns)."""
    n = int(np.prod(shape))
    item = np.dtype(dtype).itemsize
    raw = np.empty(n * item + align, dtype=np.uint8)
    off = (-raw.ctypes.data) % align
    return raw[off:off + n * item].view(dtype).reshape(shape)


# every symbol declared in include/falcon_gb300.h
EXPORTS = (
    "falcon_create", "falcon_destroy", "falcon_last_error", "falcon_num_blocks", "falcon_block_ranges",
    "falcon_block_flags", "falcon_get_background", "falcon_ghost_count", "falcon_ghost_map",
    "falcon_upload_state", "falcon_download_state", "falcon_init_synthetic", "falcon_exchange",
    "falcon_timestep", "falcon_step_rk4", "falcon_run_steps", "falcon_synchronize",
    "falcon_set_kernel_timing", "falcon_kernel_stats", "falcon_reset_kernel_stats", "falcon_timer_start",
    "falcon_timer_stop", "falcon_device_bytes", "falcon_pin_host", "falcon_unpin_host",
    "falcon_step_phase", "falcon_download_stage_state", "falcon_ghost_list_sizes",
    "falcon_tuning",
    "falcon_solver_create", "falcon_solver_destroy", "falcon_solver_last_error", "falcon_solver_info",
    "falcon_solver_problem_blocks", "falcon_solver_rhs", "falcon_solver_operator", "falcon_solver_halo_count",
    "falcon_solver_halo_map", "falcon_solver_apply", "falcon_solver_solve", "falcon_solver_solution",
    "falcon_solver_timestep", "falcon_download_state_range", "falcon_exchange_stats",
    "falcon_solver_set_rhs", "falcon_solver_coarse_shape", "falcon_solver_attach_lcc", "falcon_solver_record",
    "falcon_solver_set_smoothing", "falcon_solver_problem_residuals",
    "falcon_lcc_create", "falcon_lcc_destroy", "falcon_lcc_last_error", "falcon_lcc_num_params",
    "falcon_lcc_get_params", "falcon_lcc_set_params", "falcon_lcc_forward", "falcon_lcc_loss_grad",
    "falcon_lcc_train", "falcon_save_allcells", "falcon_save_restart", "falcon_load_restart",
    "falcon_upload_state_core", "falcon_download_state_core", "falcon_set_wait_limit",
    "falcon_set_background", "falcon_solver_set_operator", "falcon_solver_set_magnetogram",
    "falcon_solver_magnetogram", "falcon_solver_set_guess", "falcon_solver_block_ranges",
    "falcon_solver_block_flags", "falcon_solver_magnetogram_sources", "falcon_solver_vcycle_op",
    "falcon_solver_tuning", "falcon_solver_set_tile", "falcon_shard_ranges", "falcon_shard_plan",
    "falcon_set_shard", "falcon_shard_counts", "falcon_shard_pack", "falcon_shard_unpack",
    "falcon_shard_min_ratio", "falcon_shard_set_min_ratio", "falcon_lcc_set_tensor_path", "falcon_set_tuning",
    "falcon_set_step_mode", "falcon_lcc_set_wait_limit",
)

# size of the static device array behind falcon_download_state_range
STATIC_SCRATCH_BYTES = 16 << 20

_lib = None


class FalconError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("falcon error %d: %s" % (code, msg))
        self.code = code


def build(force=False):
    from ._build import build as _b
    return _b(force=force)


def lib():
    """Load the CUDA library (raises if it is absent: there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FalconError(ERR_NO_DEVICE, "libfalcon_gb300.so is not built; run falcon_gb300.build()")
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        for n in EXPORTS:
            getattr(L, n).restype = C.c_int
        L.falcon_destroy.restype = None
        L.falcon_lcc_destroy.restype = None
        L.falcon_create.argtypes = [C.POINTER(vp), C.POINTER(Config)]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class Falcon:
    """One Yin-Yang shell on one GPU (device=-1: host-side setup only)."""

    def __init__(self, cfg):
        self.L = lib()
        self.cfg = cfg
        h = C.c_void_p()
        rc = self.L.falcon_create(C.byref(h), C.byref(cfg))
        self.h = h
        if rc != OK:
            msg = self.last_error()
            self.L.falcon_destroy(h)
            self.h = None
            raise FalconError(rc, msg)
        nb, ny = C.c_int32(), C.c_int32()
        self.L.falcon_num_blocks(self.h, C.byref(nb), C.byref(ny))
        self.nblocks, self.nblocks_yin = nb.value, ny.value
        t = cfg.tree
        self.shape = (self.nblocks, NVAR, t.nk + 2 * t.ng, t.nj + 2 * t.ng, t.ni + 2 * t.ng)
        self.interior_cells = self.nblocks * t.ni * t.nj * t.nk

    def close(self):
        if getattr(self, "h", None):
            self.L.falcon_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def last_error(self):
        buf = C.create_string_buffer(1024)
        self.L.falcon_last_error(self.h, buf, C.c_size_t(1024))
        return buf.value.decode()

    def _ck(self, rc):
        if rc != OK:
            raise FalconError(rc, self.last_error())

    # ---- host-side queries
    def block_ranges(self):
        out = np.zeros((self.nblocks, 3, 2))
        self._ck(self.L.falcon_block_ranges(self.h, _ptr(out)))
        return out

    def block_flags(self):
        out = np.zeros(self.nblocks, dtype=np.int32)
        self._ck(self.L.falcon_block_flags(self.h, _ptr(out)))
        return out

    def background(self):
        t = self.cfg.tree
        out = np.zeros((self.nblocks, config.NPROF, t.ni + 2 * t.ng))
        self._ck(self.L.falcon_get_background(self.h, _ptr(out)))
        return out

    def set_background(self, prof):
        """Replace the background with the driver's radial profiles, in the
        layout of background(): [block][NPROF][ni+2ng]."""
        prof = np.ascontiguousarray(prof, dtype=np.float64)
        t = self.cfg.tree
        if prof.shape != (self.nblocks, config.NPROF, t.ni + 2 * t.ng):
            raise ValueError("background shape %s" % (prof.shape,))
        self._ck(self.L.falcon_set_background(self.h, _ptr(prof)))

    def ghost_count(self):
        n = C.c_int64()
        self._ck(self.L.falcon_ghost_count(self.h, C.byref(n)))
        return n.value

    def ghost_map(self):
        n = self.ghost_count()
        arr = (GhostEntry * n)()
        self._ck(self.L.falcon_ghost_map(self.h, arr, C.c_int64(n)))
        dt = np.dtype([("tblock", "<i4"), ("ti", "<i4"), ("tj", "<i4"), ("tk", "<i4"),
                       ("sblock", "<i4"), ("pad_", "<i4"), ("src_x", "<f8", (3,))])
        return np.frombuffer((C.c_char * (n * dt.itemsize)).from_address(C.addressof(arr)),
                             dtype=dt, count=n).copy()

    # ---- state
    def upload_state(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        if u.shape != self.shape:
            raise ValueError("state shape %s != %s" % (u.shape, self.shape))
        self._ck(self.L.falcon_upload_state(self.h, _ptr(u)))

    def download_state(self):
        u = np.empty(self.shape)
        self._ck(self.L.falcon_download_state(self.h, _ptr(u)))
        return u

    def upload_state_raw(self, u):
        """Upload without shape/dtype conversion (u: C-contiguous float64 of self.shape)."""
        self._ck(self.L.falcon_upload_state(self.h, _ptr(u)))

    def download_state_into(self, u):
        self._ck(self.L.falcon_download_state(self.h, _ptr(u)))
        return u

    def upload_state_core(self, u):
        """Upload the core of u (interior planes x interior rows of every block
        and variable, radial ghost columns included); the theta/phi ghost layers
        are recomputed on the device. u: C-contiguous float64 of self.shape,
        pinned with pin_host for the in-place path (else a full upload runs)."""
        self._ck(self.L.falcon_upload_state_core(self.h, _ptr(u)))

    def download_state_core(self, u):
        """Write the core of the state into u; its other cells are left as they are."""
        self._ck(self.L.falcon_download_state_core(self.h, _ptr(u)))
        return u

    def pin_host(self, a):
        self._ck(self.L.falcon_pin_host(self.h, _ptr(a), C.c_size_t(a.nbytes)))

    def unpin_host(self, a):
        self._ck(self.L.falcon_unpin_host(self.h, _ptr(a)))

    def init_synthetic(self, kind=0, seed=1001, mach=0.01):
        self._ck(self.L.falcon_init_synthetic(self.h, C.c_int32(kind), C.c_uint64(seed), C.c_double(mach)))

    # ---- the hot path
    def exchange(self):
        self._ck(self.L.falcon_exchange(self.h))

    def timestep(self):
        dt = C.c_double()
        self._ck(self.L.falcon_timestep(self.h, C.byref(dt)))
        return dt.value

    def advance_rk4(self, want_dt=True):
        dt = C.c_double()
        self._ck(self.L.falcon_step_rk4(self.h, C.byref(dt) if want_dt else None))
        return dt.value if want_dt else None

    def run_steps(self, n):
        self._ck(self.L.falcon_run_steps(self.h, C.c_int32(n)))

    def step_phase(self, phase):
        self._ck(self.L.falcon_step_phase(self.h, C.c_int32(phase)))

    def download_stage_state(self):
        u = np.empty(self.shape)
        self._ck(self.L.falcon_download_stage_state(self.h, _ptr(u)))
        return u

    def synchronize(self):
        self._ck(self.L.falcon_synchronize(self.h))

    # ---- block sharding over ranks
    def shard_ranges(self, nranks):
        """first[r] .. first[r+1]-1: rank r's blocks (ModAllocation_Init's partition)."""
        out = np.zeros(nranks + 1, dtype=np.int32)
        self._ck(self.L.falcon_shard_ranges(self.h, C.c_int32(nranks), _ptr(out)))
        return out

    def shard_plan(self, nranks, rank, peer, direction):
        """Ghost-map indices of the entries rank sends to peer (SHARD_SEND) or
        receives from it (SHARD_RECV), in map order."""
        n = C.c_int64()
        self._ck(self.L.falcon_shard_plan(self.h, C.c_int32(nranks), C.c_int32(rank), C.c_int32(peer),
                                          C.c_int32(direction), None, C.c_int64(0), C.byref(n)))
        out = np.zeros(n.value, dtype=np.int64)
        self._ck(self.L.falcon_shard_plan(self.h, C.c_int32(nranks), C.c_int32(rank), C.c_int32(peer),
                                          C.c_int32(direction), _ptr(out), C.c_int64(n.value), C.byref(n)))
        return out

    def set_shard(self, nranks, rank):
        self._ck(self.L.falcon_set_shard(self.h, C.c_int32(nranks), C.c_int32(rank)))

    def shard_counts(self, peer):
        a, b = C.c_int64(), C.c_int64()
        self._ck(self.L.falcon_shard_counts(self.h, C.c_int32(peer), C.byref(a), C.byref(b)))
        return a.value, b.value

    def shard_pack(self, peer):
        n, _ = self.shard_counts(peer)
        buf = np.zeros((n, 8))
        self._ck(self.L.falcon_shard_pack(self.h, C.c_int32(peer), _ptr(buf)))
        return buf

    def shard_unpack(self, peer, buf):
        buf = np.ascontiguousarray(buf, dtype=np.float64)
        self._ck(self.L.falcon_shard_unpack(self.h, C.c_int32(peer), _ptr(buf)))

    def shard_min_ratio(self):
        m = C.c_double()
        self._ck(self.L.falcon_shard_min_ratio(self.h, C.byref(m)))
        return m.value

    def shard_set_min_ratio(self, m):
        self._ck(self.L.falcon_shard_set_min_ratio(self.h, C.c_double(m)))

    def set_wait_limit(self, polls):
        """Poll limit of the step kernels' bulk-copy waits (< 0: the default)."""
        self._ck(self.L.falcon_set_wait_limit(self.h, C.c_int32(polls)))

    # ---- output and restart
    def save_allcells(self, directory, step):
        """Write directory/AllCells_<step>/ (info.dat, Block_*.dat) in the
        reference's AllCells text format; returns that directory."""
        self._ck(self.L.falcon_save_allcells(self.h, os.fsencode(directory), C.c_int32(step)))
        return os.path.join(directory, "AllCells_" + str(int(step)).rjust(8).replace(" ", "0"))

    def save_restart(self, path):
        self._ck(self.L.falcon_save_restart(self.h, os.fsencode(path)))

    def load_restart(self, path):
        self._ck(self.L.falcon_load_restart(self.h, os.fsencode(path)))

    # ---- measurement
    def set_kernel_timing(self, on):
        self._ck(self.L.falcon_set_kernel_timing(self.h, C.c_int32(1 if on else 0)))

    def kernel_stats(self):
        names = C.create_string_buffer(1024)
        ms = (C.c_double * 32)()
        cnt = (C.c_int64 * 32)()
        n = C.c_int32()
        self._ck(self.L.falcon_kernel_stats(self.h, names, C.c_size_t(1024), ms, cnt, C.c_int32(32), C.byref(n)))
        nm = names.value.decode().split("\n")
        return {nm[k]: (ms[k], cnt[k]) for k in range(n.value)}

    def reset_kernel_stats(self):
        self._ck(self.L.falcon_reset_kernel_stats(self.h))

    def timer_start(self):
        self._ck(self.L.falcon_timer_start(self.h))

    def timer_stop(self):
        ms = C.c_double()
        self._ck(self.L.falcon_timer_stop(self.h, C.byref(ms)))
        return ms.value

    def set_step_mode(self, mode):
        """STEP_GRAPH (one captured graph per step) or STEP_PERSISTENT (one
        persistent cooperative launch per step; mixed path, 16^3 blocks)."""
        self._ck(self.L.falcon_set_step_mode(self.h, C.c_int32(mode)))

    def set_tuning(self, kpar_stage, kpar_diffusion):
        """Fix the k-chunk depths of the stage and diffusion kernels (no autotuning)."""
        self._ck(self.L.falcon_set_tuning(self.h, C.c_int32(kpar_stage), C.c_int32(kpar_diffusion)))

    def tuning(self):
        a, b = C.c_int32(), C.c_int32()
        self._ck(self.L.falcon_tuning(self.h, C.byref(a), C.byref(b)))
        return {"kpar_stage": a.value, "kpar_diffusion": b.value}

    def ghost_list_sizes(self):
        c = (C.c_int64 * 3)()
        self._ck(self.L.falcon_ghost_list_sizes(self.h, c))
        return {"copy": c[0], "linear": c[1], "trilinear": c[2]}

    def exchange_stats(self):
        c = np.zeros(5, dtype=np.int64)
        self._ck(self.L.falcon_exchange_stats(self.h, _ptr(c)))
        return {"stage_copy": int(c[0]), "stage_linear": int(c[1]), "stage_trilinear": int(c[2]),
                "pushed_faces": int(c[3]), "pushed_cells": int(c[4])}

    def device_bytes(self):
        b = C.c_int64()
        self._ck(self.L.falcon_device_bytes(self.h, C.byref(b)))
        return b.value
