"""ctypes binding of the learned coarse-correction network (falcon_lcc_* in
include/falcon_gb300.h)."""
import ctypes as C

import numpy as np

from . import FalconError, OK, lib

CIN = 8
MMA_SYNC = 0      # warp-level mma.sync convolutions
TCGEN05 = 1       # 5th-generation tensor cores (tcgen05.mma, accumulator in tensor memory)


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class LCC:
    """The network on one GPU; parameters as one float32 vector."""

    def __init__(self, device=0, seed=7):
        self.L = lib()
        h = C.c_void_p()
        rc = self.L.falcon_lcc_create(C.byref(h), C.c_int32(device), C.c_uint64(seed))
        self.h = h
        if rc != OK:
            msg = self.last_error()
            self.L.falcon_lcc_destroy(h)
            self.h = None
            raise FalconError(rc, msg)
        n = C.c_int64()
        self._ck(self.L.falcon_lcc_num_params(self.h, C.byref(n)))
        self.nparams = n.value

    def close(self):
        if getattr(self, "h", None):
            self.L.falcon_lcc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def last_error(self):
        buf = C.create_string_buffer(512)
        self.L.falcon_lcc_last_error(self.h, buf, C.c_size_t(512))
        return buf.value.decode()

    def _ck(self, rc):
        if rc != OK:
            raise FalconError(rc, self.last_error())

    def set_tensor_path(self, path):
        """TCGEN05 or MMA_SYNC for the forward and backward-data convolutions."""
        self._ck(self.L.falcon_lcc_set_tensor_path(self.h, C.c_int32(path)))

    def set_wait_limit(self, polls):
        """Poll limit of the tcgen05 kernels' waits (< 0: the default)."""
        self._ck(self.L.falcon_lcc_set_wait_limit(self.h, C.c_int32(polls)))

    def params(self):
        p = np.zeros(self.nparams, dtype=np.float32)
        self._ck(self.L.falcon_lcc_get_params(self.h, _ptr(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.nparams
        self._ck(self.L.falcon_lcc_set_params(self.h, _ptr(p)))

    @staticmethod
    def _shape(x):
        n, D, H, W, c = x.shape
        assert c == CIN
        return n, D, H, W

    def forward(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        n, D, H, W = self._shape(x)
        y = np.zeros((n, D, H, W), dtype=np.float32)
        self._ck(self.L.falcon_lcc_forward(self.h, _ptr(x), C.c_int32(n), C.c_int32(D), C.c_int32(H), C.c_int32(W),
                                           _ptr(y)))
        return y

    def loss_grad(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        n, D, H, W = self._shape(x)
        g = np.zeros(self.nparams, dtype=np.float32)
        loss = C.c_double()
        self._ck(self.L.falcon_lcc_loss_grad(self.h, _ptr(x), _ptr(t), C.c_int32(n), C.c_int32(D), C.c_int32(H),
                                             C.c_int32(W), C.byref(loss), _ptr(g)))
        return loss.value, g

    def train(self, x, t, epochs=10, batch=8, lr=1e-3, seed=1):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        n, D, H, W = self._shape(x)
        losses = np.zeros(epochs, dtype=np.float32)
        self._ck(self.L.falcon_lcc_train(self.h, _ptr(x), _ptr(t), C.c_int32(n), C.c_int32(D), C.c_int32(H),
                                         C.c_int32(W), C.c_int32(epochs), C.c_int32(batch), C.c_float(lr),
                                         C.c_uint64(seed), _ptr(losses)))
        return losses


def _main(argv=None):
    """Command line: the network's forward and loss-and-gradient passes on a
    batch of seeded random panels, per tensor-core path, wall time per call.

    python -m falcon_gb300.lcc --batch 2 --shape 16 32 96 --path tcgen05 --reps 1
    """
    import argparse
    import json
    import time

    from . import build
    ap = argparse.ArgumentParser(prog="python -m falcon_gb300.lcc")
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--shape", type=int, nargs=3, default=(16, 32, 96), metavar=("D", "H", "W"))
    ap.add_argument("--path", choices=("tcgen05", "mma_sync", "both"), default="both")
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    build()
    rs = np.random.default_rng(1)
    x = rs.normal(size=(a.batch,) + tuple(a.shape) + (CIN,)).astype(np.float32)
    t = rs.normal(size=(a.batch,) + tuple(a.shape)).astype(np.float32)
    paths = {"tcgen05": TCGEN05, "mma_sync": MMA_SYNC}
    for name in (("tcgen05", "mma_sync") if a.path == "both" else (a.path,)):
        net = LCC(device=a.device, seed=3)
        net.set_tensor_path(paths[name])
        net.forward(x)
        net.loss_grad(x, t)
        t0 = time.perf_counter()
        for _ in range(a.reps):
            net.forward(x)
        t1 = time.perf_counter()
        for _ in range(a.reps):
            net.loss_grad(x, t)
        t2 = time.perf_counter()
        print(json.dumps({"path": name, "batch": a.batch, "shape": list(a.shape),
                          "forward_ms": (t1 - t0) / max(a.reps, 1) * 1e3,
                          "loss_grad_ms": (t2 - t1) / max(a.reps, 1) * 1e3}))
        net.close()
    return 0


if __name__ == "__main__":
    import sys
    sys.exit(_main())
