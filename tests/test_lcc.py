"""Learned coarse-correction network: the numpy oracle's backward pass against
finite differences (CPU), and the GPU forward pass, loss and parameter
gradients against the oracle (GPU).

Tolerances: the GPU stores activations and activation gradients in BF16 and
accumulates in FP32; the oracle rounds the same tensors to BF16 and
accumulates in FP64, so the remaining differences are accumulation order and
the BF16 roundings that it flips: relative L2 error <= 1e-2 for outputs and
the loss; per layer, gradients within 5e-3 (last layer), 1e-2 (the one before)
and 3e-2 (deeper layers, behind more BF16-rounded activation gradients).
"""
import numpy as np
import pytest

from oracle import lcc_oracle as O


def _inputs(n, D, H, W, seed):
    rs = np.random.default_rng(seed)
    x = rs.normal(size=(n, D, H, W, 8))
    # smooth along every axis so the convolutions see correlated data
    for ax in (1, 2, 3):
        x = (x + np.roll(x, 1, axis=ax) + np.roll(x, -1, axis=ax)) / 3.0
    t = x[..., 0] * 0.5 + 0.25 * np.roll(x[..., 1], 1, axis=2)
    return x.astype(np.float32), t.astype(np.float32)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_oracle_gradients_match_finite_differences():
    rs = np.random.default_rng(11)
    p = O.init_params(3).astype(np.float64)
    p += rs.normal(0, 0.01, p.size)          # nonzero biases
    x, t = _inputs(1, 8, 8, 8, 5)
    x, t = x.astype(np.float64), t.astype(np.float64)
    loss, g = O.loss_and_grads(p, x, t, bf16_acts=False)
    offs = np.cumsum([0] + [co * ci * 27 + co for ci, co in O.LAYERS])
    idx = [int(offs[l] + rs.integers(0, offs[l + 1] - offs[l])) for l in range(len(O.LAYERS)) for _ in range(2)]
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (O.loss_and_grads(pp, x, t, False)[0] - O.loss_and_grads(pm, x, t, False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * max(abs(fd), 1e-3 * np.abs(g).max()), (i, fd, g[i])


def test_oracle_param_count():
    # 27 ci co + co per layer over the fixed layer table: about 0.29M parameters
    assert O.num_params() == sum(co * ci * 27 + co for ci, co in O.LAYERS) == 294481


@pytest.mark.gpu
@pytest.mark.parametrize("path", ["mma_sync", "tcgen05"])
def test_gpu_forward_and_gradients_match_oracle(built_lib, path):
    from falcon_gb300 import lcc as L
    net = L.LCC(device=0, seed=1)
    net.set_tensor_path(L.TCGEN05 if path == "tcgen05" else L.MMA_SYNC)
    assert net.nparams == O.num_params()
    rs = np.random.default_rng(2)
    p = O.init_params(4)
    p = p + rs.normal(0, 0.01, p.size).astype(np.float32)
    net.set_params(p)
    assert np.array_equal(net.params(), p)
    x, t = _inputs(2, 8, 16, 16, 9)
    y = net.forward(x)
    yo = np.stack([O.forward(p.astype(np.float64), x[s])[0] for s in range(2)])
    assert _rel(y, yo) <= 1e-2, _rel(y, yo)
    loss, g = net.loss_grad(x, t)
    lo, go = O.loss_and_grads(p.astype(np.float64), x, t)
    assert abs(loss - lo) <= 1e-2 * lo, (loss, lo)
    offs = np.cumsum([0] + [co * ci * 27 + co for ci, co in O.LAYERS])
    errs = [_rel(g[offs[l]:offs[l + 1]], go[offs[l]:offs[l + 1]]) for l in range(len(O.LAYERS))]
    print("%s vs oracle: forward %.2e, loss %.2e, gradients per layer %s" % (
        path, _rel(y, yo), abs(loss - lo) / lo, " ".join("%.1e" % e for e in errs)))
    # the bound grows with the layers between the loss and the weights: each
    # one rounds another activation gradient to BF16 (measured on this case:
    # 1.4e-3 and 3.2e-3 for the last two layers, 2.2e-2 at most)
    bounds = [3e-2] * 8 + [1e-2, 5e-3]
    for l, e in enumerate(errs):
        assert e <= bounds[l], (l, e)


@pytest.mark.gpu
def test_gpu_training_reduces_loss(built_lib):
    from falcon_gb300.lcc import LCC
    net = LCC(device=0, seed=3)
    x, t = _inputs(16, 8, 16, 16, 21)
    losses = net.train(x, t, epochs=30, batch=4, lr=2e-3, seed=5)
    assert np.isfinite(losses).all()
    assert losses[-1] < 0.2 * losses[0], losses


@pytest.mark.gpu
def test_gpu_tcgen05_convolutions_match_mma_sync(built_lib):
    """The forward and backward-data convolutions on tcgen05 (accumulator in
    tensor memory) against the same network on mma.sync: same BF16 operands,
    FP32 sums in another order. A 3 x 8 x 8 x 24 batch: its 4,608 voxels are
    36 tiles of 128, and 24 is not a multiple of the 8-voxel core rows of one
    tile's face, so tiles straddle grid rows and samples."""
    from falcon_gb300 import lcc as L
    rs = np.random.default_rng(7)
    p = L.LCC(device=0, seed=2).params()
    p = p + rs.normal(0, 0.01, p.size).astype(np.float32)
    x, t = _inputs(3, 8, 8, 24, 13)
    out = {}
    for path in (L.MMA_SYNC, L.TCGEN05):
        net = L.LCC(device=0, seed=2)
        net.set_params(p)
        net.set_tensor_path(path)
        y = net.forward(x)
        loss, g = net.loss_grad(x, t)
        out[path] = (y, loss, g)
    (y0, l0, g0), (y1, l1, g1) = out[L.MMA_SYNC], out[L.TCGEN05]
    print("tcgen05 vs mma.sync: forward rel %.2e, loss rel %.2e" % (_rel(y1, y0), abs(l1 - l0) / l0))
    assert _rel(y1, y0) <= 2e-3
    assert abs(l1 - l0) <= 2e-3 * l0
    offs = np.cumsum([0] + [co * ci * 27 + co for ci, co in O.LAYERS])
    for l in range(len(O.LAYERS)):
        sl = slice(offs[l], offs[l + 1])
        assert _rel(g1[sl], g0[sl]) <= 2e-2, (l, _rel(g1[sl], g0[sl]))


@pytest.mark.gpu
def test_gpu_tcgen05_wait_that_runs_out_returns_timeout(built_lib):
    """With the poll limit at 0 the tcgen05 kernels' waits run out at once: the
    copies and MMAs in flight are drained, the tiles discarded, and forward,
    loss_grad and train return FALCON_ERR_TIMEOUT (no fault, no hang); with
    the default restored a fresh network gives the same results as before."""
    import falcon_gb300 as fg
    from falcon_gb300 import lcc as L
    x, t = _inputs(2, 8, 8, 24, 17)
    net = L.LCC(device=0, seed=4)
    y0 = net.forward(x)
    l0, g0 = net.loss_grad(x, t)
    net.set_wait_limit(0)
    for call in (lambda: net.forward(x), lambda: net.loss_grad(x, t),
                 lambda: net.train(x, t, epochs=1, batch=2, lr=1e-4, seed=1)):
        with pytest.raises(fg.FalconError) as e:
            call()
        assert e.value.code == fg.ERR_TIMEOUT, e.value
    net.set_wait_limit(-1)
    net.set_params(net.params())       # the failed train step may have moved the weights: reset Adam too
    assert np.isfinite(net.forward(x)).all()
    ref = L.LCC(device=0, seed=4)
    assert np.array_equal(ref.forward(x), y0)           # no atomics in the forward pass: the same bits
    l1, g1 = ref.loss_grad(x, t)                        # FP32 atomic sums in the weight gradients
    assert abs(l1 - l0) <= 1e-6 * l0 and _rel(g1, g0) <= 1e-5
