"""CPU oracle of the learned coarse-correction network (test infrastructure).

This module is the checker for the GPU network in falcon_gb300/csrc/lcc.cu:
tests compare the GPU forward pass, loss and parameter gradients with the ones
computed here. It is never called by the product path.

The reference has no learned component: the network is this project's
addition, a preconditioner stage inside the flexible CG that replaces the
coarsest-level smoothing of the V-cycle of ModLinearSolver_Multigrid_CG
(3_5/ModLinearSolver.f90:313-427), so the "reference" for this file is the
architecture fixed in the C ABI (include/falcon_gb300.h, falcon_lcc_*):

  input x [D][H][W][8] (channels last), zero padding at the grid edges
  L0 conv3 8->16 relu       L1 conv3 16->16 relu  -> s0     (grid G0)
  avgpool 2
  L2 conv3 16->32 relu      L3 conv3 32->32 relu  -> s1     (G0/2)
  avgpool 2
  L4 conv3 32->64 relu                            -> s2     (G0/4)
  avgpool 2
  L5 conv3 64->64 relu                                      (G0/8)
  up x2 + s2 -> L6 conv3 64->32 relu
  up x2 + s1 -> L7 conv3 32->16 relu
  up x2 + s0 -> L8 conv3 16->16 relu -> L9 conv3 16->1 (linear)

Parameters per layer: W[co][ci][27] (tap = (kd*3 + kh)*3 + kw, offsets -1..1)
and b[co], concatenated layer by layer. Activations are stored in BF16 on the
GPU; `bf16=True` rounds every stored activation and gradient the same way so
the comparison isolates accumulation-order differences.
"""
import numpy as np

LAYERS = [(8, 16), (16, 16), (16, 32), (32, 32), (32, 64), (64, 64), (64, 32), (32, 16), (16, 16), (16, 1)]
RELU = [True] * 9 + [False]


def num_params():
    return sum(co * ci * 27 + co for ci, co in LAYERS)


def split_params(p):
    out, o = [], 0
    for ci, co in LAYERS:
        w = p[o:o + co * ci * 27].reshape(co, ci, 27)
        o += co * ci * 27
        b = p[o:o + co]
        o += co
        out.append((w, b))
    return out


def bf16(x):
    """Round float32 values to bfloat16 (round to nearest even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    return np.where(np.isnan(a), a, out).reshape(a.shape)


def _taps():
    return [(kd, kh, kw) for kd in range(3) for kh in range(3) for kw in range(3)]


def conv(x, w, b):
    """x [D][H][W][ci], w [co][ci][27], b [co] -> [D][H][W][co] (float64)."""
    D, H, W, _ = x.shape
    xp = np.pad(x.astype(np.float64), ((1, 1), (1, 1), (1, 1), (0, 0)))
    y = np.zeros((D, H, W, w.shape[0]))
    for t, (kd, kh, kw) in enumerate(_taps()):
        y += xp[kd:kd + D, kh:kh + H, kw:kw + W, :] @ w[:, :, t].T.astype(np.float64)
    return y + b


def conv_backward(x, w, g):
    """gradients of conv for upstream gradient g [D][H][W][co]: dx, dw, db."""
    D, H, W, ci = x.shape
    xp = np.pad(x.astype(np.float64), ((1, 1), (1, 1), (1, 1), (0, 0)))
    dxp = np.zeros_like(xp)
    dw = np.zeros(w.shape)
    g = g.astype(np.float64)
    for t, (kd, kh, kw) in enumerate(_taps()):
        dxp[kd:kd + D, kh:kh + H, kw:kw + W, :] += g @ w[:, :, t].astype(np.float64)
        dw[:, :, t] = np.einsum("dhwo,dhwi->oi", g, xp[kd:kd + D, kh:kh + H, kw:kw + W, :])
    return dxp[1:-1, 1:-1, 1:-1, :], dw, g.sum(axis=(0, 1, 2))


def pool(x):
    D, H, W, C = x.shape
    return x.reshape(D // 2, 2, H // 2, 2, W // 2, 2, C).mean(axis=(1, 3, 5))


def pool_backward(g):
    return np.repeat(np.repeat(np.repeat(g, 2, 0), 2, 1), 2, 2) / 8.0


def up(x):
    return np.repeat(np.repeat(np.repeat(x, 2, 0), 2, 1), 2, 2)


def up_backward(g):
    D, H, W, C = g.shape
    return g.reshape(D // 2, 2, H // 2, 2, W // 2, 2, C).sum(axis=(1, 3, 5))


def forward(params, x, bf16_acts=True):
    """One sample: x [D][H][W][8] -> (y [D][H][W], cache)."""
    P = split_params(params)
    rnd = bf16 if bf16_acts else (lambda a: a)
    cache = {}

    def layer(l, inp):
        w, b = P[l]
        z = conv(inp, w, b)
        if RELU[l]:
            z = np.maximum(z, 0.0)
        cache[l] = (inp, z)
        return rnd(z) if l < 9 else z

    a = rnd(x)
    a = layer(0, a)
    s0 = layer(1, a)
    a = rnd(pool(s0))
    a = layer(2, a)
    s1 = layer(3, a)
    a = rnd(pool(s1))
    s2 = layer(4, a)
    a = rnd(pool(s2))
    a = layer(5, a)
    a = rnd(up(a) + s2)
    a = layer(6, a)
    a = rnd(up(a) + s1)
    a = layer(7, a)
    a = rnd(up(a) + s0)
    a = layer(8, a)
    y = layer(9, a)
    return y[..., 0], cache


def loss_and_grads(params, xs, ts, bf16_acts=True):
    """Mean-square loss over a batch (xs [n][D][H][W][8], ts [n][D][H][W]) and
    the gradient of every parameter, in the params layout."""
    P = split_params(params)
    rnd = bf16 if bf16_acts else (lambda a: a)
    n = xs.shape[0]
    nvox = n * np.prod(xs.shape[1:4])
    gw = [np.zeros(w.shape) for w, _ in P]
    gb = [np.zeros(b.shape) for _, b in P]
    loss = 0.0
    for s in range(n):
        y, c = forward(params, xs[s], bf16_acts)
        d = y - ts[s]
        loss += float((d ** 2).sum())
        g = (2.0 * d / nvox)[..., None]

        def back(l, g):
            inp, z = c[l]
            if RELU[l]:
                g = g * (z > 0)
            g = rnd(g)
            dx, dw, db = conv_backward(inp, P[l][0], g)
            gw[l] += dw
            gb[l] += db
            return dx

        g = back(9, g)
        g = back(8, g)
        gs0 = g                                   # through the skip add into s0
        g = up_backward(g)
        g = back(7, g)
        gs1 = g
        g = up_backward(g)
        g = back(6, g)
        gs2 = g
        g = up_backward(g)
        g = back(5, g)
        g = pool_backward(g) + gs2                # s2 feeds pool and the skip
        g = back(4, g)
        g = pool_backward(g) + gs1
        g = back(3, g)
        g = back(2, g)
        g = pool_backward(g) + gs0
        g = back(1, g)
        back(0, g)
    flat = []
    for l in range(len(LAYERS)):
        flat.append(gw[l].reshape(-1))
        flat.append(gb[l])
    return loss / nvox, np.concatenate(flat)


def init_params(seed):
    """He-normal weights, zero biases (the GPU initialiser draws its own
    numbers; tests set parameters explicitly)."""
    rs = np.random.default_rng(seed)
    out = []
    for ci, co in LAYERS:
        out.append(rs.normal(0, np.sqrt(2.0 / (ci * 27)), co * ci * 27))
        out.append(np.zeros(co))
    return np.concatenate(out).astype(np.float32)
