"""Known-answer tests of the CPU oracle (oracle/falcon_oracle.cpp).

The reference's own tests pin none of the ghost fill, the Yin-Yang transforms,
the spherical operators or the RK step numerically, so the oracle is pinned
here by analytic properties: involutions of the Yin-Yang maps, exactness of the
fourth-order derivative on cubics (up to the FP32 constant 1./12.), a
divergence-free radial flux, trilinear interpolation of linear fields, the
background replication check of 3_6/test_ModBlock.f90:77-104, and the FP32
constants of the reference (ModConst, root ranges).
"""
import numpy as np
import pytest

import oracle
from falcon_gb300 import config, synth

C12 = float(np.float32(1.0) / np.float32(12.0))


@pytest.fixture(scope="module")
def tiny_oracle():
    return oracle.Oracle(config.tiny())


def test_fp32_constants_of_the_reference(tiny_oracle):
    # 3_6/ModConst.f90:2,5 and 3_6/ModYinYangTree.f90:104-105 (FP32 products)
    assert C12 == 0.0833333358168602
    rng = tiny_oracle.block_ranges()
    nb_yin = tiny_oracle.nblocks_yin
    th = np.unique(rng[:nb_yin, 1, :])
    ph = np.unique(rng[:nb_yin, 2, :])
    assert th.min() == 0.7853981852531433 and th.max() == 2.356194496154785
    assert ph.min() == -2.356194496154785 and ph.max() == 2.356194496154785
    assert rng[:, 0, :].min() == 0.7 * 69549998080.0


def test_coord_conv_is_an_involution():
    rs = np.random.default_rng(7)
    for _ in range(200):
        x = np.array([7e10, rs.uniform(0.8, 2.3), rs.uniform(-2.3, 2.3)])
        y = oracle.coord_conv(oracle.coord_conv(x))
        assert np.allclose(y, x, rtol=0, atol=1e-13)


def test_vec_conv_preserves_length_and_inverts():
    rs = np.random.default_rng(8)
    for _ in range(200):
        x = np.array([7e10, rs.uniform(0.8, 2.3), rs.uniform(-2.3, 2.3)])
        v = rs.normal(size=3)
        w = oracle.vec_conv(x, v)
        assert abs(np.linalg.norm(w) - np.linalg.norm(v)) < 1e-13 * np.linalg.norm(v)
        back = oracle.vec_conv(oracle.coord_conv(x), w)
        assert np.allclose(back, v, atol=1e-13)


def _interior_block(o):
    fl = o.block_flags()
    return int(np.nonzero((fl & 6) == 0)[0][0]) if ((fl & 6) == 0).any() else 0


def test_o4_derivative_exact_on_cubics():
    """R_s1 = -vr * D_r(s1) with vr constant; D_r of a cubic is exact up to 12*f32(1/12)."""
    cfg = config.tiny()
    o = oracle.Oracle(cfg)
    b = _interior_block(o)
    xi, xj, xk, d = o.block_grid(b)
    t = cfg.tree
    p = np.zeros(o.shape[1:])
    V0 = 3.0e3
    rc = xi.mean()
    x = (xi - rc) / d[0]
    f = 1.0 + 0.3 * x - 0.2 * x ** 2 + 0.05 * x ** 3
    fp = (0.3 - 0.4 * x + 0.15 * x ** 2) / d[0]
    p[7] = f[None, None, :]
    p[1] = V0
    R = o.block_rhs(b, p)
    expect = -V0 * fp[2:2 + t.ni] * (12.0 * C12)
    got = R[7]
    assert np.allclose(got, expect[None, None, :], rtol=2e-9, atol=0)


def test_radial_flux_with_constant_r2_rho0_vr_is_divergence_free():
    cfg = config.tiny()
    o = oracle.Oracle(cfg)
    b = _interior_block(o)
    xi, xj, xk, d = o.block_grid(b)
    rho0 = o.background()[b, 1]
    p = np.zeros(o.shape[1:])
    Cst = 1.0e25
    p[1] = (Cst / (rho0 * xi * xi))[None, None, :]
    R = o.block_rhs(b, p)
    scale = (Cst / xi.mean() ** 2) / d[0]
    assert np.abs(R[0]).max() < 1e-11 * scale


def test_background_replication_matches_the_polytrope():
    """Analogue of 3_6/test_ModBlock.f90:77-104: the block's 1D profiles equal
    get_vars at the cell centres (1e-12)."""
    cfg = config.tiny()
    o = oracle.Oracle(cfg)
    bg = o.background()
    t = cfg.tree
    r_lo, r_hi = [v * synth.R_SUN for v in t.r_range_rsun]
    pc = synth.polytrope_constants(r_lo, r_hi)
    n = cfg.bg.poly_n
    for b in (0, o.nblocks - 1):
        xi = o.block_grid(b)[0]
        zeta = 1.0 + pc["K"] * (1.0 / xi - 1.0 / r_lo)
        assert np.allclose(bg[b, 1], pc["rho_b"] * zeta ** n, rtol=1e-12)
        assert np.allclose(bg[b, 2], pc["p_b"] * zeta ** (n + 1), rtol=1e-12)
        assert np.allclose(bg[b, 0], pc["g_b"] * (r_lo / xi) ** 2, rtol=1e-12)


def test_trilinear_ghosts_exact_on_linear_fields():
    """Same-panel ghost cells that are not clamped reproduce a field linear in
    (r, theta, phi) (3_6/ModMath.f90:250-293)."""
    cfg = config.tiny()
    o = oracle.Oracle(cfg)
    t = cfg.tree
    u = np.zeros(o.shape)
    grids = [o.block_grid(b) for b in range(o.nblocks)]
    A, Bc, Cc, Dc = 1.0, 2.0e-10, 0.7, -0.3
    for b, (xi, xj, xk, _) in enumerate(grids):
        P, T, R = np.meshgrid(xk, xj, xi, indexing="ij")
        u[b, 0] = A + Bc * R + Cc * T + Dc * P
    o.set_state(u)
    o.exchange()
    v = o.get_state()
    m = o.ghost_map()
    fl = o.block_flags()
    checked = 0
    for e in m[:: max(1, len(m) // 4000)]:
        tb, sb = e["tblock"], e["sblock"]
        if (fl[tb] & 1) != (fl[sb] & 1):
            continue
        xi, xj, xk, _ = grids[sb]
        pos = [-1.0 + (e["src_x"][0] - xi[0]) / (xi[3] - xi[2]),
               -1.0 + (e["src_x"][1] - xj[0]) / (xj[3] - xj[2]),
               -1.0 + (e["src_x"][2] - xk[0]) / (xk[3] - xk[2])]
        nn = (t.ni, t.nj, t.nk)
        if any(p < 1.0 or p > n for p, n in zip(pos, nn)):
            continue
        x = e["src_x"]
        want = A + Bc * x[0] + Cc * x[1] + Dc * x[2]
        got = v[tb, 0, e["tk"] + 1, e["tj"] + 1, e["ti"] + 1]
        assert abs(got - want) <= 1e-12 * abs(want), (e, got, want)
        checked += 1
    assert checked > 100


def test_step_is_deterministic_and_finite():
    cfg = config.tiny()
    o1, o2 = oracle.Oracle(cfg), oracle.Oracle(cfg)
    u0 = synth.initial_state(cfg, o1.block_ranges(), o1.block_flags())
    for o in (o1, o2):
        o.set_state(u0)
        o.exchange()
        o.exchange()
    oracle.set_threads(1)
    dt1 = o1.step()
    oracle.set_threads(0 if False else oracle.num_threads())
    dt2 = o2.step()
    assert dt1 == dt2 and dt1 > 0
    a, b = o1.get_state(), o2.get_state()
    assert np.isfinite(a).all()
    assert np.array_equal(a, b)


def test_glm_stage_is_linear_damping_of_psi():
    """GLM (3_6/ModDivB.f90:13-38) with v = B = 0: the first RK stage gives
    psi_rk = psi (1 - dt v_wave / (4 h_LLL)) cell by cell (0 < factor < 1),
    B_rk = -dt grad(psi) / 4, and the whole stage is linear in psi: doubling
    psi doubles psi_rk and B_rk bit for bit. With divb_option = 0 psi and B
    stay 0."""
    def run(divb, scale):
        cfg = config.tiny(divb_option=divb)
        o = oracle.Oracle(cfg)
        u = synth.initial_state(cfg, o.block_ranges(), o.block_flags(), seed=7, psi_amp=1e-3)
        u[:, 1:7] = 0.0          # v = B = 0
        psi = u[:, 8]
        psi[np.abs(psi) < 1e-30 * np.abs(psi).max()] = 0.0   # no underflow in the tails
        u[:, 8] = psi * scale
        o.set_state(u)
        o.exchange()
        o.phase(0)
        o.phase(1)
        return u, o.get_stage_state()
    u1, r1 = run(1, 1.0)
    u2, r2 = run(1, 2.0)
    inner = (slice(None), slice(None), slice(2, -2), slice(2, -2), slice(2, -2))
    p0, p1 = u1[inner][:, 8], r1[inner][:, 8]
    assert np.abs(p0).max() > 0
    f = p1[p0 != 0] / p0[p0 != 0]
    assert (f > 0).all() and (f < 1).all()
    assert np.abs(r1[inner][:, 4:7]).max() > 0
    assert np.array_equal(2 * r1[:, 4:7], r2[:, 4:7])
    assert np.array_equal(2 * r1[:, 8], r2[:, 8])
    _, r0 = run(0, 1.0)
    assert not np.abs(r0[inner][:, 4:7]).any()


def test_powell_source_term_against_numpy():
    """divb_option 2 adds -(div B) v to the induction equation
    (3_5/ModEquation.f90:169-176) and nothing else: the oracle's block RHS with
    and without it differ by that term, restated here in numpy with the
    spherical divergence of 3_6/ModSpherical.f90:104-159 (FP32 1/12 stencil)."""
    o0 = oracle.Oracle(config.tiny())
    o2 = oracle.Oracle(config.tiny(divb_option=2))
    cfg = config.tiny()
    u = synth.initial_state(cfg, o0.block_ranges(), o0.block_flags(), seed=11)
    rs = np.random.default_rng(3)
    b = 7
    p = u[b].copy()
    bscale = np.abs(p[4:7]).max()
    vscale = 1e-3 * bscale
    p[4:7] += 0.1 * bscale * rs.standard_normal(p[4:7].shape)   # a field with divergence
    p[1:4] = vscale * rs.standard_normal(p[1:4].shape)
    R0, R2 = o0.block_rhs(b, p), o2.block_rhs(b, p)
    others = [0, 1, 2, 3, 7, 8]
    assert np.array_equal(R0[others], R2[others])
    xi, xj, xk, d = o2.block_grid(b)
    c = float(np.float32(1.0) / np.float32(12.0))
    I = slice(2, -2)

    def D(f, axis, dx):
        n = f.shape[axis]
        s = lambda o: np.take(f, np.arange(2 + o, n - 2 + o), axis=axis)
        return (c / dx) * (((-s(2) + 8.0 * s(1)) - 8.0 * s(-1)) + s(-2))

    r = xi[None, None, :]
    st = np.sin(xj)[None, :, None]
    br, bt, bp = p[4], p[5], p[6]
    d1 = D(br * r * r, 2, d[0])[I, I, :] / (xi[2:-2] ** 2)[None, None, :]
    d2 = D(bt * st, 1, d[1])[I, :, I]
    d3 = D(bp, 0, d[2])[:, I, I]
    divb = d1 + ((d2 + d3) / np.sin(xj[2:-2])[None, :, None]) / xi[2:-2][None, None, :]
    v = p[1:4][:, I, I, I]
    want = -divb[None] * v
    got = R2[4:7] - R0[4:7]
    assert np.abs(want).max() > 0
    assert np.abs(got - want).max() <= 1e-9 * np.abs(want).max()
