"""Seeded synthetic inputs (host side, numpy).

Initial state for the shell workloads: a Gaussian entropy bump plus an
axisymmetric dipole B, v = 0. Values are filled in every cell including ghost
cells, in the Fortran block layout, like ModInitiation does
(3_6/ModInitiation.f90:143-188: Yang blocks receive the Yin-frame field rotated
with ModYinYang_VecConv_0D). The random-phase velocity field of the 21M-cell
workload is generated on the device (falcon_init_synthetic) instead: summing 512
modes over 21M cells is GPU work.

Seeds: std::mt19937_64-compatible draws are not needed here; numpy's PCG64 with
the workload seed fixes the bump centre and width.
"""
import numpy as np

R_SUN = float(np.float32(6.955e10))
K_B = float(np.float32(1.380649e-16))
M_P = float(np.float32(1.67262192369e-24))
GAMMA = float(np.float32(5.0) / np.float32(3.0))


def coord_conv(r, t, p):
    """ModYinYang_CoordConv (3_6/ModYinYang.f90:8-17), vectorised."""
    st, sp, cp, ct = np.sin(t), np.sin(p), np.cos(p), np.cos(t)
    t2 = np.arccos(st * sp)
    a = np.arccos(-(st * cp) / np.sqrt(st * st * (cp * cp) + ct * ct))
    p2 = np.copysign(np.abs(a), ct)
    return r, t2, p2


def vec_conv(r, t, p, v1, v2, v3):
    """ModYinYang_VecConv (3_6/ModYinYang.f90:34-46), vectorised."""
    _, t2, p2 = coord_conv(r, t, p)
    s1, s2, c1, s3 = np.sin(p), np.sin(p2), np.cos(p), np.sin(t2)
    o2 = -(s1 * s2 * v2) - c1 / s3 * v3
    o3 = -(s1 * s2 * v3) + c1 / s3 * v2
    return v1, o2, o3


def cell_centres(rng, n, ng):
    """ModBlock_InitGrid cell centres (3_6/ModBlock.f90:310-312), padded."""
    i = np.arange(1 - ng, n + ng + 1)
    a = (n - i).astype(np.float32) + np.float32(0.5)
    b = i.astype(np.float32) - np.float32(0.5)
    return (rng[0] * a.astype(np.float64) + rng[1] * b.astype(np.float64)) / n


def polytrope_constants(r_lo, r_hi, poly_n=1.5, contrast=100.0, mu=0.6):
    zeta_t = contrast ** (-1.0 / poly_n)
    K = (1.0 - zeta_t) / (1.0 / r_lo - 1.0 / r_hi)
    rho_b = 10.0 ** (-0.6841807359334023)
    g_b = 54340.03688603464
    p_b = rho_b * g_b * r_lo * r_lo / ((poly_n + 1.0) * K)
    R_gas = K_B / (mu * M_P)
    return dict(rho_b=rho_b, p_b=p_b, R_gas=R_gas, K=K, g_b=g_b,
                c_b=np.sqrt(GAMMA * p_b / rho_b))


def initial_state(cfg, ranges, flags, seed=1001, amp=1e-4, b_frac=1e-3, psi_amp=0.0, b_div_amp=0.0):
    """State array (nblocks, 9, nkp, njp, nip) float64 for the shell workloads.

    psi (index 8) is 0 unless psi_amp > 0, which puts a Gaussian of peak
    psi_amp * B0 * c_b (B0 the base field, c_b the base sound speed) at the
    entropy blob's centre, for runs with GLM cleaning. b_div_amp > 0 adds a
    Gaussian of peak b_div_amp * B0 there to B_r alone, a field with
    divergence (B_r is the same in both panels' coordinates)."""
    t = cfg.tree
    ng = t.ng
    nb = ranges.shape[0]
    r_lo = t.r_range_rsun[0] * R_SUN
    r_hi = t.r_range_rsun[1] * R_SUN
    pc = polytrope_constants(r_lo, r_hi, cfg.bg.poly_n, cfg.bg.density_contrast, cfg.bg.mu)
    rs = np.random.Generator(np.random.PCG64(seed))
    rc = rs.uniform(0.75, 0.95) * R_SUN
    tc = rs.uniform(np.pi / 3, 2 * np.pi / 3)
    pcen = rs.uniform(-np.pi / 2, np.pi / 2)
    sig = rs.uniform(0.03, 0.08) * R_SUN
    xc = np.array([rc * np.sin(tc) * np.cos(pcen), rc * np.sin(tc) * np.sin(pcen), rc * np.cos(tc)])
    cp_ = 2.5 * pc["R_gas"]
    B0 = b_frac * np.sqrt(pc["rho_b"]) * pc["c_b"]
    u = np.zeros((nb, 9, t.nk + 2 * ng, t.nj + 2 * ng, t.ni + 2 * ng))   # psi (index 8) starts at 0
    for b in range(nb):
        xi = cell_centres(ranges[b, 0], t.ni, ng)
        xj = cell_centres(ranges[b, 1], t.nj, ng)
        xk = cell_centres(ranges[b, 2], t.nk, ng)
        P, T, R = np.meshgrid(xk, xj, xi, indexing="ij")
        yin = bool(flags[b] & 1)
        if yin:
            Ry, Ty, Py = R, T, P
        else:
            Ry, Ty, Py = coord_conv(R, T, P)
        x = np.stack([Ry * np.sin(Ty) * np.cos(Py), Ry * np.sin(Ty) * np.sin(Py), Ry * np.cos(Ty)])
        d2 = ((x - xc[:, None, None, None]) ** 2).sum(0)
        u[b, 7] = amp * cp_ * np.exp(-d2 / (2 * sig * sig))
        q = (r_lo / Ry) ** 3
        br, bt, bp = 2 * B0 * q * np.cos(Ty), B0 * q * np.sin(Ty), np.zeros_like(Ry)
        if not yin:
            br, bt, bp = vec_conv(Ry, Ty, Py, br, bt, bp)
        u[b, 4], u[b, 5], u[b, 6] = br, bt, bp
        if b_div_amp:
            u[b, 4] += b_div_amp * B0 * np.exp(-d2 / (2 * sig * sig))
        if psi_amp:
            u[b, 8] = psi_amp * B0 * pc["c_b"] * np.exp(-d2 / (2 * sig * sig))
    return u
