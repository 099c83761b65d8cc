"""ctypes mirrors of the C-ABI structs in include/falcon_gb300.h and the named
workload presets.

The presets describe the Yin-Yang grids the benchmarks run on. They are what a
PARAM.in would carry (#DOMAIN, #GRID, #RADIALGRID, #AMR; see
3_6/ModReadParameters.f90:60-106,408-483), plus the root tiling that makes
non-power-of-two block counts per panel reachable.
"""
import ctypes as C
import math

MAX_AMR = 16
NVAR = 9          # variables of the host block arrays (the reference's Dynamo MHD block)
NVAR_EVOLVED = 8  # rho1 .. s1; psi (index 8) is evolved only with divb_option = 1
NPROF = 9
PREC_FP64 = 0
PREC_MIXED = 1

# variable order of the Dynamo MHD block (3_6/ModBlock.f90:153-163)
VAR_NAMES = ("rho1", "vr", "vt", "vp", "br", "bt", "bp", "s1", "psi")


class TreeSpec(C.Structure):
    _fields_ = [
        ("ni", C.c_int32), ("nj", C.c_int32), ("nk", C.c_int32), ("ng", C.c_int32),
        ("root_tiles", C.c_int32 * 3),
        ("radial_levels", C.c_int32),
        ("radial_option", C.c_int32),
        ("n_amr", C.c_int32),
        ("amr_divide", (C.c_int32 * 3) * MAX_AMR),
        ("amr_global", C.c_int32 * MAX_AMR),
        ("amr_range", ((C.c_double * 2) * 3) * MAX_AMR),
        ("r_range_rsun", C.c_double * 2),
    ]


class Physics(C.Structure):
    _fields_ = [
        ("if_involve_B", C.c_int32),
        ("divb_option", C.c_int32),
        ("cfl", C.c_double),
        ("heating_ratio", C.c_double),
    ]


class BackgroundSpec(C.Structure):
    _fields_ = [
        ("poly_n", C.c_double),
        ("density_contrast", C.c_double),
        ("mu", C.c_double),
        ("xi_mode", C.c_int32),
        ("pad_", C.c_int32),
    ]


class Config(C.Structure):
    _fields_ = [
        ("tree", TreeSpec),
        ("phys", Physics),
        ("bg", BackgroundSpec),
        ("precision", C.c_int32),
        ("device", C.c_int32),
    ]


class GhostEntry(C.Structure):
    _fields_ = [
        ("tblock", C.c_int32), ("ti", C.c_int32), ("tj", C.c_int32), ("tk", C.c_int32),
        ("sblock", C.c_int32), ("pad_", C.c_int32),
        ("src_x", C.c_double * 3),
    ]


def make_config(block=(8, 8, 8), ng=2, root_tiles=(1, 3, 9), radial_levels=2,
                radial_option=1, amr=((0, 1, 1),), r_range=(0.7, 1.0), cfl=0.4,
                precision=PREC_FP64, device=0, if_involve_B=1, heating_ratio=1.0,
                poly_n=1.5, density_contrast=100.0, mu=0.6, xi_mode=1, divb_option=0):
    """Build a Config. amr is a sequence of (r, theta, phi) divide flags; each level
    is global over the whole radial range, like `#AMR ... T rmin rmax`."""
    cfg = Config()
    t = cfg.tree
    t.ni, t.nj, t.nk = block
    t.ng = ng
    for d in range(3):
        t.root_tiles[d] = root_tiles[d]
    t.radial_levels = radial_levels
    t.radial_option = radial_option
    t.n_amr = len(amr)
    for l, flags in enumerate(amr):
        for d in range(3):
            t.amr_divide[l][d] = int(flags[d])
        t.amr_global[l] = 1
        t.amr_range[l][0][0] = r_range[0]
        t.amr_range[l][0][1] = r_range[1]
        t.amr_range[l][1][0] = 0.0
        t.amr_range[l][1][1] = math.pi
        t.amr_range[l][2][0] = -math.pi
        t.amr_range[l][2][1] = math.pi
    t.r_range_rsun[0], t.r_range_rsun[1] = r_range
    cfg.phys.if_involve_B = if_involve_B
    cfg.phys.divb_option = divb_option   # 1: GLM cleaning, psi evolved
    cfg.phys.cfl = cfl
    cfg.phys.heating_ratio = heating_ratio
    cfg.bg.poly_n = poly_n
    cfg.bg.density_contrast = density_contrast
    cfg.bg.mu = mu
    cfg.bg.xi_mode = xi_mode
    cfg.precision = precision
    cfg.device = device
    return cfg


def shell_fp64_cpu(**kw):
    """Plain FP64 Yin-Yang MHD, CPU-runnable: per panel 32x48x144 cells in 8^3
    blocks (4 x 6 x 18 blocks per panel, 864 blocks), 2 ghost layers.
    Radial block faces by density-scale-height bisection (Divide_r option 1)."""
    args = dict(block=(8, 8, 8), root_tiles=(1, 3, 9), radial_levels=2,
                radial_option=1, amr=((0, 1, 1),), precision=PREC_FP64)
    args.update(kw)
    return make_config(**args)


def shell_mixed_21m(**kw):
    """Mixed-precision MHD at scale: per panel 96x192x576 cells in 16^3 blocks
    (6 x 12 x 36 blocks per panel, 5,184 blocks, 21,233,664 cells)."""
    args = dict(block=(16, 16, 16), root_tiles=(3, 3, 9), radial_levels=1,
                radial_option=1, amr=((0, 1, 1), (0, 1, 1)), precision=PREC_MIXED)
    args.update(kw)
    return make_config(**args)


def tiny(**kw):
    """A small grid for quick checks: per panel 16x24x72 cells in 8^3 blocks."""
    args = dict(block=(8, 8, 8), root_tiles=(1, 3, 9), radial_levels=1,
                radial_option=1, amr=(), precision=PREC_FP64)
    args.update(kw)
    return make_config(**args)


def padded_cells(cfg):
    t = cfg.tree
    return (t.ni + 2 * t.ng) * (t.nj + 2 * t.ng) * (t.nk + 2 * t.ng)
