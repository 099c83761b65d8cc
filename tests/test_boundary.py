"""The drop-in boundary with the driver's own data.

A Fortran driver keeps its physics inputs: the background profiles that
ModBlock_InitSSM takes from ModStratification_new_get_vars
(3_6/ModBlock.f90:233-264), the face-coefficient operator of an implicit solve
(3_5/ModBlock.f90:39-44) and the PFSS magnetogram (3_5/ModPFSS.f90:21-100,
3_5/ModMagnetogram.f90:13-80). These tests pass such data through the C ABI
and check it against the seeded builds (bit for bit) and against the oracle.
"""
import numpy as np
import pytest

import falcon_gb300 as fg
import oracle
from falcon_gb300 import config, synth
from falcon_gb300 import solver as S


@pytest.fixture(scope="module", autouse=True)
def _built(built_lib):
    return built_lib


def _perturbed(prof):
    """A different, still physical background: rho0, p0 and T0 modulated
    smoothly along r, gamma1 shifted, Xi scaled."""
    p = prof.copy()
    n = p.shape[2]
    w = 1.0 + 0.05 * np.cos(np.linspace(0.0, 3.0, n))[None, :]
    p[:, 1] *= w
    p[:, 2] *= w * w
    p[:, 3] *= w
    p[:, 4] *= 1.02
    p[:, 8] *= 0.97
    return p


# ---- background --------------------------------------------------------------
def test_set_background_round_trip_and_rejects_bad_profiles():
    f = fg.Falcon(config.tiny(device=-1))
    p2 = _perturbed(f.background())
    f.set_background(p2)
    assert np.array_equal(f.background(), p2)
    for blk, q, i, v in ((3, 1, 5, -1.0), (0, 8, 0, np.nan), (2, 2, 1, 0.0), (1, 6, 3, np.inf)):
        bad = p2.copy()
        bad[blk, q, i] = v
        with pytest.raises(fg.FalconError) as e:
            f.set_background(bad)
        assert e.value.code == fg.ERR_INVALID_ARG
        assert np.array_equal(f.background(), p2)     # rejected: unchanged


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [config.PREC_FP64, config.PREC_MIXED])
def test_own_profiles_through_set_background_step_bit_identical(prec):
    """The polytrope's own profiles uploaded through falcon_set_background
    leave every step bit-identical to the built-in background."""
    mk = lambda: config.tiny(precision=prec)
    a, b = fg.Falcon(mk()), fg.Falcon(mk())
    b.set_background(b.background())
    u0 = synth.initial_state(mk(), a.block_ranges(), a.block_flags(), seed=1021)
    for x in (a, b):
        x.upload_state(u0)
        x.exchange()
    for _ in range(3):
        assert a.advance_rk4() == b.advance_rk4()
    assert np.array_equal(a.download_state(), b.download_state())


@pytest.mark.gpu
def test_driver_background_fp64_bit_identical_to_oracle():
    """A background that is not the polytrope (the driver's profiles), given
    to the GPU path and to the oracle: FP64 steps stay bit-identical to the
    oracle's, and differ from the polytrope's (the profiles took effect)."""
    cfg = config.tiny()
    f, o, ref = fg.Falcon(cfg), oracle.Oracle(config.tiny()), fg.Falcon(config.tiny())
    p2 = _perturbed(f.background())
    f.set_background(p2)
    o.set_background(p2)
    assert np.array_equal(o.background(), p2)
    u0 = synth.initial_state(cfg, o.block_ranges(), o.block_flags(), seed=1022)
    f.upload_state(u0)
    ref.upload_state(u0)
    o.set_state(u0)
    for x in (f, o, ref):
        x.exchange()
        x.exchange()
    for _ in range(3):
        dtf, dto = f.advance_rk4(), o.step()
        ref.advance_rk4()
        assert dtf == dto
    uf = f.download_state()
    assert np.array_equal(uf, o.get_state())
    assert not np.array_equal(uf, ref.download_state())


# ---- solver operator, guess and magnetogram -----------------------------------
def _reference_magnetogram(sv):
    """A transliteration of ModMagnetogram_dipole_magnetogram_ALL
    (3_5/ModMagnetogram.f90:41-77): per bipole (centre, separation vector l,
    charge q; poles at centre +- l/2) and face, q (d+ . x/r) / |d+|^3 -
    q (d- . x/r) / |d-|^3 with d = x - pole, summed bipole by bipole. Two
    points differ from the reference on purpose (both are listed with the
    reference quirks in the design notes): the face centre is taken at the
    cell-centre theta (the reference takes theta at the face xj_F(j), half a
    cell off, :51), and the Yang blocks' points are converted to the Yin
    frame the charges live in (the reference converts the Yin blocks, :52).
    FP64 here as in the library (the reference's `real` is FP32). The
    workload adds a 1 G axial dipole, Br = cos(theta)."""
    ranges, flags, first = sv.block_ranges(), sv.block_flags(), sv.problem_blocks()
    mi, mj, mk = sv.m
    out = np.zeros((sv.nblocks, mk, mj))
    for q in range(sv.nproblems):
        src = sv.magnetogram_sources(q)
        pos, neg = src[0::2], src[1::2]
        assert np.array_equal(neg[:, 3], -pos[:, 3])
        centre = 0.5 * (pos[:, :3] + neg[:, :3])
        l = pos[:, :3] - neg[:, :3]
        qd = pos[:, 3]
        for b in range(first[q], first[q + 1]):
            if not flags[b] & 4:
                continue
            r_f = ranges[b, 0, 0]
            t0, t1 = ranges[b, 1]
            p0, p1 = ranges[b, 2]
            jj = np.arange(1, mj + 1)
            kk = np.arange(1, mk + 1)
            th = (t0 * ((mj - jj).astype(np.float32) + np.float32(0.5)).astype(np.float64) +
                  t1 * (jj.astype(np.float32) - np.float32(0.5)).astype(np.float64)) / mj
            ph = (p0 * ((mk - kk).astype(np.float32) + np.float32(0.5)).astype(np.float64) +
                  p1 * (kk.astype(np.float32) - np.float32(0.5)).astype(np.float64)) / mk
            T, P = np.meshgrid(th, ph)                 # [k][j]
            if not flags[b] & 1:                      # Yang block: to the Yin frame
                rtp = np.array([oracle.coord_conv((r_f, t, p)) for t, p in zip(T.ravel(), P.ravel())])
                T, P = rtp[:, 1].reshape(T.shape), rtp[:, 2].reshape(T.shape)
            xf = r_f * np.stack([np.cos(P) * np.sin(T), np.sin(P) * np.sin(T), np.cos(T)], -1)
            br = np.zeros(T.shape)
            for n in range(len(qd)):
                xp = centre[n] + l[n] / 2.0
                xn = centre[n] - l[n] / 2.0
                dp, dn = xf - xp, xf - xn
                rp = np.sqrt((dp ** 2).sum(-1))
                rn = np.sqrt((dn ** 2).sum(-1))
                br = br + qd[n] * (dp * xf / r_f).sum(-1) / rp ** 3 - qd[n] * (dn * xf / r_f).sum(-1) / rn ** 3
            out[b] = br + np.cos(T)
    return out


def test_synthetic_magnetogram_matches_the_reference_formula():
    sv = S.Solver(S.pfss_spec([(24, 45), (16, 24)], device=-1))
    br = sv.magnetogram()
    ref = _reference_magnetogram(sv)
    bottom = (sv.block_flags() & 4) != 0
    assert bottom.any() and (~bottom).any()
    assert not br[~bottom].any()
    err = np.abs(br - ref).max() / np.abs(ref).max()
    print("magnetogram vs reference formula: max relative error %.3e" % err)
    assert err <= 1e-12


def test_driver_magnetogram_sets_the_pfss_right_hand_side():
    """b(1,:,:) = Br * S_i(1,:,:) (3_5/ModPFSS.f90:45-48): the synthetic Br set
    back gives the same right-hand side bit for bit, twice Br twice it, entries
    off the bottom blocks are ignored, and non-finite values or a conduction
    solver are rejected."""
    sv = S.Solver(S.pfss_spec([(24, 45)], device=-1))
    br, b0 = sv.magnetogram(), sv.rhs()
    junk = br.copy()
    junk[(sv.block_flags() & 4) == 0] = 123.0
    sv.set_magnetogram(junk)
    assert np.array_equal(sv.rhs(), b0)
    assert np.array_equal(sv.magnetogram(), br)
    sv.set_magnetogram(2.0 * br)
    assert np.array_equal(sv.rhs(), 2.0 * b0)
    bad = br.copy()
    bad[(sv.block_flags() & 4) != 0] = np.nan
    with pytest.raises(fg.FalconError):
        sv.set_magnetogram(bad)
    cond = S.Solver(S.conduction_spec(nr=32, nt=32, np_=96, device=-1))
    with pytest.raises(fg.FalconError):
        cond.set_magnetogram(np.zeros((cond.nblocks, cond.m[2], cond.m[1])))


def test_driver_operator_rebuilds_the_coarse_levels():
    """An operator handed in replaces level 0 and the Galerkin coarse levels
    follow it: a solver seeded differently, given another's operator, has
    that solver's coarse operators bit for bit. Bad coefficients are rejected."""
    a = S.Solver(S.conduction_spec(nr=32, nt=32, np_=96, seed=3001, device=-1))
    b = S.Solver(S.conduction_spec(nr=32, nt=32, np_=96, seed=4242, device=-1))
    assert not np.array_equal(a.operator(0)[0], b.operator(0)[0])
    b.set_operator(*a.operator(0))
    for lvl in range(a.nlevels):
        for x, y in zip(a.operator(lvl), b.operator(lvl)):
            assert np.array_equal(x, y)
    ops = list(a.operator(0))
    ops[0] = ops[0].copy()
    ops[0][0, 0, 0, 0] = -1.0
    with pytest.raises(fg.FalconError):
        b.set_operator(*ops)
    ops = list(a.operator(0))
    ops[2] = ops[2].copy()
    ops[2][1, 1, 1, 1] = np.nan
    with pytest.raises(fg.FalconError):
        b.set_operator(*ops)


@pytest.mark.gpu
def test_solver_from_driver_data_matches_seeded_build_bit_for_bit():
    """A solver whose operator, right-hand side and guess come from the
    driver solves exactly as the seeded build it was given them from."""
    a = S.Solver(S.conduction_spec(nr=32, nt=32, np_=96, seed=3001))
    b = S.Solver(S.conduction_spec(nr=32, nt=32, np_=96, seed=4242))
    b.set_operator(*a.operator(0))
    b.set_rhs(a.rhs())
    x0 = np.random.default_rng(5).normal(size=(a.nblocks,) + a.m[::-1]) * np.abs(a.rhs()).max() / \
        np.abs(a.operator(0)[0]).max()
    for s in (a, b):
        s.set_guess(x0)
    ra = a.solve(tol=1e-8, max_iter=200)
    rb = b.solve(tol=1e-8, max_iter=200)
    assert ra["iterations"] == rb["iterations"] and ra["converged"] == rb["converged"] == 1
    xa, xb = a.solution(), b.solution()
    # the atomic per-problem dot products may sum in another order from run to
    # run, so the iterates agree to the solve's tolerance, not bit for bit
    assert np.abs(xa - xb).max() <= 1e-7 * np.abs(xa).max()
    assert (a.problem_residuals() <= 1.05e-8).all() and (b.problem_residuals() <= 1.05e-8).all()


@pytest.mark.gpu
def test_pfss_solution_is_linear_in_the_driver_magnetogram():
    sv = S.Solver(S.pfss_spec([(24, 45), (32, 60)]))
    br = sv.magnetogram()
    sv.solve(tol=1e-11, max_iter=400)
    x1 = sv.solution()
    sv.set_magnetogram(-3.0 * br)
    rep = sv.solve(tol=1e-11, max_iter=400)
    x3 = sv.solution()
    assert rep["converged"] == 1
    assert np.abs(x3 + 3.0 * x1).max() <= 1e-8 * np.abs(x3).max()


@pytest.mark.parametrize("shape,dtype", [((5, 9, 20, 20, 20), np.float64), ((7,), np.float32), ((3, 1), np.int8)])
def test_host_array_is_aligned_contiguous_and_writable(shape, dtype):
    """fg.host_array gives the driver-side state array at a 4096-byte
    boundary (whole 64-byte lines for every core run), C-contiguous, of the
    requested shape and type."""
    a = fg.host_array(shape, dtype)
    assert a.ctypes.data % 4096 == 0
    assert a.shape == shape and a.dtype == np.dtype(dtype) and a.flags["C_CONTIGUOUS"]
    a[...] = 1
    assert int(a.sum()) == int(np.prod(shape))
