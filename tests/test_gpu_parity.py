"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

FP64 mode must reproduce the oracle's state (every cell, ghosts included) to
1e-12 relative per variable after every RK4 step; with no FMA contraction and
the reference's operation order it is expected to be bit-identical. The mixed
mode is checked against the FP64 GPU path after 100 steps: relative L2 error
<= 1e-6 per variable, with the norm-wise max error reported beside it.
"""
import numpy as np
import pytest

import falcon_gb300 as fg
import oracle
from falcon_gb300 import config, synth

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12      # relative, norm-wise per variable
TOL_MIXED = 1e-6


@pytest.fixture(scope="module", autouse=True)
def _built(built_lib):
    return built_lib


def _pair(mk, seed=1001):
    cfg = mk()
    f = fg.Falcon(cfg)
    o = oracle.Oracle(mk())
    u0 = synth.initial_state(cfg, o.block_ranges(), o.block_flags(), seed=seed)
    f.upload_state(u0)
    o.set_state(u0)
    for x in (f, o):
        x.exchange()
        x.exchange()
    return f, o


def relerr(a, b):
    """per-variable norm-wise error max|a-b| / max|b| over every cell."""
    nv = a.shape[1]
    d = np.abs(a - b).transpose(1, 0, 2, 3, 4).reshape(nv, -1).max(1)
    s = np.abs(b).transpose(1, 0, 2, 3, 4).reshape(nv, -1).max(1)
    return d / np.where(s > 0, s, 1.0)


def test_exchange_matches_oracle_exactly():
    f, o = _pair(config.tiny)
    assert np.array_equal(f.download_state(), o.get_state())


@pytest.mark.parametrize("prec", [config.PREC_FP64])
def test_phase_by_phase_bit_identical(prec):
    """Each phase of ModAdvance_rk4 (CFL, stages 1-4 with their exchanges, the
    diffusion pass) leaves both state buffers identical to the oracle's."""
    f, o = _pair(config.tiny)
    names = ["cfl", "stage1", "stage2", "stage3", "stage4", "diffusion"]
    for ph in range(6):
        f.step_phase(ph)
        o.phase(ph)
        a, b = f.download_state(), o.get_state()
        assert np.array_equal(a, b), (names[ph], "u", relerr(a, b))
        if 1 <= ph <= 3:
            a, b = f.download_stage_state(), o.get_stage_state()
            assert np.array_equal(a, b), (names[ph], "u_rk", relerr(a, b))


def test_timestep_matches_oracle_exactly():
    f, o = _pair(config.tiny)
    assert f.timestep() == o.timestep()


def test_fp64_steps_tiny_bit_identical():
    f, o = _pair(config.tiny)
    for _ in range(3):
        dtf = f.advance_rk4()
        dto = o.step()
        assert dtf == dto
        a, b = f.download_state(), o.get_state()
        assert np.isfinite(a).all()
        assert np.array_equal(a, b), relerr(a, b)


def test_fp64_ten_steps_cfg1_within_1e12():
    """Plain FP64 Yin-Yang MHD, 864 blocks of 8^3: state after every step."""
    f, o = _pair(config.shell_fp64_cpu)
    worst = np.zeros(config.NVAR)
    for s in range(10):
        dtf = f.advance_rk4()
        dto = o.step()
        assert abs(dtf - dto) <= TOL_FP64 * dto
        e = relerr(f.download_state(), o.get_state())
        worst = np.maximum(worst, e)
        assert (e <= TOL_FP64).all(), (s, dict(zip(config.VAR_NAMES, e)))
    print("fp64 worst relative error per var:", dict(zip(config.VAR_NAMES, worst)))


@pytest.mark.parametrize("blocks", ["8cube", "16cube"])
def test_mixed_vs_fp64_gpu_100_steps(blocks):
    """FP32 state/RHS with FP64 p1 assembly against the FP64 GPU path after
    100 steps. Gate: relative L2 error ||u_mixed-u_64||_2/||u_64||_2 <= 1e-6
    per variable; the norm-wise max error max|d|/max|u| is reported and held
    below 1e-5 (FP32 storage alone puts it near 2e-6 for B after 100 steps).
    The same shell in 16^3 blocks runs the production forms of the mixed
    kernels (half-warp radial pushes, one thread per diffusion cell with the
    k slope carried between chunks)."""
    gk = {} if blocks == "8cube" else dict(block=(16, 16, 16), radial_levels=1, amr=())
    mk64 = lambda **kw: config.shell_fp64_cpu(**gk, **kw)
    mkmx = lambda **kw: config.shell_fp64_cpu(precision=config.PREC_MIXED, **gk, **kw)
    a = fg.Falcon(mk64())
    b = fg.Falcon(mkmx())
    u0 = synth.initial_state(mk64(), a.block_ranges(), a.block_flags(), seed=1002)
    for x in (a, b):
        x.upload_state(u0)
        x.exchange()
        x.exchange()
    for _ in range(100):
        a.advance_rk4(want_dt=False)
        b.advance_rk4(want_dt=False)
    a.synchronize()
    b.synchronize()
    ua, ub = a.download_state(), b.download_state()
    ia, ib = ua[:, :, 2:-2, 2:-2, 2:-2], ub[:, :, 2:-2, 2:-2, 2:-2]
    e = relerr(ib, ia)
    nv = ia.shape[1]
    da = (ib - ia).transpose(1, 0, 2, 3, 4).reshape(nv, -1)
    ra = ia.transpose(1, 0, 2, 3, 4).reshape(nv, -1)
    l2 = np.sqrt((da ** 2).sum(1)) / np.sqrt((ra ** 2).sum(1)).clip(1e-300)
    print("mixed vs fp64 max-normwise:", dict(zip(config.VAR_NAMES, e)))
    print("mixed vs fp64 relative L2:", dict(zip(config.VAR_NAMES, l2)))
    active = np.abs(ra).max(1) > 0
    assert (l2[active] <= TOL_MIXED).all(), dict(zip(config.VAR_NAMES, l2))
    assert (e[active] <= 10 * TOL_MIXED).all(), dict(zip(config.VAR_NAMES, e))


def test_mixed_step_matches_phase_sequence():
    """The mixed step (stage kernels writing the regular ghost faces of their
    neighbours, face-only exchanges between stages, two stage buffers) leaves
    exactly the state of the phase sequence, which uses full exchanges and one
    stage buffer updated in place: every cell, ghosts included, bit for bit."""
    mk = lambda: config.shell_fp64_cpu(precision=config.PREC_MIXED)
    a, b = fg.Falcon(mk()), fg.Falcon(mk())
    st = a.exchange_stats()
    assert st["pushed_faces"] > 0 and st["pushed_cells"] > 0
    u0 = synth.initial_state(mk(), a.block_ranges(), a.block_flags(), seed=1003)
    for x in (a, b):
        x.upload_state(u0)
        x.exchange()
    for _ in range(3):
        a.advance_rk4(want_dt=False)
        for ph in range(6):
            b.step_phase(ph)
    a.synchronize()
    ua, ub = a.download_state(), b.download_state()
    assert np.isfinite(ua).all()
    assert np.array_equal(ua, ub)


@pytest.mark.parametrize("radial_option", [1, 2])
def test_mixed_step_matches_phase_sequence_16(radial_option):
    """As above on 16^3 blocks (108 blocks), where the radial faces are pushed
    by half-warp gathers: option 1 splits the shell radially at the density
    scale-height midpoint (radial neighbours of different spacing, blended
    pushes), option 2 at the arithmetic midpoint."""
    mk = lambda: config.make_config(block=(16, 16, 16), root_tiles=(1, 3, 9), radial_levels=1,
                                    radial_option=radial_option, amr=(), precision=config.PREC_MIXED)
    a, b = fg.Falcon(mk()), fg.Falcon(mk())
    st = a.exchange_stats()
    assert st["pushed_faces"] > 0 and st["pushed_cells"] > 0
    u0 = synth.initial_state(mk(), a.block_ranges(), a.block_flags(), seed=1004)
    for x in (a, b):
        x.upload_state(u0)
        x.exchange()
    for _ in range(3):
        a.advance_rk4(want_dt=False)
        for ph in range(6):
            b.step_phase(ph)
    a.synchronize()
    ua, ub = a.download_state(), b.download_state()
    assert np.isfinite(ua).all()
    assert np.array_equal(ua, ub)


@pytest.mark.parametrize("blocks", ["8cube", "16cube"])
def test_every_kchunk_variant_computes_the_same_step(blocks):
    """Each compiled variant of the mixed stage and diffusion kernels (k-chunk
    depths; for 16^3 diffusion one or two threads per cell column), fixed
    with falcon_set_tuning instead of the autotuner, gives the same three
    steps bit for bit, pushes, fused CFL minimum and dt included."""
    blk = (8, 8, 8) if blocks == "8cube" else (16, 16, 16)
    mk = lambda: config.make_config(block=blk, root_tiles=(1, 3, 9), radial_levels=1, amr=(),
                                    precision=config.PREC_MIXED)
    kp = (2, 4, 8) if blocks == "8cube" else (1, 2, 4)
    ref = None
    for ks, kd in [(kp[0], kp[0]), (kp[1], kp[1]), (kp[2], kp[0]), (kp[0], kp[2])]:
        f = fg.Falcon(mk())
        f.set_tuning(ks, kd)
        assert f.tuning() == {"kpar_stage": ks, "kpar_diffusion": kd}
        u0 = synth.initial_state(mk(), f.block_ranges(), f.block_flags(), seed=1031)
        f.upload_state(u0)
        f.exchange()
        dts = [f.advance_rk4() for _ in range(3)]
        out = (dts, f.download_state())
        assert np.isfinite(out[1]).all()
        if ref is None:
            ref = out
        else:
            assert out[0] == ref[0], (ks, kd)
            assert np.array_equal(out[1], ref[1]), (ks, kd)
        f.close()
    g = fg.Falcon(mk())
    with pytest.raises(fg.FalconError):
        g.set_tuning(3, kp[0])


def test_persistent_step_equals_graph_step():
    """The persistent step (one cooperative launch: dt, four stages with their
    face exchanges, diffusion, final exchange, bounded grid barriers) against
    the captured graph, from the same state, on 16^3 blocks split radially
    (blended radial pushes) and on the 1,296-block shell: the same dt and the
    same state bit for bit after four steps, the first of them starting from a
    freshly uploaded state (its CFL minimum from k_cfl)."""
    for mk in (lambda: config.make_config(block=(16, 16, 16), root_tiles=(1, 3, 9), radial_levels=1, radial_option=1,
                                          amr=(), precision=config.PREC_MIXED),
               lambda: config.make_config(block=(16, 16, 16), root_tiles=(3, 3, 9), radial_levels=1, radial_option=1,
                                          amr=((0, 1, 1),), precision=config.PREC_MIXED)):
        a, b = fg.Falcon(mk()), fg.Falcon(mk())
        b.set_step_mode(fg.STEP_PERSISTENT)
        u0 = synth.initial_state(mk(), a.block_ranges(), a.block_flags(), seed=1041)
        for x in (a, b):
            x.upload_state(u0)
            x.exchange()
        for _ in range(4):
            assert a.advance_rk4() == b.advance_rk4()
        ua, ub = a.download_state(), b.download_state()
        assert np.isfinite(ua).all()
        assert np.array_equal(ua, ub)
        a.close()
        b.close()
    f = fg.Falcon(config.tiny(precision=config.PREC_MIXED))    # 8^3 blocks: not covered
    with pytest.raises(fg.FalconError):
        f.set_step_mode(fg.STEP_PERSISTENT)
    f64 = fg.Falcon(config.make_config(block=(16, 16, 16), root_tiles=(1, 3, 9), radial_levels=1, amr=()))
    with pytest.raises(fg.FalconError):
        f64.set_step_mode(fg.STEP_PERSISTENT)


def test_persistent_step_wait_that_runs_out_returns_timeout():
    """With the poll limit at 0 every bounded wait of the persistent step runs
    out at once (the copy waits in the kernel bodies and the grid barriers,
    which then let their CTA go on): the step returns FALCON_ERR_TIMEOUT, not a
    hang or a fault, and with the default limit restored and the state
    uploaded again the next step equals the graph step's bit for bit."""
    mk = lambda: config.make_config(block=(16, 16, 16), root_tiles=(1, 3, 9), radial_levels=1, amr=(),
                                    precision=config.PREC_MIXED)
    f, ref = fg.Falcon(mk()), fg.Falcon(mk())
    f.set_step_mode(fg.STEP_PERSISTENT)
    u0 = synth.initial_state(mk(), f.block_ranges(), f.block_flags(), seed=1042)
    for x in (f, ref):
        x.upload_state(u0)
        x.exchange()
    f.advance_rk4()
    f.upload_state(u0)
    f.exchange()
    f.set_wait_limit(0)
    with pytest.raises(fg.FalconError) as e:
        f.advance_rk4()
    assert e.value.code == fg.ERR_TIMEOUT, e.value
    f.set_wait_limit(-1)
    f.upload_state(u0)
    f.exchange()
    assert f.advance_rk4() == ref.advance_rk4()
    assert np.array_equal(f.download_state(), ref.download_state())


@pytest.mark.parametrize("prec", [config.PREC_FP64, config.PREC_MIXED])
def test_seeded_synthetic_state_is_reproducible(prec):
    """falcon_init_synthetic with one seed gives the same state bit for bit in
    two contexts: the velocity field's normalisation sums per-CTA partial sums
    in a fixed order (no floating-point atomics)."""
    mk = lambda: config.make_config(block=(16, 16, 16), root_tiles=(1, 3, 9), radial_levels=1, amr=(), precision=prec)
    a, b = fg.Falcon(mk()), fg.Falcon(mk())
    for f in (a, b):
        f.init_synthetic(kind=1, seed=1002, mach=0.01)
    ua, ub = a.download_state(), b.download_state()
    assert np.isfinite(ua).all() and np.abs(ua[:, 1:4]).max() > 0
    assert np.array_equal(ua, ub)


def test_full_size_mixed_properties():
    """21M cells, 5,184 blocks of 16^3: steps stay finite, the exchange is
    idempotent (bit-exact), dt is positive and stable."""
    f = fg.Falcon(config.shell_mixed_21m())
    f.init_synthetic(kind=1, seed=1002, mach=0.01)
    f.exchange()
    f.exchange()
    dts = [f.advance_rk4() for _ in range(3)]
    assert all(d > 0 for d in dts)
    assert max(dts) / min(dts) < 1.5
    u1 = f.download_state()
    f.exchange()
    u2 = f.download_state()
    assert np.isfinite(u1).all()
    assert np.array_equal(u1, u2)


def test_mixed_vs_fp64_full_size_100_steps():
    """The headline workload's accuracy on the headline workload itself: the
    21,233,664-cell shell (5,184 blocks of 16^3) from the seeded random-phase
    Kolmogorov velocity (rms Mach 0.01, seed 1002), 100 RK4 steps in MIXED
    and in FP64 on the GPU (each with its own dt sequence). Gate per evolved
    variable over the interior cells: relative L2 <= 1e-6 and norm-wise max
    <= 1e-5."""
    from falcon_gb300.compare import state_errors, worst
    ctxs = []
    for prec in (config.PREC_FP64, config.PREC_MIXED):
        f = fg.Falcon(config.shell_mixed_21m(precision=prec))
        f.init_synthetic(kind=1, seed=1002, mach=0.01)
        f.exchange()
        f.exchange()
        f.run_steps(100)
        f.synchronize()
        ctxs.append(f)
    u64 = ctxs[0].download_state()
    ctxs[0].close()
    umx = ctxs[1].download_state()
    ctxs[1].close()
    e = state_errors(umx, u64)
    print("21M-cell mixed vs fp64 after 100 steps:", e)
    assert np.isfinite(umx).all()
    assert worst(e, "rel_l2") <= TOL_MIXED, e
    assert worst(e, "rel_max") <= 10 * TOL_MIXED, e


def test_fp64_full_size_block16_vs_oracle_one_step():
    """16^3 blocks in FP64: one step against the oracle on a reduced shell
    (per panel 32 x 48 x 144 cells, 2 x 3 x 9 blocks)."""
    mk = lambda **kw: config.make_config(block=(16, 16, 16), root_tiles=(1, 3, 9), radial_levels=1,
                                         radial_option=1, amr=(), **kw)
    f, o = _pair(mk)
    dtf, dto = f.advance_rk4(), o.step()
    assert dtf == dto
    e = relerr(f.download_state(), o.get_state())
    assert (e <= TOL_FP64).all(), dict(zip(config.VAR_NAMES, e))


def test_nan_in_state_is_reported_not_trapped():
    f, o = _pair(config.tiny)
    u = f.download_state()
    u[3, 7, 5, 5, 5] = np.nan
    f.upload_state(u)
    with pytest.raises(fg.FalconError) as e:
        f.advance_rk4()
    assert e.value.code == fg.ERR_NAN_DETECTED


def test_nan_formed_in_a_mixed_step_is_reported_by_the_next():
    """A NaN that first appears inside a mixed step (here: FP32 products of a
    huge but finite velocity overflow) is caught by the next step's CFL
    minimum, which the diffusion pass forms from the values it writes, and
    reported as FALCON_ERR_NAN_DETECTED rather than propagated."""
    mk = lambda: config.make_config(block=(16, 16, 16), root_tiles=(1, 3, 9), radial_levels=1, amr=(),
                                    precision=config.PREC_MIXED)
    f = fg.Falcon(mk())
    u0 = synth.initial_state(mk(), f.block_ranges(), f.block_flags(), seed=1012)
    u0[5, 1, 8, 8, 8] = 1e30   # vr of one interior cell: finite, its square is not
    f.upload_state(u0)
    with pytest.raises(fg.FalconError) as e:
        for _ in range(4):
            f.advance_rk4()
    assert e.value.code == fg.ERR_NAN_DETECTED


@pytest.mark.parametrize("prec", [config.PREC_FP64, config.PREC_MIXED])
def test_copy_wait_that_runs_out_returns_timeout(prec):
    """The step kernels' waits for their bulk copies are bounded. With the
    poll limit at 0 every wait runs out on a valid state: each CTA leaves
    uniformly after its copies in flight have landed, the step returns
    FALCON_ERR_TIMEOUT (not a hang, not a fault, not 'NaN detected'), and the
    context stays usable: with the default limit restored and the state
    uploaded again, the next step equals a fresh context's bit for bit."""
    mk = lambda: config.make_config(block=(16, 16, 16), root_tiles=(1, 3, 9), radial_levels=1, amr=(),
                                    precision=prec)
    f, ref = fg.Falcon(mk()), fg.Falcon(mk())
    u0 = synth.initial_state(mk(), f.block_ranges(), f.block_flags(), seed=1013)
    for x in (f, ref):
        x.upload_state(u0)
        x.exchange()
    f.advance_rk4()            # the autotuner runs before the first step: keep it out of the test
    f.upload_state(u0)
    f.exchange()
    f.set_wait_limit(0)
    with pytest.raises(fg.FalconError) as e:
        f.advance_rk4()
    assert e.value.code == fg.ERR_TIMEOUT, e.value
    assert "wait ran out" in str(e.value)
    f.set_wait_limit(-1)
    f.upload_state(u0)
    f.exchange()
    dt_f, dt_r = f.advance_rk4(), ref.advance_rk4()
    assert dt_f == dt_r
    assert np.array_equal(f.download_state(), ref.download_state())


# ---- div-B control: GLM cleaning (divb_option 1, psi evolved) and the ----
# ---- Powell source term (divb_option 2) --------------------------------
def _init_divb(cfg, ranges, flags, divb, seed):
    if divb == 1:
        return synth.initial_state(cfg, ranges, flags, seed=seed, psi_amp=1e-3)
    return synth.initial_state(cfg, ranges, flags, seed=seed, b_div_amp=0.3)


def _divb_pair(mk, divb, seed=1004):
    cfg = mk(divb_option=divb)
    f = fg.Falcon(cfg)
    o = oracle.Oracle(mk(divb_option=divb))
    u0 = _init_divb(cfg, o.block_ranges(), o.block_flags(), divb, seed)
    f.upload_state(u0)
    o.set_state(u0)
    for x in (f, o):
        x.exchange()
        x.exchange()
    return f, o


@pytest.mark.parametrize("divb", [1, 2])
def test_divb_phase_by_phase_bit_identical(divb):
    """GLM: the terms in each RK stage (-grad psi on B, the psi equation with
    the step-start wave speed and h_LLL), psi's diffusion and exchange.
    Powell: -(div B) v on B. Both state buffers, psi included, identical to
    the oracle after every phase."""
    f, o = _divb_pair(config.tiny, divb)
    names = ["cfl", "stage1", "stage2", "stage3", "stage4", "diffusion"]
    for ph in range(6):
        f.step_phase(ph)
        o.phase(ph)
        a, b = f.download_state(), o.get_state()
        assert (np.abs(b[:, 8]).max() > 0) == (divb == 1)
        assert np.array_equal(a, b), (names[ph], "u", relerr(a, b))
        if 1 <= ph <= 3:
            a, b = f.download_stage_state(), o.get_stage_state()
            assert np.array_equal(a, b), (names[ph], "u_rk", relerr(a, b))


@pytest.mark.parametrize("divb", [1, 2])
def test_divb_fp64_steps_bit_identical(divb):
    f, o = _divb_pair(config.tiny, divb)
    for _ in range(3):
        assert f.advance_rk4() == o.step()
        a, b = f.download_state(), o.get_state()
        assert np.isfinite(a).all()
        assert np.array_equal(a, b), relerr(a, b)


@pytest.mark.parametrize("divb", [1, 2])
def test_divb_fp64_ten_steps_cfg1_within_1e12(divb):
    f, o = _divb_pair(config.shell_fp64_cpu, divb)
    for s in range(10):
        dtf, dto = f.advance_rk4(), o.step()
        assert abs(dtf - dto) <= TOL_FP64 * dto
        e = relerr(f.download_state(), o.get_state())
        assert (e <= TOL_FP64).all(), (s, dict(zip(config.VAR_NAMES, e)))


@pytest.mark.parametrize("blocks", ["8cube", "16cube"])
@pytest.mark.parametrize("divb", [1, 2])
def test_divb_mixed_vs_fp64_gpu_100_steps(divb, blocks):
    """The mixed path with GLM or Powell against the FP64 GPU path after 100
    steps: relative L2 <= 1e-6 for every variable, psi included (psi is
    driven by the divergence of B formed from FP32 values); also on the same
    shell in 16^3 blocks."""
    gk = {} if blocks == "8cube" else dict(block=(16, 16, 16), radial_levels=1, amr=())
    mk64 = lambda: config.shell_fp64_cpu(divb_option=divb, **gk)
    mkmx = lambda: config.shell_fp64_cpu(divb_option=divb, precision=config.PREC_MIXED, **gk)
    a, b = fg.Falcon(mk64()), fg.Falcon(mkmx())
    u0 = _init_divb(mk64(), a.block_ranges(), a.block_flags(), divb, 1005)
    for x in (a, b):
        x.upload_state(u0)
        x.exchange()
        x.exchange()
    for _ in range(100):
        a.advance_rk4(want_dt=False)
        b.advance_rk4(want_dt=False)
    a.synchronize()
    b.synchronize()
    ia = a.download_state()[:, :, 2:-2, 2:-2, 2:-2]
    ib = b.download_state()[:, :, 2:-2, 2:-2, 2:-2]
    nv = ia.shape[1]
    da = (ib - ia).transpose(1, 0, 2, 3, 4).reshape(nv, -1)
    ra = ia.transpose(1, 0, 2, 3, 4).reshape(nv, -1)
    l2 = np.sqrt((da ** 2).sum(1)) / np.sqrt((ra ** 2).sum(1)).clip(1e-300)
    print("divb_option %d mixed vs fp64 relative L2:" % divb, dict(zip(config.VAR_NAMES, l2)))
    active = np.abs(ra).max(1) > 0
    assert active[8] == (divb == 1)
    assert (l2[active] <= TOL_MIXED).all(), dict(zip(config.VAR_NAMES, l2))


@pytest.mark.parametrize("divb", [1, 2])
def test_divb_mixed_step_matches_phase_sequence(divb):
    mk = lambda: config.shell_fp64_cpu(divb_option=divb, precision=config.PREC_MIXED)
    a, b = fg.Falcon(mk()), fg.Falcon(mk())
    u0 = _init_divb(mk(), a.block_ranges(), a.block_flags(), divb, 1006)
    for x in (a, b):
        x.upload_state(u0)
        x.exchange()
    for _ in range(3):
        a.advance_rk4(want_dt=False)
        for ph in range(6):
            b.step_phase(ph)
    a.synchronize()
    ua, ub = a.download_state(), b.download_state()
    assert np.isfinite(ua).all()
    assert np.array_equal(ua, ub)


@pytest.mark.parametrize("prec", [config.PREC_FP64, config.PREC_MIXED])
def test_upload_rejects_nonzero_psi_without_glm(prec):
    """Without GLM psi is not evolved (the reference leaves it 0): an upload
    with a non-zero psi fails and leaves the device state as it was."""
    f = fg.Falcon(config.tiny(precision=prec))
    u0 = synth.initial_state(config.tiny(), f.block_ranges(), f.block_flags(), seed=1007)
    f.upload_state(u0)
    before = f.download_state()
    u1 = u0.copy()
    u1[3, 8, 4, 5, 6] = 1e-9
    with pytest.raises(fg.FalconError) as e:
        f.upload_state(u1)
    assert e.value.code == fg.ERR_INVALID_ARG and "psi" in str(e.value)
    assert np.array_equal(before, f.download_state())


@pytest.mark.parametrize("divb", [0, 1])
def test_mixed_transfers_through_pinned_buffers_match_staged(divb):
    """A pinned host array is read and written in place by the GPU (no
    staging copy); the device state and the downloads are bit-identical to
    the staged path's, and the psi check still rejects before any change."""
    mk = lambda: config.tiny(precision=config.PREC_MIXED, divb_option=divb)
    a, b = fg.Falcon(mk()), fg.Falcon(mk())
    u0 = synth.initial_state(mk(), a.block_ranges(), a.block_flags(), seed=1008, psi_amp=1e-3 if divb else 0.0)
    pinned = np.ascontiguousarray(u0.copy())
    a.pin_host(pinned)
    try:
        a.upload_state_raw(pinned)
        b.upload_state(u0)
        for x in (a, b):
            x.exchange()
            x.advance_rk4(want_dt=False)
        out = np.zeros_like(pinned)
        a.pin_host(out)
        try:
            a.download_state_into(out)
            assert np.array_equal(out, b.download_state())
            assert np.array_equal(a.download_state(), b.download_state())
        finally:
            a.unpin_host(out)
        if divb == 0:
            before = a.download_state()
            pinned[2, 8, 3, 3, 3] = 5.0
            with pytest.raises(fg.FalconError) as e:
                a.upload_state_raw(pinned)
            assert e.value.code == fg.ERR_INVALID_ARG
            assert np.array_equal(before, a.download_state())
    finally:
        a.unpin_host(pinned)


def _core_mask(shape):
    """Core cells of the state array: interior planes x interior rows (whole rows)."""
    m = np.zeros(shape, dtype=bool)
    m[:, :, 2:-2, 2:-2, :] = True
    return m


@pytest.mark.gpu
@pytest.mark.parametrize("how", ["upload", "upload_core", "init_synthetic"])
def test_new_state_replaces_the_pending_cfl_minimum(how):
    """A mixed step leaves the CFL minimum of u^{n+1}, formed by its diffusion
    pass, pending for the next step. A state put in its place (full or core
    upload, synthetic initial condition) is timed by its own minimum only:
    after a step of a state with faster waves, the next dt equals the dt a
    fresh context computes for the new state."""
    mk = lambda: config.make_config(block=(16, 16, 16), root_tiles=(1, 3, 9), radial_levels=1, amr=(),
                                    precision=config.PREC_MIXED)
    a, b = fg.Falcon(mk()), fg.Falcon(mk())
    if how == "init_synthetic":
        a.init_synthetic(kind=1, seed=1002, mach=0.3)
        a.advance_rk4()
        a.init_synthetic(kind=1, seed=1002, mach=0.01)
        b.init_synthetic(kind=1, seed=1002, mach=0.01)
    else:
        slow = synth.initial_state(mk(), a.block_ranges(), a.block_flags(), seed=1011, b_frac=1e-3)
        fast = synth.initial_state(mk(), a.block_ranges(), a.block_flags(), seed=1011, b_frac=0.5)
        a.upload_state(fast)
        a.exchange()
        a.advance_rk4()
        if how == "upload":
            a.upload_state(slow)
        else:
            host = np.ascontiguousarray(slow.copy())
            a.pin_host(host)
            try:
                a.upload_state_core(host)
            finally:
                a.unpin_host(host)
        b.upload_state(slow)
        b.exchange()
    dt_a, dt_b = a.advance_rk4(), b.advance_rk4()
    assert dt_a == dt_b, (dt_a, dt_b)
    assert a.advance_rk4() == b.advance_rk4()


@pytest.mark.parametrize("divb", [0, 1])
@pytest.mark.parametrize("grid", ["8cube", "16cube", "16amr"])
def test_core_transfers_match_full(divb, grid):
    """Core upload (interior planes x interior rows moved, theta/phi ghost
    layers recomputed on the device) leaves the state that a full upload and
    an exchange leave: two steps later both agree bit for bit on every cell
    that is core or a ghost-map target. The core download writes exactly the
    core cells of the full download and no other; a non-zero psi without GLM
    is rejected with the state unchanged."""
    kw = dict(precision=config.PREC_MIXED, divb_option=divb)
    if grid == "8cube":
        mk = lambda: config.tiny(**kw)
    else:
        amr = ((0, 1, 1),) if grid == "16amr" else ()
        mk = lambda: config.make_config(block=(16, 16, 16), root_tiles=(1, 3, 9), radial_levels=1, amr=amr, **kw)
    a, b = fg.Falcon(mk()), fg.Falcon(mk())
    u0 = synth.initial_state(mk(), a.block_ranges(), a.block_flags(), seed=1011, psi_amp=1e-3 if divb else 0.0)
    host = np.ascontiguousarray(u0.copy())
    a.pin_host(host)
    try:
        a.upload_state_core(host)
        b.upload_state(u0)
        b.exchange()
        # the stage buffer starts as a copy of the state after either upload
        # (interior cells: the core's radial ghost columns are recomputed by
        # the core upload's exchange, the full upload keeps u0's)
        inner = (slice(None), slice(None), slice(2, -2), slice(2, -2), slice(2, -2))
        assert np.array_equal(a.download_stage_state()[inner], b.download_stage_state()[inner])
        for x in (a, b):
            for _ in range(2):
                x.advance_rk4(want_dt=False)
        full = b.download_state()
        core = _core_mask(full.shape)
        gm = a.ghost_map()
        listed = np.zeros(full.shape, dtype=bool)
        listed[gm["tblock"], :, gm["tk"] + 1, gm["tj"] + 1, gm["ti"] + 1] = True
        ua = a.download_state()
        assert np.isfinite(ua[core]).all()
        assert np.array_equal(ua[core | listed], full[core | listed])
        host[...] = np.nan
        a.download_state_core(host)
        assert np.array_equal(host[core], full[core])
        assert np.isnan(host[~core]).all()
        if divb == 0:
            before = a.download_state()
            host[...] = u0
            host[2, 8, 3, 3, 3] = 5.0
            with pytest.raises(fg.FalconError) as e:
                a.upload_state_core(host)
            assert e.value.code == fg.ERR_INVALID_ARG and "psi" in str(e.value)
            assert np.array_equal(before, a.download_state())
    finally:
        a.unpin_host(host)


@pytest.mark.gpu
def test_core_upload_after_a_nan_step_starts_clean():
    """A step that met a NaN leaves NaNs in both state buffers and the stage
    buffer. A state put in place by the core upload must not read any of them
    (some ghost cells enter the step's interpolations with weight 0): its next
    steps equal, on every core and listed cell, those of a context that never
    saw the NaN."""
    mk = lambda: config.make_config(block=(16, 16, 16), root_tiles=(1, 3, 9), radial_levels=1, amr=((0, 1, 1),),
                                    precision=config.PREC_MIXED)
    a, b = fg.Falcon(mk()), fg.Falcon(mk())
    u0 = synth.initial_state(mk(), a.block_ranges(), a.block_flags(), seed=1011)
    bad = u0.copy()
    bad[:, 0] = np.nan
    a.upload_state(bad)
    with pytest.raises(fg.FalconError) as e:
        a.advance_rk4()
    assert e.value.code == fg.ERR_NAN_DETECTED
    host = np.ascontiguousarray(u0.copy())
    a.pin_host(host)
    try:
        a.upload_state_core(host)
    finally:
        a.unpin_host(host)
    b.upload_state(u0)
    b.exchange()
    for _ in range(2):
        assert a.advance_rk4() == b.advance_rk4()
    full = b.download_state()
    ua = a.download_state()
    gm = a.ghost_map()
    sel = _core_mask(full.shape)
    sel[gm["tblock"], :, gm["tk"] + 1, gm["tj"] + 1, gm["ti"] + 1] = True
    assert np.isfinite(ua[sel]).all()
    assert np.array_equal(ua[sel], full[sel])
