"""Implicit solvers: operator, halo map and SpMV parity with the CPU oracle,
and solves checked by an independent FP64 residual computed on the CPU.

Reference components: 3_5/ModPFSS.f90:21-100 (PFSS operator),
3_5/ModGC.f90:53-284 (1-layer face-ghost halo), 3_5/ModLinearSolver.f90:15-84
(SpMV), 3_5/ModLinearSolver.f90:313-427 (MG-preconditioned CG).
"""
import numpy as np
import pytest

import oracle
from falcon_gb300 import config, solver as S


@pytest.fixture(scope="module", autouse=True)
def _built(built_lib, oracle_lib):
    return built_lib


SIZES = [(24, 45), (33, 60)]


def oracle_for_pfss(nr, nt, block=8, r_range=(1.0, 2.5)):
    """The oracle's tree for one PFSS problem, with the product's mapping."""
    Nr = -(-nr // block)
    Nt = -(-(nt // 2) // block)
    cfg = config.make_config(block=(block,) * 3, root_tiles=(Nr, Nt, 3 * Nt), radial_levels=0, radial_option=2,
                             amr=(), r_range=r_range)
    return oracle.Oracle(cfg)


def test_pfss_operator_bit_identical_to_reference_formulas():
    sv = S.Solver(S.pfss_spec(SIZES, device=-1))
    first = sv.problem_blocks()
    A = sv.operator(0)
    for q, (nr, nt) in enumerate(SIZES):
        o = oracle_for_pfss(nr, nt)
        B = oracle.pfss_operator(o, 8)
        sl = slice(first[q], first[q + 1])
        assert o.nblocks == first[q + 1] - first[q]
        for a, b in zip(A, B):
            assert np.array_equal(a[sl], b)


def test_halo_map_matches_reference_order_independent():
    sv = S.Solver(S.pfss_spec(SIZES, device=-1))
    first = sv.problem_blocks()
    idx, wx = sv.halo_map(0)
    for q, (nr, nt) in enumerate(SIZES):
        o = oracle_for_pfss(nr, nt)
        ridx, rwx, clamped = oracle.hc_halo(o, 8)
        mine = idx[(idx[:, 0] >= first[q]) & (idx[:, 0] < first[q + 1])].copy()
        mwx = wx[(idx[:, 0] >= first[q]) & (idx[:, 0] < first[q + 1])]
        mine[:, 0] -= first[q]
        mine[:, 4] -= first[q]
        key = lambda a: np.lexsort((a[:, 3], a[:, 2], a[:, 1], a[:, 0]))
        om, orr = key(mine), key(ridx)
        mine, mwx = mine[om], mwx[om]
        ridx, rwx, clamped = ridx[orr], rwx[orr], clamped[orr]
        assert len(mine) == len(ridx)
        # same targets, owners and source-frame coordinates (bit-exact)
        assert np.array_equal(mine[:, :5], ridx[:, :5])
        assert np.array_equal(mwx[:, 3:], rwx[:, 3:])
        # unclamped entries: identical base cells and weights
        u = clamped == 0
        assert np.array_equal(mine[u, 5:], ridx[u, 5:])
        assert np.array_equal(mwx[u, :3], rwx[u, :3])
        assert u.mean() > 0.5


def test_galerkin_coarse_operator_is_ptap():
    sv = S.Solver(S.conduction_spec(nr=32, nt=32, np_=96, block=16, nlevels=2, device=-1))
    Aii, Ai, Aj, Ak = sv.operator(0)
    C = sv.operator(1)
    b = 3
    m = 16
    # dense block operator (interior couplings only) and P^T A P
    n = m ** 3
    idx = lambda i, j, k: (k * m + j) * m + i
    Ad = np.zeros((n, n))
    for k in range(m):
        for j in range(m):
            for i in range(m):
                c = idx(i, j, k)
                Ad[c, c] = Aii[b, k, j, i]
                if i > 0: Ad[c, idx(i - 1, j, k)] = Ai[b, k, j, i]
                if i < m - 1: Ad[c, idx(i + 1, j, k)] = Ai[b, k, j, i + 1]
                if j > 0: Ad[c, idx(i, j - 1, k)] = Aj[b, k, j, i]
                if j < m - 1: Ad[c, idx(i, j + 1, k)] = Aj[b, k, j + 1, i]
                if k > 0: Ad[c, idx(i, j, k - 1)] = Ak[b, k, j, i]
                if k < m - 1: Ad[c, idx(i, j, k + 1)] = Ak[b, k + 1, j, i]
    mc = m // 2
    P = np.zeros((n, mc ** 3))
    for k in range(m):
        for j in range(m):
            for i in range(m):
                P[idx(i, j, k), ((k // 2) * mc + j // 2) * mc + i // 2] = 1.0
    G = P.T @ Ad @ P
    assert np.allclose(np.diag(G), C[0][b].reshape(-1), rtol=1e-13, atol=0)
    # one coupling per direction
    assert np.isclose(G[0, 1], C[1][b, 0, 0, 1], rtol=1e-13)
    assert np.isclose(G[0, mc], C[2][b, 0, 1, 0], rtol=1e-13)
    assert np.isclose(G[0, mc * mc], C[3][b, 1, 0, 0], rtol=1e-13)


def _padded(sv, x):
    m = sv.m[0]
    xp = np.zeros((sv.nblocks, m + 2, m + 2, m + 2))
    xp[:, 1:-1, 1:-1, 1:-1] = x
    return xp


def _cpu_residual(sv, x):
    """||b - A x|| / ||b|| per problem with the oracle's halo fill and SpMV."""
    m = sv.m[0]
    idx, wx = sv.halo_map(0)
    xp = oracle.halo_fill(m, idx, wx, _padded(sv, x))
    y = oracle.spmv(m, sv.operator(0), xp)
    r = sv.rhs() - y
    first = sv.problem_blocks()
    out = []
    for q in range(sv.nproblems):
        sl = slice(first[q], first[q + 1])
        out.append(np.linalg.norm(r[sl]) / np.linalg.norm(sv.rhs()[sl]))
    return np.array(out)


@pytest.mark.gpu
def test_gpu_spmv_bit_identical_to_oracle():
    sv = S.Solver(S.pfss_spec(SIZES, device=0))
    rs = np.random.default_rng(3)
    x = rs.normal(size=(sv.nblocks,) + sv.m[::-1])
    y = sv.apply(x)
    m = sv.m[0]
    idx, wx = sv.halo_map(0)
    xp = oracle.halo_fill(m, idx, wx, _padded(sv, x))
    y0 = oracle.spmv(m, sv.operator(0), xp)
    assert np.array_equal(y, y0)


@pytest.mark.gpu
def test_gpu_batched_pfss_converges_and_mg_helps():
    sizes = [(24, 45), (40, 80), (33, 60), (64, 100)]
    sv = S.Solver(S.pfss_spec(sizes, device=0))
    rep = sv.solve(tol=1e-10, max_iter=2000, precond=S.PRECOND_MG)
    assert rep["converged"] == 1 and rep["rel_residual"] <= 1e-10
    res = _cpu_residual(sv, sv.solution())
    assert (res <= 1.05e-10).all(), res
    rep0 = sv.solve(tol=1e-10, max_iter=4000, precond=S.PRECOND_NONE, check=False)
    print("pfss MG:", rep, "plain CG:", rep0)
    assert rep["iterations"] < rep0["iterations"]


@pytest.mark.gpu
def test_gpu_conduction_small_converges():
    sv = S.Solver(S.conduction_spec(nr=32, nt=32, np_=96, block=16, device=0))
    rep = sv.solve(tol=1e-8, max_iter=500, precond=S.PRECOND_MG)
    res = _cpu_residual(sv, sv.solution())
    print("conduction small:", rep, res)
    assert rep["converged"] == 1 and (res <= 1.05e-8).all()


def _assemble_csr(sv):
    """The level-0 operator as an explicit sparse matrix over interior cells:
    face coefficients (3_5/ModLinearSolver.f90:43-50) with each ghost
    neighbour replaced by its trilinear interpolation weights onto the source
    block's interior (the halo map); physical-boundary ghosts carry no halo
    entry and stay zero, as on the GPU."""
    import scipy.sparse as sp
    m = sv.m[0]
    nb = sv.nblocks
    Aii, Ai, Aj, Ak = sv.operator(0)
    idx, wx = sv.halo_map(0)
    halo = {(int(e[0]), int(e[1]), int(e[2]), int(e[3])): q for q, e in enumerate(idx)}
    col = lambda b, i, j, k: ((b * m + (k - 1)) * m + (j - 1)) * m + (i - 1)
    rows, cols, vals = [], [], []
    for b in range(nb):
        for k in range(1, m + 1):
            for j in range(1, m + 1):
                for i in range(1, m + 1):
                    r = col(b, i, j, k)
                    rows.append(r); cols.append(r); vals.append(Aii[b, k - 1, j - 1, i - 1])
                    nbrs = ((Ai[b, k - 1, j - 1, i - 1], (i - 1, j, k)), (Ai[b, k - 1, j - 1, i], (i + 1, j, k)),
                            (Aj[b, k - 1, j - 1, i - 1], (i, j - 1, k)), (Aj[b, k - 1, j, i - 1], (i, j + 1, k)),
                            (Ak[b, k - 1, j - 1, i - 1], (i, j, k - 1)), (Ak[b, k, j - 1, i - 1], (i, j, k + 1)))
                    for c, (a1, a2, a3) in nbrs:
                        if c == 0.0:
                            continue
                        if 1 <= a1 <= m and 1 <= a2 <= m and 1 <= a3 <= m:
                            rows.append(r); cols.append(col(b, a1, a2, a3)); vals.append(c)
                            continue
                        q = halo.get((b, a1, a2, a3))
                        if q is None:
                            continue
                        sb, i0, j0, k0 = (int(v) for v in idx[q, 4:8])
                        w = wx[q, :3]
                        for corner in range(8):
                            o = (corner & 1, (corner >> 1) & 1, corner >> 2)
                            f = 1.0
                            for d in range(3):
                                f *= w[d] if o[d] else 1.0 - w[d]
                            if f != 0.0:
                                rows.append(r); cols.append(col(sb, i0 + o[0], j0 + o[1], k0 + o[2])); vals.append(c * f)
    n = nb * m ** 3
    return sp.csr_matrix((vals, (rows, cols)), shape=(n, n))


@pytest.mark.gpu
def test_gpu_pfss_solution_matches_cpu_direct_solve():
    """FP64 error of a GPU PFSS solve against a CPU direct (sparse LU) solve of
    the same operator: the assembled matrix reproduces the oracle's SpMV, and
    the GPU solution (true residual <= 1e-11) agrees within the conditioning
    of the problem."""
    import scipy.sparse.linalg as spl
    sv = S.Solver(S.pfss_spec([(16, 24)], device=0))
    A = _assemble_csr(sv)
    rs = np.random.default_rng(17)
    x = rs.normal(size=(sv.nblocks,) + sv.m[::-1])
    m = sv.m[0]
    idx, wx = sv.halo_map(0)
    xp = np.zeros((sv.nblocks, m + 2, m + 2, m + 2))
    xp[:, 1:-1, 1:-1, 1:-1] = x
    y0 = oracle.spmv(m, sv.operator(0), oracle.halo_fill(m, idx, wx, xp)).reshape(-1)
    assert np.allclose(A @ x.reshape(-1), y0, rtol=1e-12, atol=1e-12 * np.abs(y0).max())
    b = sv.rhs().reshape(-1)
    x_ref = spl.spsolve(A.tocsc(), b)
    assert np.linalg.norm(A @ x_ref - b) <= 1e-12 * np.linalg.norm(b)
    rep = sv.solve(tol=1e-11, max_iter=1000, precond=S.PRECOND_MG)
    xg = sv.solution().reshape(-1)
    err = np.linalg.norm(xg - x_ref) / np.linalg.norm(x_ref)
    print("pfss 16x24: GPU vs CPU direct solve relative error", err, rep)
    assert err <= 1e-6


@pytest.mark.gpu
def test_gpu_large_pfss_batch_converges_every_problem():
    """32 PFSS problems of the benchmark's random sizes (72,744 blocks, 37M
    cells): every problem reaches 1e-10 on its FP64 true residual. Large
    arrays are where an upload not ordered after its buffer's zero-fill lost
    the operator; this size failed before that was fixed."""
    sizes = S.random_pfss_sizes(64, seed=5000)[:32]
    sv = S.Solver(S.pfss_spec(sizes, device=0))
    assert sv.nblocks > 65536
    rep = sv.solve(tol=1e-10, max_iter=200, precond=S.PRECOND_MG, check=False)
    rel = sv.problem_residuals()
    print("32-problem PFSS batch:", rep, "max FP64 residual %.3e" % rel.max())
    assert rep["converged"] == 1 and (rel <= 1.05e-10).all(), rel.max()
    sv.close()


@pytest.mark.gpu
def test_gpu_solve_reports_not_converged_on_its_fp64_residual():
    """Convergence is judged on the FP64 true residual only: a solve cut off
    by max_iter, or asked for a tolerance below what FP64 attains, returns
    FALCON_ERR_NOT_CONVERGED with converged = 0, and its reported residual is
    the FP64 ||b - A x|| / ||b|| of the returned solution."""
    import falcon_gb300 as fg
    sv = S.Solver(S.pfss_spec([(24, 45), (32, 60)], device=0))
    with pytest.raises(fg.FalconError) as e:
        sv.solve(tol=1e-10, max_iter=3)
    assert e.value.code == fg.ERR_NOT_CONVERGED
    rep = sv.solve(tol=1e-10, max_iter=3, check=False)
    rel = sv.problem_residuals()
    assert rep["converged"] == 0 and rep["iterations"] == 3
    assert rep["rel_residual"] > 1e-10
    assert abs(rep["rel_residual"] - rel.max()) <= 1e-9 * rel.max()
    # below FP64's attainable accuracy: stops at the floor, not converged
    rep = sv.solve(tol=1e-19, max_iter=400, check=False)
    rel = sv.problem_residuals()
    print("tol 1e-19:", rep, rel)
    assert rep["converged"] == 0 and rep["floor_residual"] > 0
    assert rep["rel_residual"] < 1e-12 and rel.max() < 1e-12
    # and a reachable tolerance converges, judged on the same FP64 residual
    rep = sv.solve(tol=1e-11, max_iter=400)
    assert rep["converged"] == 1 and (sv.problem_residuals() <= 1e-11).all()


def test_cpu_reference_mg_solve_matches_direct_solve():
    """The oracle's FP64 MG-PCG (the CPU reference solve for the batched PFSS
    error check) agrees with a sparse direct solve of the same operator."""
    import scipy.sparse.linalg as spl
    sv = S.Solver(S.pfss_spec([(16, 24), (16, 30)], device=-1))
    A = _assemble_csr(sv)
    b = sv.rhs()
    x_ref = spl.spsolve(A.tocsc(), b.reshape(-1)).reshape(b.shape)
    ops = [sv.operator(l) for l in range(sv.nlevels)]
    halos = [sv.halo_map(l) for l in range(sv.nlevels)]
    first = sv.problem_blocks()
    bprob = np.repeat(np.arange(sv.nproblems), np.diff(first))
    x, it, rel = oracle.mg_solve(ops, halos, bprob, sv.nproblems, b, np.zeros_like(b), 1e-13, 300, (1, 1, 32))
    print("cpu mg-pcg:", it, rel)
    assert (rel <= 1e-13).all()
    for q in range(sv.nproblems):
        sl = slice(first[q], first[q + 1])
        assert np.linalg.norm(x[sl] - x_ref[sl]) <= 1e-9 * np.linalg.norm(x_ref[sl])


def _vcycle_solver():
    return S.Solver(S.pfss_spec([(24, 45), (16, 30)], device=0))


@pytest.mark.gpu
@pytest.mark.parametrize("level", [0, 1])
def test_gpu_restriction_and_prolongation_bit_identical_to_oracle(level):
    """k_restrict and k_prolong_add against the restatements of
    ModMath_rebin_3D_factor2 (sum order of 3_6/ModMath.f90:360-367, no /8)
    and ModMath_prolongate_3D_factor2 (3_6/ModMath.f90:370-384): FP32, bit for bit."""
    sv = _vcycle_solver()
    rs = np.random.default_rng(40 + level)
    shp = lambda l: (sv.nblocks,) + sv.level_shape(l)[::-1]
    res = rs.normal(size=shp(level)).astype(np.float32)
    assert np.array_equal(sv.vcycle_op(S.VCYCLE_RESTRICT, level, res), oracle.mg_restrict(res))
    zc = rs.normal(size=shp(level + 1)).astype(np.float32)
    zf = rs.normal(size=shp(level)).astype(np.float32)
    assert np.array_equal(sv.vcycle_op(S.VCYCLE_PROLONG_ADD, level, zc, zf), oracle.mg_prolong_add(zc, zf))


@pytest.mark.gpu
@pytest.mark.parametrize("level", [0, 1, 2])
def test_gpu_smoother_half_sweeps_and_residual_match_oracle(level):
    """One red-black half sweep of each colour (k_rbgs) and the FP32 residual
    (k_resid32) against the oracle's FP32 restatement of the Jacobi cell
    update of ModMultigrid_Jacobi_Mz_r (3_5/ModMultigrid.f90:316-324). Cells
    of the other colour are untouched bit for bit; updated cells agree to
    FP32 rounding (the GPU sweep uses explicit FMAs and a fast division, its
    halo is interpolated in FP32, the oracle's in FP64): tolerance 2e-5 of the
    largest |z|."""
    sv = _vcycle_solver()
    rs = np.random.default_rng(50 + level)
    shp = (sv.nblocks,) + sv.level_shape(level)[::-1]
    m = shp[1]
    A = sv.operator(level)
    r = rs.normal(size=shp).astype(np.float32)
    z = rs.normal(size=shp).astype(np.float32)
    idx, wx = sv.halo_map(level)
    zp = np.zeros((sv.nblocks, m + 2, m + 2, m + 2))
    zp[:, 1:-1, 1:-1, 1:-1] = z
    zp = oracle.halo_fill(m, idx, wx, zp).astype(np.float32)
    kk, jj, ii = np.meshgrid(np.arange(1, m + 1), np.arange(1, m + 1), np.arange(1, m + 1), indexing="ij")
    for colour, op in ((0, S.VCYCLE_SMOOTH_RED), (1, S.VCYCLE_SMOOTH_BLACK)):
        g = sv.vcycle_op(op, level, r, z)
        o = oracle.mg_rbgs(A, r, zp, colour)[:, 1:-1, 1:-1, 1:-1]
        upd = ((ii + jj + kk) & 1) == colour
        assert np.array_equal(g[:, ~upd], z[:, ~upd])
        err = np.abs(g[:, upd] - o[:, upd]).max() / np.abs(o).max()
        print("level %d colour %d: max rel diff %.2e" % (level, colour, err))
        assert err <= 2e-5
    y = oracle.spmv(m, A, zp.astype(np.float64))
    g = sv.vcycle_op(S.VCYCLE_RESIDUAL, level, r, z)
    ref = r.astype(np.float64) - y
    assert np.abs(g - ref).max() <= 2e-5 * np.abs(ref).max()


@pytest.mark.gpu
def test_gpu_pfss_batch64_error_per_solve_against_cpu_fp64_solve():
    """The batched PFSS workload: 64 problems of the seeded random sizes
    (nr 24..64, ntheta 45..180; 70.8M cells) solved together on the GPU to
    1e-10, then each problem's FP64 error against a CPU FP64 solve. The CPU
    reference is the oracle's FP64 MG-PCG on the same operator, started from
    the GPU solution and run until each problem's FP64 true residual is
    <= 1e-13: its correction is A^-1 r_gpu, the GPU solution's error, computed
    on the CPU in FP64. Per problem: ||x_gpu - x_cpu|| / ||x_cpu||."""
    import time
    sizes = S.random_pfss_sizes(64, seed=5000)
    sv = S.Solver(S.pfss_spec(sizes, device=0))
    rep = sv.solve(tol=1e-10, max_iter=300)
    assert rep["converged"] == 1
    x_gpu = sv.solution()
    rel_gpu = sv.problem_residuals()
    t0 = time.time()
    ops = [sv.operator(l) for l in range(sv.nlevels)]
    halos = [sv.halo_map(l) for l in range(sv.nlevels)]
    first = sv.problem_blocks()
    bprob = np.repeat(np.arange(sv.nproblems), np.diff(first))
    x_cpu, it, rel_cpu = oracle.mg_solve(ops, halos, bprob, sv.nproblems, sv.rhs(), x_gpu, 1e-13, 100, (1, 1, 32))
    err = np.array([np.linalg.norm(x_gpu[first[q]:first[q + 1]] - x_cpu[first[q]:first[q + 1]]) /
                    np.linalg.norm(x_cpu[first[q]:first[q + 1]]) for q in range(sv.nproblems)])
    print("pfss batch64: GPU %s; CPU reference %d iterations in %.1f s, max residual %.2e" %
          (rep, it, time.time() - t0, rel_cpu.max()))
    print("per-problem FP64 error vs the CPU solve: max %.3e median %.3e min %.3e" %
          (err.max(), np.median(err), err.min()))
    print("per-problem GPU FP64 residual: max %.3e median %.3e" % (rel_gpu.max(), np.median(rel_gpu)))
    assert (rel_gpu <= 1e-10).all()
    assert (rel_cpu <= 1e-13).all()
    assert err.max() <= 1e-7, err


@pytest.mark.gpu
def test_gpu_solver_tile_shapes_and_autotuner():
    """The autotuner picks one of its candidate tiles at the first solve, and
    every tile shape (cells and threads per CTA of the cell kernels) solves the
    same batch to the same FP64 tolerance; each inner solve is one graph
    launch with its loop on the device, so the iteration count does not
    depend on the shape either."""
    sv = S.Solver(S.pfss_spec([(24, 45), (40, 80)], device=0))
    rep0 = sv.solve(tol=1e-10, max_iter=400)
    t = sv.tuning()
    print("tuned:", t, rep0)
    assert t["tuned"] and t["cells_per_cta"] in (512, 1024, 2048, 4096) and t["threads_per_cta"] in (128, 256, 512)
    x0 = sv.solution()
    for chunk, tpb in ((512, 128), (4096, 512), (1024, 256)):
        sv.set_tile(chunk, tpb)
        rep = sv.solve(tol=1e-10, max_iter=400)
        assert rep["converged"] == 1 and (sv.problem_residuals() <= 1e-10).all()
        assert abs(rep["iterations"] - rep0["iterations"]) <= 2
        assert np.abs(sv.solution() - x0).max() <= 1e-8 * np.abs(x0).max()
    with pytest.raises(Exception):
        sv.set_tile(100, 128)
