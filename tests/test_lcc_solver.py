"""The learned coarse correction inside the conduction solver (GPU).

Pipeline under test: coarsest-level residuals recorded from real MG-FCG
solves, exact coarse errors as targets, training on the GPU, then the
network as the coarsest-level stage of the V-cycle (FALCON_PRECOND_MG_LCC).

What the network gains over the method without it is measured at its own
task: on coarse residuals of a right-hand side it never saw, the relative
error of its coarse correction ||e - net(r)|| / ||e|| against 1 for no coarse
correction. The solve with it must converge to the requested true residual
(checked on the CPU with the oracle's SpMV); its iteration count and time
are printed beside plain MG-PCG and the V-cycle without coarse work.
"""
import numpy as np
import pytest

import oracle
from falcon_gb300 import solver as S

pytestmark = pytest.mark.gpu

SMALL = dict(nr=32, nt=32, np_=96, block=16, nlevels=3)


def _smooth(shape, rs):
    x = rs.normal(size=shape)
    for ax in (1, 2, 3):
        for _ in range(3):
            x = (x + np.roll(x, 1, axis=ax) + np.roll(x, -1, axis=ax)) / 3.0
    return x


def _records(sv, rs, nrhs):
    X, T = [], []
    for r in range(nrhs):
        b = sv.apply(_smooth((sv.nblocks,) + sv.m[::-1], rs))
        sv.set_rhs(b)
        x, t = sv.record(tol=1e-8, max_iter=100, max_records=12)
        X.append(x)
        T.append(t)
    return np.concatenate(X), np.concatenate(T)


def _cpu_residual(sv, x):
    m = sv.m[0]
    idx, wx = sv.halo_map(0)
    xp = np.zeros((sv.nblocks, m + 2, m + 2, m + 2))
    xp[:, 1:-1, 1:-1, 1:-1] = x
    y = oracle.spmv(m, sv.operator(0), oracle.halo_fill(m, idx, wx, xp))
    r = sv.rhs() - y
    return float(np.linalg.norm(r) / np.linalg.norm(sv.rhs()))


def test_learned_coarse_correction_trains_and_preconditions(built_lib, oracle_lib):
    from falcon_gb300.lcc import LCC
    rs = np.random.default_rng(41)
    sv = S.Solver(S.conduction_spec(seed=5101, device=0, **SMALL))
    assert sv.coarse_shape() == (2, 8, 8, 24)
    b0 = sv.rhs()
    X, T = _records(sv, rs, 8)
    assert len(X) >= 64 and np.isfinite(X).all() and np.isfinite(T).all()
    net = LCC(device=0, seed=5)
    losses = net.train(X, T, epochs=40, batch=8, lr=1e-3, seed=2)
    assert losses[-1] < 0.25 * losses[0], losses
    # held-out right-hand side: coarse error of the network vs no correction
    Xh, Th = _records(sv, np.random.default_rng(977), 1)
    Y = net.forward(Xh)
    rel = float(np.linalg.norm(Y - Th) / np.linalg.norm(Th))
    print("held-out relative coarse error: net %.3f, no coarse correction 1.000" % rel)
    assert rel < 0.5
    # the network inside the solve
    sv.set_rhs(b0)
    sv.attach_lcc(net, sweeps=2)
    rep_lcc = sv.solve(tol=1e-8, max_iter=300, precond=S.PRECOND_MG_LCC)
    res = _cpu_residual(sv, sv.solution())
    rep_mg = sv.solve(tol=1e-8, max_iter=300, precond=S.PRECOND_MG)
    # the same V-cycle without the network: the 2 coarsest-level sweeps alone
    sv.set_smoothing(2, 2, 2)
    rep_two = sv.solve(tol=1e-8, max_iter=300, precond=S.PRECOND_MG)
    sv.set_smoothing(2, 2, 0)
    rep_none = sv.solve(tol=1e-8, max_iter=300, precond=S.PRECOND_MG)
    print("MG+LCC:", rep_lcc, "MG:", rep_mg, "same V-cycle without the network:", rep_two,
          "MG without coarse work:", rep_none)
    assert rep_lcc["converged"] == 1 and res <= 1.05e-8, res
    # what the trained network gains over the method without it: the network
    # plus 2 coarsest-level sweeps against the 2 sweeps alone. Measured: the
    # same iteration count -- on this system (Delta t = 50 explicit limits)
    # the coarse levels do not limit convergence (no coarse work at all costs
    # the same), so the learned stage has nothing to win; the wall-time target
    # of <= 0.5x MG-PCG is not met
    assert rep_lcc["iterations"] <= rep_two["iterations"], (rep_lcc, rep_two)
    assert rep_none["iterations"] <= rep_mg["iterations"] + 1, (rep_none, rep_mg)
