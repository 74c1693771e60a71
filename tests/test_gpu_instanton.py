"""GPU parity of the ring-polymer instanton path (action, adjoint gradient,
Hessian band, log-determinant, L-BFGS) against the CPU oracle and LAPACK dsbevd."""
import numpy as np
import pytest

import pgconfigs

pytestmark = pytest.mark.gpu


def _system(ctx, oracle, name):
    c = pgconfigs.load(name)
    ctx.set_system(c["ndim"], c["natom"], c["mass"], c["pes_id"], c["params"], c["V0"])
    pes = oracle.Pes(c["pes_id"], c["ndim"], c["natom"], c["params"], V0=c["V0"])
    return c, pes, np.array(c["mass"], dtype=float)


def _linear_path(w1, w2, N, noise=0.0, seed=0):
    """rpi_ser.f90:157-163: bead k at ((N-k) w1 + (k-1) w2)/(N-1), k = 1..N."""
    k = np.arange(1, N + 1)
    nd = len(w1)
    x = np.concatenate([((N - k) * w1[d] + (k - 1) * w2[d]) / (N - 1) for d in range(nd)])
    if noise:
        x = x + noise * np.random.RandomState(seed).randn(x.size)
    return x


@pytest.mark.parametrize("name", ["c1", "c3", "c0"])
def test_action_and_gradient_match_oracle(ctx, pg, oracle, name):
    c, pes, mass = _system(ctx, oracle, name)
    w1, w2 = np.array(c["well1"]), np.array(c["well2"])
    N = 24
    betans = np.array([3.0, 11.0, 40.0])
    xs = np.concatenate([_linear_path(w1, w2, N, 0.02, s) for s in range(3)])
    b = np.tile(w2, 3)
    UM, g = ctx.instanton_fg(N, xs, w1, b, betans)
    n = N * len(w1)
    for k in range(3):
        xk = xs[k * n:(k + 1) * n]
        uo, go = oracle.UMforceenergy(pes, mass, N, betans[k], xk, w1, w2)
        assert abs(UM[k] - uo) <= 1e-12 * max(1.0, abs(uo))
        np.testing.assert_allclose(g[k * n:(k + 1) * n], go, rtol=1e-11, atol=1e-13)


def test_gradient_matches_finite_differences(ctx, pg, oracle):
    """The adjoint gradient against central differences of the GPU action (step 1e-5)."""
    c, pes, mass = _system(ctx, oracle, "c3")
    w1, w2 = np.array(c["well1"]), np.array(c["well2"])
    N = 8
    x = _linear_path(w1, w2, N, 0.05, 3)
    betan = 20.0
    _, g = ctx.instanton_fg(N, x, w1, w2, [betan])
    h = 1e-5
    idx = np.random.RandomState(0).choice(x.size, 40, replace=False)
    xs = []
    for i in idx:
        for sgn in (1, -1):
            xx = x.copy()
            xx[i] += sgn * h
            xs.append(xx)
    xs = np.concatenate(xs)
    U, _ = ctx.instanton_fg(N, xs, w1, np.tile(w2, len(idx) * 2), np.full(len(idx) * 2, betan))
    fd = (U[0::2] - U[1::2]) / (2 * h)
    np.testing.assert_allclose(g[idx], fd, rtol=1e-6, atol=1e-8)


@pytest.mark.parametrize("name,quirks,singlewell", [("c3", False, False), ("c3", True, False),
                                                    ("c3", False, True), ("c1", True, False),
                                                    ("c0", False, False)])
def test_um_hessian_band_matches_oracle(ctx, pg, oracle, name, quirks, singlewell):
    c, pes, mass = _system(ctx, oracle, name)
    w1, w2 = np.array(c["well1"]), np.array(c["well2"])
    N = 10
    x = _linear_path(w1, w2, N, 0.03, 1)
    band = ctx.um_hessian(N, 9.0, x, singlewell=singlewell, quirks=quirks)
    bo = oracle.UMhessian(pes, mass, N, 9.0, x, singlewell=singlewell, quirks=quirks)
    np.testing.assert_allclose(band, bo, rtol=1e-11, atol=1e-14)


def _oracle_logdet(oracle, pes, mass, N, betan, x, singlewell, skip, quirks=False):
    band = oracle.UMhessian(pes, mass, N, betan, x, singlewell=singlewell, quirks=quirks)
    return oracle.logdet_band(band, skip)


@pytest.mark.parametrize("name", ["c3", "c1"])
def test_logdet_matches_dsbevd(ctx, pg, oracle, name):
    c, pes, mass = _system(ctx, oracle, name)
    w1, w2 = np.array(c["well1"]), np.array(c["well2"])
    N = 24
    betans = np.array([4.0, 15.0])
    xs = np.concatenate([_linear_path(w1, w2, N, 0.01, s) for s in range(2)])
    for singlewell, skip in ((False, True), (True, False), (False, False)):
        ld, emin, nsk = ctx.instanton_logdet(N, xs, betans, singlewell=singlewell, skip_lowest=skip)
        n = N * len(w1)
        for k in range(2):
            ref, nneg, w0 = _oracle_logdet(oracle, pes, mass, N, betans[k], xs[k * n:(k + 1) * n], singlewell, skip)
            assert abs(ld[k] - ref) <= 1e-9 * max(1.0, abs(ref)), (singlewell, skip, ld[k], ref)
            assert abs(emin[k] - w0) <= 1e-7 * abs(w0) + 1e-14
            # eigenvalues left out of the sum: the lowest when skipped, and every eta^2 <= 0
            excluded = nneg + (1 if skip else 0)
            assert nsk[k] == excluded


def test_lbfgs_matches_scipy_lbfgsb(ctx, pg, oracle):
    """On-device L-BFGS reaches the same instanton action as scipy's L-BFGS-B (the
    algorithm the reference vendors), both started from the rpi_ser linear path."""
    c, pes, mass = _system(ctx, oracle, "c3")
    w1, w2 = np.array(c["well1"]), np.array(c["well2"])
    N = 16
    betas = np.array(c["betas"])[[0, -1]]
    betans = betas / N
    x0 = np.concatenate([_linear_path(w1, w2, N) for _ in range(2)])
    x, UM, it, st = ctx.instanton_optimize(N, x0, w1, np.tile(w2, 2), betans, m=10, factr=1e2, pgtol=1e-9,
                                           maxiter=200000)
    assert np.all(st == 0), (st, it)
    n = N * len(w1)
    for k in range(2):
        xo, fo, r = oracle.instanton_lbfgs(pes, mass, N, betans[k], x0[k * n:(k + 1) * n], w1, w2, m=10,
                                           factr=1e2, pgtol=1e-9, maxiter=200000)
        assert abs(UM[k] - fo) <= 1e-8 * abs(fo), (UM[k], fo)
        _, g = ctx.instanton_fg(N, x[k * n:(k + 1) * n], w1, w2, [betans[k]])
        assert np.max(np.abs(g)) < 1e-6


@pytest.mark.parametrize("name", ["c1", "c3", "c0"])
def test_free_ended_action_and_gradient_match_oracle_and_fd(ctx, pg, oracle, name):
    """fixedends = .false.: the action and gradient without the end-point springs
    (instantonmod.f90:35-44, 63-72, 115-124, 138) against the oracle to 1e-11 and
    against central differences of the GPU action (step 1e-5); the end points
    are not passed (NULL), as instanton(xtilde) passes none."""
    c, pes, mass = _system(ctx, oracle, name)
    w1, w2 = np.array(c["well1"]), np.array(c["well2"])
    N = 24
    betans = np.array([3.0, 11.0, 40.0])
    xs = np.concatenate([_linear_path(w1, w2, N, 0.02, s) for s in range(3)])
    n = N * len(w1)
    ctx.set_fixedends(False)
    try:
        UM, g = ctx.instanton_fg(N, xs, None, None, betans)
        for k in range(3):
            uo, go = oracle.UMforceenergy(pes, mass, N, betans[k], xs[k * n:(k + 1) * n], w1, w2, False)
            assert abs(UM[k] - uo) <= 1e-12 * max(1.0, abs(uo))
            np.testing.assert_allclose(g[k * n:(k + 1) * n], go, rtol=1e-11, atol=1e-13)
        h = 1e-5
        x = xs[:n]
        idx = np.random.RandomState(1).choice(n, min(n, 30), replace=False)
        # the end beads of every dof, where the free ends change the gradient
        idx = np.unique(np.concatenate([idx, np.arange(len(w1)) * N, np.arange(len(w1)) * N + N - 1]))
        pts = []
        for i in idx:
            for sgn in (1, -1):
                xx = x.copy()
                xx[i] += sgn * h
                pts.append(xx)
        U, _ = ctx.instanton_fg(N, np.concatenate(pts), None, None, np.full(len(pts), betans[0]))
        fd = (U[0::2] - U[1::2]) / (2 * h)
        np.testing.assert_allclose(g[idx], fd, rtol=1e-6, atol=1e-8)
    finally:
        ctx.set_fixedends(True)
    # back to fixed ends: the end springs are there again
    UMf, _ = ctx.instanton_fg(N, xs[:n], w1, w2, betans[:1])
    uo = oracle.UM(pes, mass, N, betans[0], xs[:n], w1, w2, True)
    assert abs(UMf[0] - uo) <= 1e-12 * max(1.0, abs(uo))


@pytest.mark.parametrize("name", ["c3", "c0"])
def test_free_ended_lbfgs_matches_scipy_lbfgsb(ctx, pg, oracle, name):
    """The free-ended instanton (instanton(xtilde), instantonmod.f90:724-762): the
    on-device L-BFGS reaches scipy L-BFGS-B's action on the oracle's free-ended
    UM to 1e-8, both started from the rpi_ser linear path."""
    c, pes, mass = _system(ctx, oracle, name)
    w1, w2 = np.array(c["well1"]), np.array(c["well2"])
    N = 16 if name == "c3" else 32
    betas = np.array(c["betas"])[[0, -1]] if "betas" in c else np.array([c["beta"], 0.5 * c["beta"]])
    betans = betas / N
    x0 = np.concatenate([_linear_path(w1, w2, N) for _ in range(2)])
    ctx.set_fixedends(False)
    try:
        x, UM, it, st = ctx.instanton_optimize(N, x0, None, None, betans, m=10, factr=1e2, pgtol=1e-9,
                                               maxiter=200000)
    finally:
        ctx.set_fixedends(True)
    assert np.all(st == 0), (st, it)
    n = N * len(w1)
    for k in range(2):
        xo, fo, r = oracle.instanton_lbfgs(pes, mass, N, betans[k], x0[k * n:(k + 1) * n], None, None, m=10,
                                           factr=1e2, pgtol=1e-9, maxiter=200000, fixedends=False)
        assert abs(UM[k] - fo) <= 1e-8 * abs(fo), (UM[k], fo)
        # the optimiser's value is the free-ended action of the path it returns
        uo = oracle.UM(pes, mass, N, betans[k], x[k * n:(k + 1) * n], w1, w2, False)
        assert abs(UM[k] - uo) <= 1e-12 * max(1.0, abs(uo))


def test_lbfgs_cluster_sizes_reach_the_same_instanton(ctx, pg, oracle):
    """The optimiser spread over a thread-block cluster of 1, 2, 4 or 8 CTAs per
    polymer (dot products reduced across the cluster through distributed shared
    memory): every cluster size converges, and the actions agree with each other
    and with scipy L-BFGS-B on the oracle's action to 1e-9 (the sums run in
    different orders, so the iterates differ at round-off)."""
    c, pes, mass = _system(ctx, oracle, "c3")
    w1, w2 = np.array(c["well1"]), np.array(c["well2"])
    N = 64
    betas = np.array(c["betas"])[[0, 15, -1]]
    betans = betas / N
    x0 = np.concatenate([_linear_path(w1, w2, N) for _ in range(3)])
    res = {}
    for cs in (1, 2, 4, 8, 0):
        x, UM, it, st = ctx.instanton_optimize(N, x0, w1, np.tile(w2, 3), betans, m=10, factr=1e2, pgtol=1e-9,
                                               maxiter=200000, cluster_ctas=cs)
        assert np.all(st == 0), (cs, st, it)
        res[cs] = UM
    n = N * len(w1)
    for k in range(3):
        _, fo, _ = oracle.instanton_lbfgs(pes, mass, N, betans[k], x0[k * n:(k + 1) * n], w1, w2, m=10, factr=1e2,
                                          pgtol=1e-9, maxiter=200000)
        for cs, UM in res.items():
            assert abs(UM[k] - fo) <= 1e-9 * abs(fo), (cs, k, UM[k], fo)
    with pytest.raises(pg.PgError):
        ctx.instanton_optimize(N, x0, w1, np.tile(w2, 3), betans, cluster_ctas=3)
