"""The configurations at their full sizes on the GPU, each bounded to seconds.

c0  mcmod_1d, P = 32, 11 lambda points, the full 20,000 steps: the plain
    (reference step order) and fused FP64 forms against the CPU oracle's
    reference-order run of the same rings and seeds (pimd_par.f90:399-424).
c1  mcmod_2dtest, P = 128, the full batch of 1,024 x 16 = 16,384 rings:
    mixed precision (persistent tcgen05 step kernel) against the FP64 form,
    same seeds, 600 steps: the splitting within the metric's 1 % and every
    lambda point's mean far inside its statistical error.
c2  9-atom surface, P = 256, the full 256 x 12 = 3,072 rings: the persistent
    folded tcgen05 step against FP64, same seeds, 300 steps, the same checks.
c3  instanton, N = 512 beads, 27 dofs (13,824-dim Hessian): the batched GPU
    L-BFGS at the lowest and highest beta against scipy L-BFGS-B (the
    algorithm of the reference's lbfgsb.f) on the oracle's action to 1e-8,
    and the log-determinants against LAPACK dsbevd on the oracle's band.
"""
import os

import numpy as np
import pytest

import pgconfigs

pytestmark = pytest.mark.gpu


def test_c0_full_run_fp64_forms_match_the_oracle(pg, oracle):
    import drivers
    c = pgconfigs.load("c0")
    plain = drivers.run_ti(c, precision=pg.PG_FP64, form=pg.PG_FORM_PLAIN)
    fused = drivers.run_ti(c, precision=pg.PG_FP64, form=pg.PG_FORM_FUSED)
    ti = pgconfigs.TiInputs(c, gauleg=oracle.gauleg)
    pes = oracle.Pes(c["pes_id"], c["ndim"], c["natom"], c["params"], V0=c["V0"])
    mass = np.array(c["mass"])
    prm = oracle.TiParams(ti.P, c["beta"], c["dt"], tau=c["tau"], gamma=c["gamma"], thermostat=2,
                          nm_resident=False, imin=c["imin"], init_sigma=c["init_sigma"])
    nd, P = ti.nd, ti.P
    x = np.zeros(ti.nrings * nd * P)
    p = np.zeros(ti.nrings * nd * P)
    for r in range(ti.nrings):
        li = ti.ring_lambda[r]
        xx, pp = oracle.ring_init(pes, mass, prm, ti.xref[li], int(ti.ring_seed[r]), int(ti.ring_stream[r]),
                                  a=ti.a, b=ti.b[li])
        x[r * nd * P:(r + 1) * nd * P] = xx
        p[r * nd * P:(r + 1) * nd * P] = pp
    rr = oracle.ti_run_batch(pes, mass, prm, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl,
                             ti.xref, c["nmc"], os.cpu_count() or 1, x, p)
    integ = np.array([rr[i].dhdr_sum / rr[i].nsamples / ti.betan ** 2 for i in range(ti.nrings)])
    dA, _, _ = oracle.ti_assemble(ti.w, integ, 1, ti.betan)
    assert plain["nmc"] == c["nmc"] == 20000
    assert abs(plain["dA"] - dA) <= 1e-12 * abs(dA)
    assert abs(fused["dA"] - dA) <= 1e-10 * abs(dA)  # NM-resident order: same physics, other rounding
    np.testing.assert_allclose(plain["integrand_mean"], integ, rtol=1e-11, atol=1e-13 * np.max(np.abs(integ)))


@pytest.mark.parametrize("name,nmc,imin", [("c1", 600, 200), ("c2", 300, 100)])
def test_full_batch_mixed_precision_tracks_fp64(pg, name, nmc, imin):
    """The metric's precision condition on the whole batch: mixed precision
    (FP32 forces and state, split-BF16 tcgen05 NM transform, FP64 estimator)
    against the FP64 form, same rings and Philox streams."""
    import drivers
    c = dict(pgconfigs.load(name), imin=imin)
    mixed = drivers.run_ti(c, precision=pg.PG_MIXED, form=pg.PG_FORM_AUTO, nmc=nmc, chunk=nmc)
    fp64 = drivers.run_ti(c, precision=pg.PG_FP64, form=pg.PG_FORM_FUSED, nmc=nmc, chunk=nmc)
    assert mixed["nrings"] == fp64["nrings"] == c["nrep"] * c["nintegral"]
    assert mixed["form"] == pg.PG_FORM_TENSOR
    assert mixed["nan_rings"] == 0 and fp64["nan_rings"] == 0
    rel = abs(mixed["delta"] / fp64["delta"] - 1.0)
    assert rel <= 0.01, rel
    # every lambda point: the precision difference is far inside the statistical error
    var = np.asarray(fp64["integrand_var"])
    se = np.sqrt(np.maximum(var, 0.0) / c["nrep"])
    diff = np.abs(np.asarray(mixed["integrand_mean"]) - np.asarray(fp64["integrand_mean"]))
    assert np.all(diff <= 0.1 * se + 1e-12 * np.abs(np.asarray(fp64["integrand_mean"]))), (diff / se)
    assert abs(mixed["ln_qratio"] - fp64["ln_qratio"]) <= 0.1 * fp64["ln_qratio_stderr"]


def test_c3_full_size_instanton_matches_scipy_and_dsbevd(ctx, pg, oracle):
    c = pgconfigs.load("c3")
    ctx.set_system(c["ndim"], c["natom"], c["mass"], c["pes_id"], c["params"], c["V0"])
    pes = oracle.Pes(c["pes_id"], c["ndim"], c["natom"], c["params"], V0=c["V0"])
    mass = np.array(c["mass"], dtype=float)
    w1, w2 = np.array(c["well1"]), np.array(c["well2"])
    N, nd = 512, len(w1)
    assert c["N"] == N and N * nd == 13824
    betas = np.array(c["betas"])[[0, -1]]
    betans = betas / N
    k = np.arange(1, N + 1)
    x0 = np.concatenate([((N - k) * w1[d] + (k - 1) * w2[d]) / (N - 1) for d in range(nd)])
    x, UM, it, st = ctx.instanton_optimize(N, np.tile(x0, 2), w1, np.tile(w2, 2), betans, m=10, factr=1e2,
                                           pgtol=1e-8, maxiter=200000)
    assert np.all(st == 0), (st, it)
    n = N * nd
    for j in range(2):
        _, fo, _ = oracle.instanton_lbfgs(pes, mass, N, betans[j], x0, w1, w2, m=10, factr=1e2, pgtol=1e-8,
                                          maxiter=200000)
        assert abs(UM[j] - fo) <= 1e-8 * abs(fo), (j, UM[j], fo)
    # log-determinants at the highest beta's instanton and at the well (13,824 x 13,824, band 28)
    xj = x[n:]
    ld, emin, nsk = ctx.instanton_logdet(N, xj, betans[1:], singlewell=False, skip_lowest=True)
    ref, nneg, w0 = oracle.logdet_band(oracle.UMhessian(pes, mass, N, betans[1], xj), True)
    assert abs(ld[0] - ref) <= 1e-9 * abs(ref), (ld[0], ref)
    assert nsk[0] == nneg + 1
    xh = np.repeat(w1, N)
    ld0, _, _ = ctx.instanton_logdet(N, xh, betans[1:], singlewell=True, skip_lowest=False)
    ref0, _, _ = oracle.logdet_band(oracle.UMhessian(pes, mass, N, betans[1], xh, singlewell=True), False)
    assert abs(ld0[0] - ref0) <= 1e-9 * abs(ref0), (ld0[0], ref0)
