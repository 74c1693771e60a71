"""Faults made on the host, never on the GPU: a NaN written into one ring's
start positions.  The reference stops the whole program on a NaN
(verletmodule.f90:533-536, 577-580); here the ring is flagged
(PG_RING_NAN), stops, and is left out of its lambda point's mean, while every
other ring runs as if the faulty one were absent.

CPU: the oracle's ring propagation, and the namelist driver through the
oracle-backed stand-in (tests/standin).  GPU: the FP64 fused and plain forms
through the C-ABI (NaN arithmetic only: nothing faults or waits)."""
import os
import re
import subprocess

import numpy as np
import pytest

import pgconfigs


def test_oracle_flags_and_stops_a_nan_ring(oracle):
    c = pgconfigs.load("c0")
    ti = pgconfigs.TiInputs(c, nrep=2, nintegral=2, gauleg=oracle.gauleg)
    pes = oracle.Pes(c["pes_id"], 1, 1, c["params"])
    prm = oracle.TiParams(ti.P, c["beta"], c["dt"], tau=c["tau"], gamma=c["gamma"], thermostat=2,
                          nm_resident=True, imin=5, init_sigma=c["init_sigma"])
    out = []
    for bad in (False, True):
        x, p = oracle.ring_init(pes, c["mass"], prm, ti.xref[0], 0, 0, a=ti.a, b=ti.b[0])
        if bad:
            x[3] = np.nan
        res = oracle.ring_propagate(pes, c["mass"], prm, ti.a, ti.b[0], ti.dbdl[0], ti.xref[0], 0, 0, 0, 50, x, p)
        out.append(res)
    assert out[0].status == 0 and out[0].nsamples == 45
    assert out[1].status == 1 and out[1].nsamples == 0  # stopped in its first step, before any sample


def _write_inputs(d, c):
    (d / "masses.dat").write_text("H %.17g\n" % c["mass"][0])
    (d / "well1.dat").write_text("%.17g\n" % c["well1"][0])
    (d / "well2.dat").write_text("%.17g\n" % c["well2"][0])
    (d / "pes.dat").write_text("\n".join("%.17g" % v for v in c["params"]) + "\n")


def test_driver_leaves_a_nan_ring_out(oracle, tmp_path):
    """pimd_ti.cpp through the stand-in with a NaN injected into ring 4 (lambda
    point 1, replica 1 of 3): the run completes, reports one ring with a NaN,
    and Delta A is the oracle's over the other rings."""
    import standin
    exe = standin.build_driver("pimd_ti", tmp_path)
    c = dict(pgconfigs.load("c0"), imin=20, P=16, nintegral=3)
    _write_inputs(tmp_path, c)
    text = ("&MCDATA n=16, beta=%.17g, NMC=120, dt=%.17g, imin=20, tau=%.17g, gamma=%.17g, nintegral=3,\n"
            " nrep=3, thermostat=2, ndim=1, natom=1, readpath=F, pes='1d', pes_params='pes.dat',\n"
            " precision='fp64', form='fused', init='well', init_sigma=%.17g, seed=0 /\n"
            % (c["beta"], c["dt"], c["tau"], c["gamma"], c["init_sigma"]))
    r = subprocess.run([exe], input=text, capture_output=True, text=True, cwd=str(tmp_path), timeout=300,
                       env=dict(os.environ, PG_STANDIN_NAN_RING="4"))
    assert r.returncode == 0, r.stderr
    assert re.search(r"rings with a NaN:\s*1\b", r.stdout)
    dA = float(re.search(r"final Delta A=\s*(\S+)", r.stdout).group(1))
    ti = pgconfigs.TiInputs(dict(c, nrep=3, seeds=[0, 1, 2]), gauleg=oracle.gauleg)
    pes = oracle.Pes(c["pes_id"], 1, 1, c["params"])
    prm = oracle.TiParams(ti.P, c["beta"], c["dt"], tau=c["tau"], gamma=c["gamma"], thermostat=2,
                          nm_resident=True, imin=20, init_sigma=c["init_sigma"])
    ints = {}
    for ring in range(ti.nrings):
        if ring == 4:
            continue
        li = int(ti.ring_lambda[ring])
        x, p = oracle.ring_init(pes, c["mass"], prm, ti.xref[li], int(ti.ring_seed[ring]),
                                int(ti.ring_stream[ring]), a=ti.a, b=ti.b[li])
        res = oracle.ring_propagate(pes, c["mass"], prm, ti.a, ti.b[li], ti.dbdl[li], ti.xref[li],
                                    int(ti.ring_seed[ring]), int(ti.ring_stream[ring]), 0, 120, x, p)
        ints.setdefault(li, []).append(res.dhdr_sum / res.nsamples / ti.betan ** 2)
    assert len(ints[1]) == 2
    ref = sum(ti.w[li] * np.mean(v) for li, v in ints.items())
    assert dA == pytest.approx(ref, rel=1e-12)


def test_driver_stops_when_a_lambda_point_loses_every_ring(oracle, tmp_path):
    """Every ring of lambda point 2 (rings 3, 4, 5) starts from a NaN: that point
    has no estimate, so the driver stops with a message naming it instead of
    integrating a zero (exit status 3)."""
    import standin
    exe = standin.build_driver("pimd_ti", tmp_path)
    c = dict(pgconfigs.load("c0"), imin=20, P=16, nintegral=3)
    _write_inputs(tmp_path, c)
    text = ("&MCDATA n=16, beta=%.17g, NMC=60, dt=%.17g, imin=20, tau=%.17g, gamma=%.17g, nintegral=3,\n"
            " nrep=3, thermostat=2, ndim=1, natom=1, readpath=F, pes='1d', pes_params='pes.dat',\n"
            " precision='fp64', form='fused', init='well', init_sigma=%.17g, seed=0 /\n"
            % (c["beta"], c["dt"], c["tau"], c["gamma"], c["init_sigma"]))
    r = subprocess.run([exe], input=text, capture_output=True, text=True, cwd=str(tmp_path), timeout=300,
                       env=dict(os.environ, PG_STANDIN_NAN_RING="3,4,5"))
    assert r.returncode == 3, (r.returncode, r.stderr)
    assert "integration point 2 has no valid ring" in r.stderr
    assert "final Delta A" not in r.stdout


def test_python_driver_error_bar_uses_the_rings_each_point_kept():
    """The standard error of Delta A divides each point's variance by the rings
    it kept (sigmaA / nrep when all count, pimd_par.f90:422); a point with none
    stops the Python driver as it stops the namelist driver."""
    import drivers
    assert drivers._lambda_stderr2([0.5, 0.5], [4.0, 9.0], [4, 9]) == pytest.approx(0.5, rel=1e-15)
    assert drivers._lambda_stderr2([1.0, 2.0], [3.0, 3.0], [3, 3]) == pytest.approx((3.0 + 12.0) / 3, rel=1e-15)
    with pytest.raises(RuntimeError, match=r"\[2\]"):
        drivers._lambda_stderr2([0.5, 0.5], [1.0, 0.0], [3, 0])


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fused", "plain"])
def test_nan_ring_is_flagged_and_isolated(ctx, pg, form):
    c = dict(pgconfigs.load("c1"), P=16)
    ti = pgconfigs.TiInputs(c, nrep=3, nintegral=2)
    ctx.set_system(c["ndim"], c["natom"], c["mass"], c["pes_id"], c["params"], c["V0"])
    cfg = ti.ti_config(pg, pg.PG_FP64, pg.PG_FORM_FUSED if form == "fused" else pg.PG_FORM_PLAIN)
    cfg.imin = 3
    x0 = np.array([ti.xref[li] for li in ti.ring_lambda])
    runs = []
    for bad in (False, True):
        xs = x0.copy()
        if bad:
            xs[4, 5] = np.nan  # ring 4: lambda point 1, replica 1
        ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref, x0=xs)
        ctx.ti_advance(40)
        runs.append((ctx.ti_results(), ctx.ti_lambda_reduce()))
        ctx.ti_release()
    (s0, n0, _, st0), (m0, v0, c0) = runs[0]
    (s1, n1, _, st1), (m1, v1, c1) = runs[1]
    assert np.all(st0 == 0)
    assert st1[4] & pg.PG_RING_NAN and np.all(np.delete(st1, 4) == 0)
    others = np.arange(ti.nrings) != 4
    np.testing.assert_array_equal(s1[others], s0[others])  # the rings are independent
    np.testing.assert_array_equal(n1[others], n0[others])
    assert list(c1) == [3, 2] and list(c0) == [3, 3]
    integ = s0 / n0 / ti.betan ** 2
    assert m1[0] == m0[0]
    assert m1[1] == pytest.approx(np.mean(integ[[3, 5]]), rel=1e-13)


@pytest.mark.gpu
def test_transform_wait_that_runs_out_is_reported_and_the_context_stays_usable(ctx, pg):
    """Failure detection without a GPU fault: with the wait limit (a deadline
    from the kernel's start) at 0, the tensor-core transform's first bounded
    wait -- for the bulk copy of T -- gives up, the kernel lets the copy land and
    issues no GEMM, and the call returns PG_ERR_NUMERIC; back at the default
    limit, the same context transforms the same columns correctly."""
    P = 128
    cols = np.random.RandomState(5).randn(128 * P)  # one tile
    ref = ctx.nm_transform(P, cols, pg.PG_FP64)
    ctx.set_wait_limit(0)
    try:
        with pytest.raises(pg.PgError) as e:
            ctx.nm_transform(P, cols, pg.PG_MIXED)
        assert e.value.code == pg.PG_ERR_NUMERIC
        assert "wait limit" in str(e.value)
    finally:
        ctx.set_wait_limit(2000000000)
    out = ctx.nm_transform(P, cols, pg.PG_MIXED)
    assert np.max(np.abs(out - ref)) <= 3e-5 * np.max(np.abs(ref))
