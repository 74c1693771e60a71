"""GPU parity of the TI-PIMD path against the CPU oracle, through the C-ABI.

FP64 forms are compared trajectory-by-trajectory over short runs (same Philox
streams, so the only differences are libm / FMA rounding): fused NM-resident
kernel vs the oracle's NM-resident step, plain per-step form vs the oracle's
reference-order (ten-transform) step.  The mixed-precision forms are compared
with the FP64 form over short runs (FP32 tolerance)."""
import os

import numpy as np
import pytest

import pgconfigs

pytestmark = pytest.mark.gpu


def _pes(oracle, c):
    return oracle.Pes(c["pes_id"], c["ndim"], c["natom"], c["params"], V0=c["V0"])


def _set_system(ctx, c):
    ctx.set_system(c["ndim"], c["natom"], c["mass"], c["pes_id"], c["params"], c["V0"])


def _small_2d(P=16, nrep=2, nint=3, beta=None):
    c = dict(pgconfigs.load("c1"))
    c["P"] = P
    if beta is not None:
        c["beta"] = beta
    ti = pgconfigs.TiInputs(c, nrep=nrep, nintegral=nint)
    return c, ti


def _oracle_run(oracle, c, ti, prm, nsteps, x0=None, p0=None):
    pes = _pes(oracle, c)
    mass = np.array(c["mass"])
    nd, P = ti.nd, ti.P
    xs, ps, sums, ns, nre = [], [], [], [], []
    for r in range(ti.nrings):
        li = ti.ring_lambda[r]
        if x0 is None:
            x, p = oracle.ring_init(pes, mass, prm, ti.xref[li], int(ti.ring_seed[r]), int(ti.ring_stream[r]),
                                    a=ti.a, b=ti.b[li])
        else:
            x = x0[r].copy()
            p = p0[r].copy()
        res = oracle.ring_propagate(pes, mass, prm, ti.a, ti.b[li], ti.dbdl[li], ti.xref[li],
                                    int(ti.ring_seed[r]), int(ti.ring_stream[r]), 0, nsteps, x, p)
        xs.append(x)
        ps.append(p)
        sums.append(res.dhdr_sum)
        ns.append(res.nsamples)
        nre.append(res.nreinit)
    return np.array(xs), np.array(ps), np.array(sums), np.array(ns), np.array(nre)


def _oracle_prm(oracle, c, ti, nm_resident, thermostat=2, cayley=False, dhdr_limit=-1.0, noutput=100000):
    return oracle.TiParams(ti.P, c["beta"], c["dt"], tau=c["tau"], gamma=c["gamma"], thermostat=thermostat,
                           cayley=cayley, nm_resident=nm_resident, imin=3,
                           noutput=noutput, dhdr_limit=dhdr_limit, init_sigma=c["init_sigma"])


def _gpu_cfg(pg, c, ti, precision, form, thermostat=2, cayley=False, dhdr_limit=-1.0, noutput=100000):
    t = ti.ti_config(pg, precision, form)
    t.thermostat = thermostat
    t.cayley = int(cayley)
    t.imin = 3
    t.dhdr_limit = dhdr_limit
    t.noutput = noutput
    return t


@pytest.mark.parametrize("name", ["c0", "c1", "c2", "c4"])
def test_pes_eval_matches_oracle(ctx, pg, oracle, name):
    c = pgconfigs.load(name)
    _set_system(ctx, c)
    pes = _pes(oracle, c)
    rs = np.random.RandomState(4)
    w = np.array(c["well1"])
    X = np.array([w + 0.1 * rs.randn(w.size) for _ in range(64)])
    V, G = ctx.pes_eval(X.ravel(), pg.PG_FP64)
    for i in range(len(X)):
        assert abs(V[i] - pes.V(X[i])) <= 1e-13 * max(1.0, abs(pes.V(X[i])))
        np.testing.assert_allclose(G[i], pes.Vprime(X[i]), rtol=1e-12, atol=1e-14)
    Vf, Gf = ctx.pes_eval(X.ravel(), pg.PG_MIXED)
    gs = np.max(np.abs(G))
    assert np.max(np.abs(Gf - G)) < 2e-5 * gs + 1e-6


def test_unrolled_nine_atom_surface_matches_the_table_driven_one(ctx, pg, oracle):
    """The FP32 9-atom surface runs fully unrolled (coordinates and gradient in
    registers) when its table lists all 36 pairs i < j in order; the same terms
    with the table's rows reversed take the table-driven path.  Both agree with
    each other to FP32 rounding and with the oracle (FP64)."""
    c = pgconfigs.load("c2")
    p = np.array(c["params"], dtype=float)
    npair = int(p[0])
    rows = p[1:1 + 5 * npair].reshape(npair, 5)
    p_rev = np.concatenate([[npair], rows[::-1].ravel(), p[1 + 5 * npair:]])
    rs = np.random.RandomState(8)
    w = np.array(c["well1"])
    X = np.array([w + 0.1 * rs.randn(w.size) for _ in range(64)])
    out = []
    for params in (p, p_rev):
        ctx.set_system(c["ndim"], c["natom"], c["mass"], c["pes_id"], list(params), c["V0"])
        out.append(ctx.pes_eval(X.ravel(), pg.PG_MIXED))
    (Vu, Gu), (Vt, Gt) = out
    pes = _pes(oracle, c)
    Vo = np.array([pes.V(x) for x in X])
    Go = np.array([pes.Vprime(x) for x in X])
    gs = np.max(np.abs(Go))
    assert np.max(np.abs(Gu - Gt.reshape(Gu.shape))) < 4e-6 * gs
    assert np.max(np.abs(Gu - Go)) < 2e-5 * gs + 1e-6
    assert np.max(np.abs(Vu - Vo)) < 2e-6 * max(1.0, np.max(np.abs(Vo)))
    assert np.max(np.abs(Vu - Vt)) < 2e-6 * max(1.0, np.max(np.abs(Vo)))


@pytest.mark.parametrize("name", ["c0", "c1", "c2", "c4"])
def test_pes_hessian_matches_oracle(ctx, pg, oracle, name):
    c = pgconfigs.load(name)
    _set_system(ctx, c)
    pes = _pes(oracle, c)
    rs = np.random.RandomState(5)
    w = np.array(c["well1"])
    X = np.array([w + 0.05 * rs.randn(w.size) for _ in range(8)])
    for quirks in (False, True):
        H = ctx.pes_hessian(X.ravel(), quirks=quirks)
        for i in range(len(X)):
            np.testing.assert_allclose(H[i], pes.Vdoubleprime(X[i], quirks=quirks), rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("P", [16, 32, 128, 256])
def test_nm_transform_matches_oracle(ctx, pg, oracle, P):
    T, _, _, _ = oracle.init_nm(P, 1, 1, [1.0], 1.0, 1.0, [0.0], [0.0])
    cols = np.random.RandomState(P).randn(40, P)
    out = ctx.nm_transform(P, cols.ravel(), pg.PG_FP64).reshape(40, P)
    np.testing.assert_allclose(out, cols @ T.T, rtol=0, atol=1e-13 * P)
    outf = ctx.nm_transform(P, cols.ravel(), pg.PG_MIXED).reshape(40, P)
    assert np.max(np.abs(outf - out)) < 3e-5 * np.max(np.abs(out))


@pytest.mark.parametrize("thermostat,cayley", [(2, False), (1, False), (2, True)])
def test_fused_fp64_matches_oracle_nm_resident(ctx, pg, oracle, thermostat, cayley):
    c, ti = _small_2d()
    _set_system(ctx, c)
    nsteps = 80
    cfg = _gpu_cfg(pg, c, ti, pg.PG_FP64, pg.PG_FORM_FUSED, thermostat, cayley, noutput=9)
    ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
    ctx.ti_advance(nsteps)
    x, p = ctx.ti_state()
    s, n, ri, st = ctx.ti_results()
    prm = _oracle_prm(oracle, c, ti, True, thermostat, cayley, noutput=9)
    xo, po, so, no, _ = _oracle_run(oracle, c, ti, prm, nsteps)
    assert np.all(st == 0)
    np.testing.assert_array_equal(n, no)
    np.testing.assert_allclose(x.reshape(xo.shape), xo, rtol=0, atol=1e-9)
    np.testing.assert_allclose(p.reshape(po.shape), po, rtol=0, atol=1e-7 * np.max(np.abs(po)))
    np.testing.assert_allclose(s, so, rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("thermostat", [2, 1])
def test_plain_form_matches_oracle_reference_order(ctx, pg, oracle, thermostat):
    c, ti = _small_2d()
    _set_system(ctx, c)
    nsteps = 60
    cfg = _gpu_cfg(pg, c, ti, pg.PG_FP64, pg.PG_FORM_PLAIN, thermostat, noutput=9)
    ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
    ctx.ti_advance(nsteps)
    x, p = ctx.ti_state()
    s, n, ri, st = ctx.ti_results()
    prm = _oracle_prm(oracle, c, ti, False, thermostat, noutput=9)
    xo, po, so, no, _ = _oracle_run(oracle, c, ti, prm, nsteps)
    assert np.all(st == 0)
    np.testing.assert_array_equal(n, no)
    np.testing.assert_allclose(x.reshape(xo.shape), xo, rtol=0, atol=1e-9)
    np.testing.assert_allclose(s, so, rtol=1e-9, atol=1e-9)


def test_c0_plain_and_fused_fp64_match_oracle(ctx, pg, oracle):
    c = pgconfigs.load("c0")
    ti = pgconfigs.TiInputs(c)
    _set_system(ctx, c)
    nsteps = 100
    prm_ref = _oracle_prm(oracle, c, ti, False)
    xo, po, so, no, _ = _oracle_run(oracle, c, ti, prm_ref, nsteps)
    for form in (pg.PG_FORM_PLAIN, pg.PG_FORM_FUSED):
        cfg = _gpu_cfg(pg, c, ti, pg.PG_FP64, form)
        ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
        ctx.ti_advance(nsteps)
        x, p = ctx.ti_state()
        s, n, _, st = ctx.ti_results()
        np.testing.assert_allclose(x.reshape(xo.shape), xo, rtol=0, atol=1e-9)
        np.testing.assert_allclose(s, so, rtol=1e-9)


def test_dhdr_limit_reinit_matches_oracle(ctx, pg, oracle):
    c, ti = _small_2d(nrep=1, nint=2)
    _set_system(ctx, c)
    nsteps = 30
    lim = 2000.0
    cfg = _gpu_cfg(pg, c, ti, pg.PG_FP64, pg.PG_FORM_FUSED, dhdr_limit=lim)
    ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
    ctx.ti_advance(nsteps)
    x, _ = ctx.ti_state()
    s, n, ri, st = ctx.ti_results()
    prm = _oracle_prm(oracle, c, ti, True, dhdr_limit=lim)
    xo, po, so, no, reo = _oracle_run(oracle, c, ti, prm, nsteps)
    np.testing.assert_array_equal(ri, reo)
    assert np.sum(ri) > 0
    np.testing.assert_allclose(x.reshape(xo.shape), xo, rtol=0, atol=1e-9)
    np.testing.assert_allclose(s, so, rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("P", [32, 128])
def test_tensor_blocked_dhdr_limit_tracks_simt(ctx, pg, P):
    """dHdrlimit re-initialisation in the blocked tcgen05 form
    (verletmodule.f90:404-409): the force kernel of step s flags a ring whose
    estimate of step s - 1 is over the limit, and k_ti_reinit re-initialises it
    (the SIMT form's streams for that step) with its forces before the kick.  The
    estimator weights db/dlambda of the three lambda points are scaled by 0.1, 1
    and 10 (the dynamics do not use them), so with a limit of 2e4 the last point
    goes over at every step and the others never do (|contr| ~ 7e3 here).
    Against the FP32 SIMT form on the same streams: the same re-initialisation
    and sample counts, positions and sums; and the rings that are never flagged
    run bitwise as under a limit that is never reached.  P = 128 also goes to
    the blocked form."""
    c, ti = _small_2d(P=P, nrep=2, nint=3)
    ti.dbdl = np.array(ti.dbdl, dtype=float) * np.array([0.1, 1.0, 10.0])[:, None]
    _set_system(ctx, c)
    nsteps, lim = 40, 2.0e4
    runs = {}
    for name, form, dl in (("tensor", pg.PG_FORM_TENSOR, lim), ("simt", pg.PG_FORM_FUSED, lim),
                           ("tensor_nolim", pg.PG_FORM_TENSOR, 1.0e30)):
        cfg = _gpu_cfg(pg, c, ti, pg.PG_MIXED, form, dhdr_limit=dl)
        ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
        assert ctx.ti_form(1)[0] == form
        ctx.ti_advance(nsteps)
        x, p = ctx.ti_state()
        s, n, ri, st = ctx.ti_results()
        runs[name] = (x.reshape(ti.nrings, -1), p.reshape(ti.nrings, -1), s, n, ri, st)
    xt, pt, st_, nt, rt, stat = runs["tensor"]
    xs, ps, ss, ns, rs, _ = runs["simt"]
    flagged = np.asarray(ti.ring_lambda) == 2
    assert np.all(stat == 0)
    assert np.all(rt[flagged] == nsteps - 3) and np.all(rt[~flagged] == 0)
    np.testing.assert_array_equal(rt, rs)
    np.testing.assert_array_equal(nt, ns)
    assert np.all(st_[flagged] == 0.0) and np.all(ss[flagged] == 0.0)
    np.testing.assert_allclose(xt, xs, rtol=0, atol=2e-3)
    np.testing.assert_allclose(st_, ss, rtol=2e-4, atol=0)
    xn, pn, sn, nn, _, _ = runs["tensor_nolim"]
    np.testing.assert_array_equal(xt[~flagged], xn[~flagged])
    np.testing.assert_array_equal(pt[~flagged], pn[~flagged])
    np.testing.assert_array_equal(st_[~flagged], sn[~flagged])


@pytest.mark.parametrize("form", ["fused64", "plain", "mixed", "tensor_tile", "tensor_blocked"])
def test_chunked_advance_and_checkpoint_are_bitwise(ctx, pg, tmp_path, form):
    c, ti = _small_2d(P=128 if form == "tensor_tile" else 32)
    _set_system(ctx, c)
    prec = pg.PG_FP64 if form in ("fused64", "plain") else pg.PG_MIXED
    fm = {"fused64": pg.PG_FORM_FUSED, "plain": pg.PG_FORM_PLAIN, "mixed": pg.PG_FORM_AUTO,
          "tensor_tile": pg.PG_FORM_TENSOR, "tensor_blocked": pg.PG_FORM_TENSOR}[form]
    cfg = _gpu_cfg(pg, c, ti, prec, fm)
    ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
    ctx.ti_advance(70)
    x1, p1 = ctx.ti_state()
    s1 = ctx.ti_results()[0]
    ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
    ctx.ti_advance(30)
    path = str(tmp_path / "ck.bin")
    ctx.ti_checkpoint_save(path)
    ctx.ti_advance(10)  # diverge, then restore
    ctx.ti_checkpoint_load(path)
    assert ctx.ti_step() == 30
    ctx.ti_advance(40)
    x2, p2 = ctx.ti_state()
    s2 = ctx.ti_results()[0]
    np.testing.assert_array_equal(x1, x2)
    np.testing.assert_array_equal(p1, p2)
    np.testing.assert_array_equal(s1, s2)


def test_lambda_reduce_matches_host_formula(ctx, pg):
    c, ti = _small_2d(nrep=5, nint=3)
    _set_system(ctx, c)
    cfg = _gpu_cfg(pg, c, ti, pg.PG_FP64, pg.PG_FORM_FUSED)
    ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
    ctx.ti_advance(40)
    s, n, _, _ = ctx.ti_results()
    m, v, cnt = ctx.ti_lambda_reduce()
    integ = (s / n / ti.betan ** 2).reshape(3, 5)
    np.testing.assert_allclose(m, integ.mean(1), rtol=1e-13)
    np.testing.assert_allclose(v, (integ ** 2).mean(1) - integ.mean(1) ** 2, rtol=1e-9, atol=1e-12)
    assert list(cnt) == [5, 5, 5]


@pytest.mark.parametrize("P", [16, 128])
def test_mixed_forms_track_fp64(ctx, pg, P):
    """Short runs from identical starts: FP32 state + FP32 forces (+ split-BF16
    tensor-core transform at P = 128) stay within FP32 round-off of FP64."""
    c, ti = _small_2d(P=P, nrep=4, nint=2)
    _set_system(ctx, c)
    nsteps = 20
    cfg = _gpu_cfg(pg, c, ti, pg.PG_FP64, pg.PG_FORM_FUSED)
    ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
    ctx.ti_advance(nsteps)
    x64, p64 = ctx.ti_state()
    s64 = ctx.ti_results()[0]
    for form in (pg.PG_FORM_FUSED, pg.PG_FORM_AUTO):
        cfg = _gpu_cfg(pg, c, ti, pg.PG_MIXED, form)
        ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
        ctx.ti_advance(nsteps)
        x32, p32 = ctx.ti_state()
        s32 = ctx.ti_results()[0]
        assert np.max(np.abs(x32 - x64)) < 2e-3, form
        assert np.max(np.abs(p32 - p64)) < 2e-3 * np.max(np.abs(p64)), form
        np.testing.assert_allclose(s32, s64, rtol=2e-4)


def test_propagate_pimd_dropin(ctx, pg, oracle):
    c, ti = _small_2d(nrep=1, nint=3)
    _set_system(ctx, c)
    pes = _pes(oracle, c)
    mass = np.array(c["mass"])
    prm = _oracle_prm(oracle, c, ti, True)
    x0, p0 = [], []
    for r in range(ti.nrings):
        li = ti.ring_lambda[r]
        x, p = oracle.ring_init(pes, mass, prm, ti.xref[li], int(ti.ring_seed[r]), int(ti.ring_stream[r]),
                                a=ti.a, b=ti.b[li])
        x0.append(x)
        p0.append(p)
    x0, p0 = np.array(x0), np.array(p0)
    cfg = _gpu_cfg(pg, c, ti, pg.PG_FP64, pg.PG_FORM_FUSED)
    x, p, dh, st = ctx.propagate_pimd(cfg, 50, ti.a, ti.b, ti.dbdl, ti.ring_seed, ti.ring_stream, x0, p0)
    xo, po, so, no, _ = _oracle_run(oracle, c, ti, prm, 50, x0=x0, p0=p0)
    np.testing.assert_allclose(x.reshape(xo.shape), xo, atol=1e-9)
    np.testing.assert_allclose(dh, so / no, rtol=1e-9)


def _run(ctx, pg, c, ti, precision, form, nsteps, thermostat=2):
    cfg = _gpu_cfg(pg, c, ti, precision, form, thermostat)
    ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
    ctx.ti_advance(nsteps)
    x, p = ctx.ti_state()
    s, n, ri, st = ctx.ti_results()
    return x, p, s, n, st


def test_tensor_tile_two_chunks_per_cta_multi_launch(ctx, pg):
    """12,000 rings at P = 128: more 64-column chunks than CTAs (two per CTA on
    most), 60 steps = launches of 50 + 10 MD steps, against 30 + 30; and the
    FP32 SIMT form from the same state."""
    c, ti = _small_2d(P=128, nrep=1000, nint=12)
    _set_system(ctx, c)
    x1, p1, s1, n1, st1 = _run(ctx, pg, c, ti, pg.PG_MIXED, pg.PG_FORM_TENSOR, 60)
    cfg = _gpu_cfg(pg, c, ti, pg.PG_MIXED, pg.PG_FORM_TENSOR)
    ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
    ctx.ti_advance(30)
    ctx.ti_advance(30)
    x2, p2 = ctx.ti_state()
    s2 = ctx.ti_results()[0]
    np.testing.assert_array_equal(x1, x2)
    np.testing.assert_array_equal(s1, s2)
    x3, p3, s3, n3, st3 = _run(ctx, pg, c, ti, pg.PG_MIXED, pg.PG_FORM_FUSED, 60)
    assert np.all(st1 == 0) and np.all(st3 == 0)
    np.testing.assert_array_equal(n1, n3)
    assert np.max(np.abs(x1 - x3)) < 2e-3
    np.testing.assert_allclose(s1, s3, rtol=2e-4, atol=1e-6 * np.max(np.abs(s3)))


def test_tensor_tile_three_chunks_per_cta_state_in_l2(ctx, pg):
    """20,000 rings at P = 128: three 64-column chunks on most CTAs, so q stays
    in global memory (the other step-kernel variant); 60 steps as 50 + 10 against
    30 + 30 bitwise, and against the FP32 SIMT form."""
    c, ti = _small_2d(P=128, nrep=1000, nint=20)
    _set_system(ctx, c)
    x1, p1, s1, n1, st1 = _run(ctx, pg, c, ti, pg.PG_MIXED, pg.PG_FORM_TENSOR, 60)
    cfg = _gpu_cfg(pg, c, ti, pg.PG_MIXED, pg.PG_FORM_TENSOR)
    ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
    ctx.ti_advance(30)
    ctx.ti_advance(30)
    x2, p2 = ctx.ti_state()
    s2 = ctx.ti_results()[0]
    np.testing.assert_array_equal(x1, x2)
    np.testing.assert_array_equal(s1, s2)
    x3, p3, s3, n3, st3 = _run(ctx, pg, c, ti, pg.PG_MIXED, pg.PG_FORM_FUSED, 60)
    assert np.all(st1 == 0) and np.all(st3 == 0)
    np.testing.assert_array_equal(n1, n3)
    assert np.max(np.abs(x1 - x3)) < 2e-3
    np.testing.assert_allclose(s1, s3, rtol=2e-4, atol=1e-6 * np.max(np.abs(s3)))


@pytest.mark.parametrize("nrep,nint", [(4, 2), (50, 3)])
def test_tensor_form_tracks_simt_fp32(ctx, pg, nrep, nint):
    """tcgen05 split-BF16 kernel vs the FP32 SIMT kernel over a short run from the
    same state (150 rings = 2 full CTAs + a partial one in the second case)."""
    c, ti = _small_2d(P=128, nrep=nrep, nint=nint)
    _set_system(ctx, c)
    x1, p1, s1, n1, st1 = _run(ctx, pg, c, ti, pg.PG_MIXED, pg.PG_FORM_FUSED, 20)
    x2, p2, s2, n2, st2 = _run(ctx, pg, c, ti, pg.PG_MIXED, pg.PG_FORM_TENSOR, 20)
    assert np.all(st1 == 0) and np.all(st2 == 0)
    np.testing.assert_array_equal(n1, n2)
    assert np.max(np.abs(x1 - x2)) < 2e-3
    assert np.max(np.abs(p1 - p2)) < 2e-3 * np.max(np.abs(p1))
    np.testing.assert_allclose(s2, s1, rtol=2e-4)


def test_tensor_form_1d_surface(ctx, pg):
    c = dict(pgconfigs.load("c0"))
    c["P"] = 128
    ti = pgconfigs.TiInputs(c, nrep=3, nintegral=3)
    _set_system(ctx, c)
    x1, p1, s1, n1, st1 = _run(ctx, pg, c, ti, pg.PG_FP64, pg.PG_FORM_FUSED, 20)
    x2, p2, s2, n2, st2 = _run(ctx, pg, c, ti, pg.PG_MIXED, pg.PG_FORM_TENSOR, 20)
    assert np.all(st2 == 0)
    assert np.max(np.abs(x1 - x2)) < 2e-3
    np.testing.assert_allclose(s2, s1, rtol=2e-4)


@pytest.mark.parametrize("form", ["fused", "tensor"])
def test_mixed_long_run_has_no_nan(ctx, pg, form):
    """Regression: thousands of steps over a thousand rings stay finite (the FP32
    Box-Muller radius once hit rsqrt(0) near u = 1)."""
    c, ti = _small_2d(P=128, nrep=64, nint=16)
    _set_system(ctx, c)
    fm = pg.PG_FORM_FUSED if form == "fused" else pg.PG_FORM_TENSOR
    cfg = _gpu_cfg(pg, c, ti, pg.PG_MIXED, fm)
    ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
    ctx.ti_advance(3000)
    s, n, _, st = ctx.ti_results()
    assert np.all(st == 0), np.sum(st != 0)
    assert np.all(np.isfinite(s))


def _small_synth9(P=16, nrep=2, nint=2):
    c = dict(pgconfigs.load("c2"))
    c["P"] = P
    ti = pgconfigs.TiInputs(c, nrep=nrep, nintegral=nint)
    return c, ti


def test_fused_fp64_many_dofs_matches_oracle(ctx, pg, oracle):
    """27 dofs: the ring transforms run in four passes of up to eight dofs."""
    c, ti = _small_synth9()
    _set_system(ctx, c)
    nsteps = 30
    cfg = _gpu_cfg(pg, c, ti, pg.PG_FP64, pg.PG_FORM_FUSED)
    ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
    ctx.ti_advance(nsteps)
    x, p = ctx.ti_state()
    s, n, _, st = ctx.ti_results()
    prm = _oracle_prm(oracle, c, ti, True)
    xo, po, so, no, _ = _oracle_run(oracle, c, ti, prm, nsteps)
    assert np.all(st == 0)
    np.testing.assert_array_equal(n, no)
    np.testing.assert_allclose(x.reshape(xo.shape), xo, rtol=0, atol=1e-9)
    np.testing.assert_allclose(s, so, rtol=1e-9, atol=1e-12)
    # FP32 state + forces track FP64 over the same steps
    cfg = _gpu_cfg(pg, c, ti, pg.PG_MIXED, pg.PG_FORM_FUSED)
    ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
    ctx.ti_advance(nsteps)
    x32, _ = ctx.ti_state()
    assert np.max(np.abs(x32.reshape(xo.shape) - xo)) < 2e-3


def test_advance_group_equals_separate_advances(pg):
    """Two bead numbers in two contexts, advanced together on concurrent streams,
    give bitwise the results of advancing each alone."""
    runs = []
    for together in (False, True):
        ctxs, tis = [], []
        for P in (16, 32):
            c, ti = _small_2d(P=P, nrep=3, nint=2)
            cx = pg.Context(0)
            _set_system(cx, c)
            cfg = _gpu_cfg(pg, c, ti, pg.PG_MIXED, pg.PG_FORM_FUSED)
            cx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
            ctxs.append(cx)
        if together:
            ms = pg.Context.ti_advance_group(ctxs, 40)
            assert ms > 0.0
        else:
            for cx in ctxs:
                cx.ti_advance(40)
        runs.append([(cx.ti_state(), cx.ti_results()[:2], cx.ti_step()) for cx in ctxs])
        for cx in ctxs:
            cx.close()
    for (st_a, res_a, step_a), (st_b, res_b, step_b) in zip(*runs):
        assert step_a == step_b == 40
        for u, v in zip(st_a + res_a, st_b + res_b):
            np.testing.assert_array_equal(u, v)


def test_advance_group_one_graph_over_tensor_and_simt_batches(pg):
    """An uneven-P group in one graph launch: the persistent tcgen05 step kernel
    (P = 128, 2-D surface), the persistent folded step (P = 256, 27-dof surface)
    and the fused SIMT form (P = 64) as concurrent branches of one captured graph,
    advanced twice by 25 steps (the second call replays the cached graph), give
    bitwise the state and estimator sums of advancing each batch alone by 50."""
    specs = [("c1", 128, pg.PG_FORM_TENSOR, 40), ("c2", 256, pg.PG_FORM_TENSOR, 3), ("c1", 64, pg.PG_FORM_FUSED, 5)]
    runs = []
    for together in (False, True):
        ctxs = []
        for name, P, form, nrep in specs:
            c = dict(pgconfigs.load(name))
            c["P"] = P
            ti = pgconfigs.TiInputs(c, nrep=nrep, nintegral=2)
            cx = pg.Context(0)
            _set_system(cx, c)
            cfg = _gpu_cfg(pg, c, ti, pg.PG_MIXED, form)
            cx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
            assert cx.ti_form(1)[0] == form
            ctxs.append(cx)
        if together:
            for _ in range(2):
                assert pg.Context.ti_advance_group(ctxs, 25) > 0.0
        else:
            for cx in ctxs:
                cx.ti_advance(50)
        runs.append([(cx.ti_state(), cx.ti_results()[:2], cx.ti_step()) for cx in ctxs])
        for cx in ctxs:
            cx.close()
    for (st_a, res_a, step_a), (st_b, res_b, step_b) in zip(*runs):
        assert step_a == step_b == 50
        for u, v in zip(st_a + res_a, st_b + res_b):
            np.testing.assert_array_equal(u, v)


def _tensor_vs_simt(ctx, pg, c, ti, nsteps=20):
    _set_system(ctx, c)
    x1, p1, s1, n1, st1 = _run(ctx, pg, c, ti, pg.PG_MIXED, pg.PG_FORM_FUSED, nsteps)
    x2, p2, s2, n2, st2 = _run(ctx, pg, c, ti, pg.PG_MIXED, pg.PG_FORM_TENSOR, nsteps)
    assert ctx.ti_form(1)[0] == pg.PG_FORM_TENSOR
    assert np.all(st1 == 0) and np.all(st2 == 0)
    np.testing.assert_array_equal(n1, n2)
    return x1, p1, s1, x2, p2, s2


@pytest.mark.parametrize("P,nrep", [(256, 3), (384, 2), (512, 2)])
def test_tensor_blocked_many_dofs_tracks_simt(ctx, pg, P, nrep):
    """Blocked split-BF16 GEMMs on the 27-dof surface, 6 or 4 rings = 162 or 108
    columns (a partial 64-column tile), against the FP32 SIMT form from the same
    state: P = 256 (2 x 2 blocks of T), P = 384 (3 x 3, 192 TMEM columns),
    P = 512 (4 x 4, 256 TMEM columns)."""
    c = dict(pgconfigs.load("c2"))
    c["P"] = P
    ti = pgconfigs.TiInputs(c, nrep=nrep, nintegral=2)
    x1, p1, s1, x2, p2, s2 = _tensor_vs_simt(ctx, pg, c, ti)
    assert np.max(np.abs(x1 - x2)) < 2e-3
    assert np.max(np.abs(p1 - p2)) < 2e-3 * np.max(np.abs(p1))
    np.testing.assert_allclose(s2, s1, rtol=2e-4)


def test_tensor_blocked_padded_small_p(ctx, pg):
    """P = 32 on the 1-D surface: T zero-padded into one 128 x 128 block."""
    c = dict(pgconfigs.load("c0"))
    ti = pgconfigs.TiInputs(c, nrep=5, nintegral=3)
    x1, p1, s1, x2, p2, s2 = _tensor_vs_simt(ctx, pg, c, ti)
    assert np.max(np.abs(x1 - x2)) < 2e-3
    np.testing.assert_allclose(s2, s1, rtol=2e-4)


def _c_at_256(cfgname):
    c = dict(pgconfigs.load(cfgname))
    c["P"] = 256
    if "dt_per_P" in c:
        c["dt"] = c["dt_per_P"]["256"]
    return c


@pytest.mark.parametrize("cfgname,nrep,nint,kernel", [("c2", 3, 2, "k_tf_step ("), ("c2", 40, 12, "k_tf_step ("),
                                                      ("c2", 120, 12, "k_tf_step ("), ("c4", 2, 2, "k_tb_")])
def test_tensor_folded_p256_tracks_simt(ctx, pg, cfgname, nrep, nint, kernel):
    """The persistent folded step (k_tf_step: P = 256 with T folded into two
    resident 128 x 128 halves, one CTA per SM over whole rings, two warp groups
    on alternate two-ring chunks) against the FP32 SIMT form from the same
    state, on the 9-atom surface: 6 rings (one CTA per ring, the second group
    idle), 480 rings (one chunk per group) and 1,440 rings (up to 3 chunks per
    group, the next chunk's positions formed ahead).  The 18-atom (54-dof)
    surface runs the blocked kernels at P = 256."""
    c = _c_at_256(cfgname)
    ti = pgconfigs.TiInputs(c, nrep=nrep, nintegral=nint, P=256)
    x1, p1, s1, x2, p2, s2 = _tensor_vs_simt(ctx, pg, c, ti)
    names = [k[0] for k in ctx.ti_kernel_times(5)]
    assert names[0].startswith(kernel), names
    assert np.max(np.abs(x1 - x2)) < 2e-3
    assert np.max(np.abs(p1 - p2)) < 2e-3 * np.max(np.abs(p1))
    np.testing.assert_allclose(s2, s1, rtol=2e-4)


def test_tensor_folded_launch_boundaries_and_checkpoint_are_bitwise(ctx, pg, tmp_path):
    """k_tf_step keeps the ring state in global memory between steps, so 70
    steps in one advance (launches of 50 + 20) and 30 + 40 across a checkpoint
    reload give the same bits."""
    c = _c_at_256("c2")
    ti = pgconfigs.TiInputs(c, nrep=5, nintegral=3, P=256)
    _set_system(ctx, c)
    cfg = _gpu_cfg(pg, c, ti, pg.PG_MIXED, pg.PG_FORM_TENSOR)
    ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
    ctx.ti_advance(70)
    x1, p1 = ctx.ti_state()
    s1 = ctx.ti_results()[0]
    ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
    ctx.ti_advance(30)
    path = str(tmp_path / "ck.bin")
    ctx.ti_checkpoint_save(path)
    ctx.ti_advance(10)
    ctx.ti_checkpoint_load(path)
    ctx.ti_advance(40)
    x2, p2 = ctx.ti_state()
    s2 = ctx.ti_results()[0]
    np.testing.assert_array_equal(x1, x2)
    np.testing.assert_array_equal(p1, p2)
    np.testing.assert_array_equal(s1, s2)


@pytest.mark.parametrize("cfgname,P", [("c1", 128), ("c2", 256)])
def test_tensor_forms_with_cayley_rotation(ctx, pg, cfgname, P):
    """cayley = 1 (verletmodule.f90:520-526): the per-mode rotation coefficients
    the tensor forms apply are the Cayley ones; fused tile (P = 128) and
    persistent folded (P = 256, 27 dofs) forms track the FP32 SIMT form."""
    c = dict(pgconfigs.load(cfgname))
    c["P"] = P
    ti = pgconfigs.TiInputs(c, nrep=3, nintegral=2)
    _set_system(ctx, c)
    out = []
    for form in (pg.PG_FORM_FUSED, pg.PG_FORM_TENSOR):
        cfg = _gpu_cfg(pg, c, ti, pg.PG_MIXED, form, cayley=True)
        ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
        assert ctx.ti_form(1)[0] == form
        ctx.ti_advance(20)
        out.append((ctx.ti_state()[0], ctx.ti_results()[0]))
    assert np.max(np.abs(out[0][0] - out[1][0])) < 2e-3
    np.testing.assert_allclose(out[1][1], out[0][1], rtol=2e-4)


@pytest.mark.parametrize("P,nrep,nint", [(15, 1, 1), (7, 3, 1), (33, 1, 3)])
def test_fused_fp64_odd_shapes_match_oracle(ctx, pg, oracle, P, nrep, nint):
    """Ragged shapes: odd bead numbers (not a multiple of the transform passes or
    of a warp) and a single ring."""
    c, ti = _small_2d(P=P, nrep=nrep, nint=nint)
    _set_system(ctx, c)
    nsteps = 40
    cfg = _gpu_cfg(pg, c, ti, pg.PG_FP64, pg.PG_FORM_FUSED)
    ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
    ctx.ti_advance(nsteps)
    x, _ = ctx.ti_state()
    s, n, _, st = ctx.ti_results()
    prm = _oracle_prm(oracle, c, ti, True)
    xo, po, so, no, _ = _oracle_run(oracle, c, ti, prm, nsteps)
    assert np.all(st == 0)
    np.testing.assert_array_equal(n, no)
    np.testing.assert_allclose(x.reshape(xo.shape), xo, rtol=0, atol=1e-9)
    np.testing.assert_allclose(s, so, rtol=1e-9, atol=1e-12)


def test_tensor_form_single_ring_and_rejections(ctx, pg):
    """One ring on the fused tiles (a 2-column chunk) tracks the SIMT form; the
    tensor form is refused where it does not apply (P % 4 != 0 with either
    thermostat, with or without dHdrlimit)."""
    c, ti = _small_2d(P=128, nrep=1, nint=1)
    x1, p1, s1, x2, p2, s2 = _tensor_vs_simt(ctx, pg, c, ti)
    assert np.max(np.abs(x1 - x2)) < 2e-3
    for P, thermostat, lim in ((30, 1, -1.0), (30, 2, -1.0), (30, 2, 1.0)):
        c, ti = _small_2d(P=P, nrep=1, nint=1)
        cfg = _gpu_cfg(pg, c, ti, pg.PG_MIXED, pg.PG_FORM_TENSOR, thermostat, dhdr_limit=lim)
        with pytest.raises(pg.PgError):
            ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)


@pytest.mark.parametrize("cfgname,P,nrep", [("c1", 128, 3), ("c2", 256, 3), ("c0", 64, 5)])
def test_tensor_blocked_andersen_tracks_simt(ctx, pg, cfgname, P, nrep):
    """Andersen thermostat (verletmodule.f90:204-234) on the blocked tcgen05 form:
    with noutput = 9 every ring is resampled several times in 40 steps; the
    same Poisson schedule and Andersen normals as the FP32 SIMT form, so the
    runs track each other at the FP32 / split-BF16 tolerance."""
    c = dict(pgconfigs.load(cfgname))
    c["P"] = P
    ti = pgconfigs.TiInputs(c, nrep=nrep, nintegral=2)
    _set_system(ctx, c)
    out = []
    for form in (pg.PG_FORM_FUSED, pg.PG_FORM_TENSOR):
        cfg = _gpu_cfg(pg, c, ti, pg.PG_MIXED, form, thermostat=1, noutput=9)
        ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
        assert ctx.ti_form(1)[0] == form
        ctx.ti_advance(25)
        ctx.ti_advance(15)  # a second graph, continuing the schedule
        x, p = ctx.ti_state()
        s, n, _, st = ctx.ti_results()
        out.append((x, p, s, n, st))
    (x1, p1, s1, n1, st1), (x2, p2, s2, n2, st2) = out
    assert np.all(st1 == 0) and np.all(st2 == 0)
    np.testing.assert_array_equal(n1, n2)
    assert np.max(np.abs(x1 - x2)) < 2e-3
    assert np.max(np.abs(p1 - p2)) < 2e-3 * np.max(np.abs(p1))
    np.testing.assert_allclose(s2, s1, rtol=2e-4)


def test_autotune_records_and_reuses_its_choice(ctx, pg, tmp_path):
    """PG_TUNE_ON tunes an AUTO batch once (one record in the JSON-lines cache),
    PG_TUNE_CACHE takes the record without tuning again, and both give the same
    trajectory (the tuned setup ends with a fresh setup); a cache miss in
    PG_TUNE_CACHE mode keeps the built-in choice and writes nothing."""
    c, ti = _small_2d(P=128, nrep=20, nint=4)
    _set_system(ctx, c)
    path = tmp_path / "tune.jsonl"
    cfg = _gpu_cfg(pg, c, ti, pg.PG_MIXED, pg.PG_FORM_AUTO)
    args = (ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
    try:
        ctx.set_tuning(path, pg.PG_TUNE_CACHE)  # miss: built-in choice, nothing written
        ctx.ti_setup(cfg, *args)
        assert ctx.ti_tuning()[1:] == (0, 0)
        assert not path.exists()
        ctx.set_tuning(path, pg.PG_TUNE_ON)
        ctx.ti_setup(cfg, *args)
        choice = ctx.ti_tuning()
        lines = path.read_text().splitlines()
        assert len(lines) == 1 and '"form": %d' % choice[0] in lines[0]
        assert choice[0] in (pg.PG_FORM_FUSED, pg.PG_FORM_TENSOR)
        ctx.ti_advance(30)
        x1 = ctx.ti_state()[0]
        s1 = ctx.ti_results()[0]
        ctx.set_tuning(path, pg.PG_TUNE_CACHE)
        ctx.ti_setup(cfg, *args)
        assert ctx.ti_tuning() == choice
        ctx.ti_advance(30)
        np.testing.assert_array_equal(ctx.ti_state()[0], x1)
        np.testing.assert_array_equal(ctx.ti_results()[0], s1)
        assert len(path.read_text().splitlines()) == 1
        # FP64: the fused SIMT form only, tuned over threads per ring
        cfg64 = _gpu_cfg(pg, c, ti, pg.PG_FP64, pg.PG_FORM_AUTO)
        ctx.set_tuning(path, pg.PG_TUNE_ON)
        ctx.ti_setup(cfg64, *args)
        f64, th64, _ = ctx.ti_tuning()
        assert f64 == pg.PG_FORM_FUSED and th64 in (32, 64, 128)
        assert len(path.read_text().splitlines()) == 2
    finally:
        ctx.set_tuning(None, pg.PG_TUNE_OFF)


def test_readhess_start_runs_through_the_driver(pg):
    """run_ti(readhess=True): the polymer Hessian of each lambda point from the
    library, the readhess displacements on the path (numpy), the batch set up
    from them; a short run stays finite and differs from the undisplaced start."""
    import drivers
    c = dict(pgconfigs.load("c1"))
    c["P"] = 32
    c["imin"] = 0  # estimator samples from the first step
    r1 = drivers.run_ti(c, nmc=40, nrep=2, nintegral=3, chunk=40, readhess=True)
    r0 = drivers.run_ti(c, nmc=40, nrep=2, nintegral=3, chunk=40)
    assert r1["nan_rings"] == 0 and np.all(np.isfinite(r1["integrand_mean"]))
    assert r1["integrand_mean"] != r0["integrand_mean"]
