"""The Python drivers' host logic on the CPU (python/drivers.py): each runs in a
subprocess whose binding loads the oracle-backed stand-in for the C-ABI
(tests/standin) in place of libpimdgpu, and its results are checked against
the oracle here.  The stand-in's optimiser returns the start path, so the RPI
checks cover what the driver does around the optimisation: the V0 move, the
end-point springs, the log-dets and the assembly."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import pgconfigs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r'''
import json, sys
sys.path[:0] = [%(py)r, %(pkg)r]
import numpy as np
import pimdgpu as pg
pg.LIBPATH = %(so)r
import drivers, pgconfigs
job = json.loads(sys.stdin.read())
out = {}
if job["kind"] == "rpi":
    c = dict(pgconfigs.load("c1"), well1=job["w1"], well2=job["w2"], V0=job["V0"])
    for fe in (True, False):
        r = drivers.run_rpi(c, N=job["N"], betas=job["betas"], fixedends=fe)
        out[str(fe)] = dict(S=[q["S"] for q in r["results"]], delta=[q["delta"] for q in r["results"]],
                            vpath=r["vpath"].tolist())
elif job["kind"] == "ti":
    c = dict(pgconfigs.load("c0"), imin=50, cayley=job.get("cayley", False), thermostat=job.get("thermostat", 2),
             noutput=job.get("noutput", 100000))
    r = drivers.run_ti(c, precision=pg.PG_FP64, form=pg.PG_FORM_FUSED, nmc=job["nmc"], nrep=2)
    out = dict(dA=r["dA"], qratio=r["qratio"], delta=r["delta"], mean=r["integrand_mean"], nan_rings=r["nan_rings"])
elif job["kind"] == "ti_mixed":
    c = dict(pgconfigs.load("c0"), imin=20, nintegral=2, P_per_ring=job["P_per_ring"])
    r = drivers.run_ti_mixed(c, precision=pg.PG_FP64, form=pg.PG_FORM_FUSED, nmc=job["nmc"], chunk=50)
    out = dict(per_P=[dict(P=q["P"], dA=q["dA"], nrings=q["nrings"]) for q in r["per_P"]])
elif job["kind"] == "ti_readhess":
    c = dict(pgconfigs.load("c1"), P=8, imin=0)
    r = drivers.run_ti(c, precision=pg.PG_FP64, form=pg.PG_FORM_FUSED, nmc=4, nrep=2, nintegral=2, readhess=True)
    out = dict(dA=r["dA"])
elif job["kind"] == "rpi_path":
    c = pgconfigs.load("c3")
    r = drivers.run_rpi(c, N=job["N"], betas=job["betas"], path=[np.array(f) for f in job["frames"]])
    out = dict(S=[q["S"] for q in r["results"]], x=np.asarray(r["x"]).tolist())
elif job["kind"] == "ti_path":
    c = dict(pgconfigs.load("c1"), P=job["P"], imin=job["imin"])
    r = drivers.run_ti(c, precision=pg.PG_FP64, form=pg.PG_FORM_FUSED, nmc=job["nmc"], nrep=2, nintegral=3,
                       frames=[np.array(f) for f in job["frames"]], instapath=True, centre=True, init="path")
    out = dict(dA=r["dA"])
elif job["kind"] == "ti_restart":
    c = dict(pgconfigs.load("c0"), imin=50, P=16, noutput=job.get("noutput", 100000))
    r = drivers.run_ti(c, precision=pg.PG_FP64, form=pg.PG_FORM_FUSED, nmc=job["nmc"], nrep=3,
                       restart=job["restart"], nproc=2, labels=["H"], directory=job["dir"], chunk=30)
    out = dict(dA=r["dA"])
elif job["kind"] == "angular":
    c = pgconfigs.load(job["cfg"])
    rows = drivers.run_rpi_angular(c, job["N"], job["beta"], job["npoints"], cutofftheta=job["ct"],
                                   cutoffphi=job["cp"])
    out = dict(rows=rows.tolist())
elif job["kind"] == "crossover":
    c = pgconfigs.load("c1")
    ctx = pg.Context(0)
    ctx.set_system(2, 1, c["mass"], c["pes_id"], c["params"], c["V0"])
    b, eta = drivers.crossover_beta(ctx, c["ts"], c["mass"])
    ctx.close()
    out = dict(beta_c=b, eta2=list(eta))
print(json.dumps(out))
'''


@pytest.fixture(scope="module")
def run_job(oracle, tmp_path_factory):
    import standin
    so = standin.build_library(tmp_path_factory.mktemp("standin_so"))
    src = SCRIPT % dict(py=os.path.join(ROOT, "pimd-tunneling_gb300", "python"),
                        pkg=os.path.join(ROOT, "pimd-tunneling_gb300"), so=so)

    def run(job, env=None):
        r = subprocess.run([sys.executable, "-c", src], input=json.dumps(job), capture_output=True, text=True,
                           timeout=300, env=dict(os.environ, **(env or {})))
        assert r.returncode == 0, r.stderr
        return json.loads(r.stdout.strip().split("\n")[-1])

    return run


def test_run_rpi_host_logic(oracle, run_job):
    c = pgconfigs.load("c1")
    m1, m2 = np.array(c["well1"]), np.array(c["well2"])
    u = (m1 - m2) / np.linalg.norm(m1 - m2)
    w1, w2 = m1 + 0.3 * u, m2  # the straight start path passes below well 1
    N, betas = 8, [c["beta"] / 16, c["beta"] / 12]
    v0 = oracle.Pes(c["pes_id"], 2, 1, c["params"]).V(w1)  # V0 = V(well 1), rpi_ser.f90:95
    out = run_job(dict(kind="rpi", w1=list(w1), w2=list(w2), V0=v0, N=N, betas=betas))
    pes = oracle.Pes(c["pes_id"], 2, 1, c["params"], V0=v0)
    mass = c["mass"]
    k = np.arange(1, N + 1)
    x = np.concatenate([((N - k) * w1[d] + (k - 1) * w2[d]) / (N - 1) for d in range(2)])
    vpath = np.array([pes.V(x.reshape(2, N)[:, b]) for b in range(N)])
    vmin = min(vpath.min(), 0.0)
    assert vmin < 0
    for fe in (True, False):
        got = out[str(fe)]
        for i, beta in enumerate(betas):
            betan = beta / N  # rpi_ser.f90:45
            np.testing.assert_allclose(got["vpath"][i], vpath, rtol=1e-13, atol=1e-15)
            UM = oracle.UM(pes, mass, N, betan, x, w1, w2, fixedends=fe) - N * vmin
            ld0 = oracle.logdet_band(oracle.UMhessian(pes, mass, N, betan, np.repeat(w1, N), singlewell=True),
                                     False)[0]
            ld = oracle.logdet_band(oracle.UMhessian(pes, mass, N, betan, x), True)[0]
            S = betan * UM
            om = betan * np.exp(-S) * np.sqrt(S / (2 * oracle.PI_REF)) / np.exp(0.5 * (ld - ld0))
            assert got["S"][i] == pytest.approx(S, rel=1e-12)
            assert got["delta"][i] == pytest.approx(2 * om / betan, rel=1e-8)


@pytest.mark.parametrize("cayley,thermostat", [(False, 2), (True, 2), (False, 1)])
def test_run_ti_host_logic(oracle, run_job, cayley, thermostat):
    """Langevin, Cayley and Andersen (Poisson mean noutput = 25) batches of run_ti
    against the oracle ring by ring."""
    out = run_job(dict(kind="ti", nmc=300, cayley=cayley, thermostat=thermostat, noutput=25))
    c = dict(pgconfigs.load("c0"), imin=50, nrep=2, seeds=[0, 1])
    ti = pgconfigs.TiInputs(c, gauleg=oracle.gauleg)
    pes = oracle.Pes(c["pes_id"], c["ndim"], c["natom"], c["params"])
    prm = oracle.TiParams(ti.P, c["beta"], c["dt"], tau=c["tau"], gamma=c["gamma"], thermostat=thermostat,
                          cayley=cayley, nm_resident=True, imin=c["imin"], init_sigma=c["init_sigma"], noutput=25)
    ints = np.zeros(ti.nrings)
    for r in range(ti.nrings):
        li = int(ti.ring_lambda[r])
        x, p = oracle.ring_init(pes, c["mass"], prm, ti.xref[li], int(ti.ring_seed[r]), int(ti.ring_stream[r]),
                                a=ti.a, b=ti.b[li])
        res = oracle.ring_propagate(pes, c["mass"], prm, ti.a, ti.b[li], ti.dbdl[li], ti.xref[li],
                                    int(ti.ring_seed[r]), int(ti.ring_stream[r]), 0, 300, x, p)
        ints[r] = res.dhdr_sum / res.nsamples / ti.betan ** 2
    mean = np.array([ints[ti.ring_lambda == i].mean() for i in range(ti.nint)])
    np.testing.assert_allclose(out["mean"], mean, rtol=1e-12)
    dA = float(np.dot(ti.w, mean))
    assert out["dA"] == pytest.approx(dA, rel=1e-12)
    q = np.exp(-dA * ti.betan)  # pimd_par.f90:420
    assert out["qratio"] == pytest.approx(q, rel=1e-12)
    assert out["delta"] == pytest.approx(2.0 * np.arctanh(q) / c["beta"], rel=1e-10)


def test_crossover_beta_host_logic(oracle, run_job):
    out = run_job(dict(kind="crossover"))
    c = pgconfigs.load("c1")
    b, eta = oracle.crossover_beta(oracle.Pes(c["pes_id"], 2, 1, c["params"]), c["mass"], c["ts"])
    assert out["beta_c"] == pytest.approx(b, rel=1e-12)
    np.testing.assert_allclose(out["eta2"], eta, rtol=1e-12)


def test_run_ti_mixed_host_logic(oracle, run_job):
    """run_ti_mixed: one batch per bead number, advanced together; Delta A per P
    from the rings of that P, each against the oracle ring by ring."""
    Pr = [8, 16, 8, 16]  # 2 lambda points x 2 replicas, ring r = point * nrep + replica
    out = run_job(dict(kind="ti_mixed", P_per_ring=Pr, nmc=120))
    c = dict(pgconfigs.load("c0"), imin=20, nintegral=2)
    pes = oracle.Pes(c["pes_id"], c["ndim"], c["natom"], c["params"])
    got = {q["P"]: q for q in out["per_P"]}
    assert sorted(got) == [8, 16] and all(q["nrings"] == 2 for q in got.values())
    for P in (8, 16):
        ti = pgconfigs.TiInputs(dict(c, P=P), nrep=2, nintegral=2, P=P, gauleg=oracle.gauleg)
        prm = oracle.TiParams(P, c["beta"], c["dt"], tau=c["tau"], gamma=c["gamma"], thermostat=2,
                              nm_resident=True, imin=c["imin"], init_sigma=c["init_sigma"])
        ints = {}
        for r in [i for i, p in enumerate(Pr) if p == P]:
            li = int(ti.ring_lambda[r])
            x, p = oracle.ring_init(pes, c["mass"], prm, ti.xref[li], int(ti.ring_seed[r]),
                                    int(ti.ring_stream[r]), a=ti.a, b=ti.b[li])
            res = oracle.ring_propagate(pes, c["mass"], prm, ti.a, ti.b[li], ti.dbdl[li], ti.xref[li],
                                        int(ti.ring_seed[r]), int(ti.ring_stream[r]), 0, 120, x, p)
            ints.setdefault(li, []).append(res.dhdr_sum / res.nsamples / ti.betan ** 2)
        dA = sum(ti.w[li] * np.mean(v) for li, v in ints.items())
        assert got[P]["dA"] == pytest.approx(dA, rel=1e-12)


def test_run_ti_readhess_host_logic(oracle, run_job, tmp_path):
    """run_ti(readhess=True): the start positions handed to the batch are the
    path beads of each ring's lambda point plus the readhess displacements of
    the polymer Hessian there (pg_um_hessian, singlewell false, betan =
    beta/(P+1)) with normals from the ring's own Philox stream."""
    import drivers
    out = run_job(dict(kind="ti_readhess"), env=dict(PG_STANDIN_X0=str(tmp_path / "x0.txt")))
    assert np.isfinite(out["dA"])
    c = dict(pgconfigs.load("c1"), P=8, imin=0)
    ti = pgconfigs.TiInputs(c, nrep=2, nintegral=2, gauleg=oracle.gauleg)
    pes = oracle.Pes(c["pes_id"], 2, 1, c["params"], V0=c["V0"])
    x0 = np.loadtxt(str(tmp_path / "x0.txt")).reshape(ti.nrings, -1)
    for r in range(ti.nrings):
        li = int(ti.ring_lambda[r])
        band = oracle.UMhessian(pes, c["mass"], ti.P, ti.betan, ti.xref[li])
        z = np.random.Generator(np.random.Philox(key=int(ti.ring_seed[r]), counter=[int(ti.ring_stream[r]), 49, 0,
                                                                                      0])).standard_normal(2 * ti.P)
        dx = drivers.readhess_displacements(band, ti.P, 2, 1, c["mass"], c["beta"], z[None, :])[0]
        np.testing.assert_allclose(x0[r], ti.xref[li] + dx, rtol=0, atol=1e-12)
    assert not np.allclose(x0[0], x0[1])


def test_run_rpi_path_guess_host_logic(oracle, run_job):
    """run_rpi(path=frames): the frames of a 3-D system aligned by the first
    frame's angles, splined against normalised arc length, N beads at
    (k-1)/(N-1) (instantonmod.f90:916-950, rpi_ser.f90:133-146)."""
    import align
    c = pgconfigs.load("c3")
    w1, w2 = np.array(c["well1"]), np.array(c["well2"])
    rng = np.random.default_rng(9)
    frames = [w1, 0.5 * (w1 + w2) + 0.05 * rng.normal(size=27), w2]
    N, betas = 6, [c["betas"][3]]
    out = run_job(dict(kind="rpi_path", frames=[list(f) for f in frames], N=N, betas=betas))
    fr = np.array(align.align_frames(frames))
    lam = np.concatenate([[0.0], np.cumsum(np.linalg.norm(np.diff(fr, axis=0), axis=1))])
    lam /= lam[-1]
    x = np.concatenate([[oracle.splint(lam, fr[:, d], oracle.spline(lam, fr[:, d]), t)
                         for t in np.arange(N) / (N - 1)] for d in range(27)])
    np.testing.assert_allclose(out["x"], x, rtol=0, atol=1e-12)
    pes = oracle.Pes(c["pes_id"], 3, 9, c["params"], V0=c["V0"])
    vmin = min(0.0, min(pes.V(x.reshape(27, N)[:, b]) for b in range(N)))
    betan = betas[0] / N
    S = betan * (oracle.UM(pes, c["mass"], N, betan, x, w1, w2) - N * vmin)
    assert out["S"][0] == pytest.approx(S, rel=1e-12)


def test_run_ti_path_flow_matches_the_namelist_driver(oracle, run_job, tmp_path):
    """run_ti(frames=..., instapath=True, centre=True, init='path') and the
    namelist driver with readpath / instapath / centre build the same batch:
    both through the stand-in, Delta A agrees to round-off."""
    import standin
    c = pgconfigs.load("c1")
    m1, m2 = np.array(c["well1"]), np.array(c["well2"])
    f1, f2 = m1 + 0.1 * (m2 - m1), m2 - 0.1 * (m2 - m1)
    P, nmc, imin = 24, 30, 10
    out = run_job(dict(kind="ti_path", frames=[list(f1), list(f2)], P=P, nmc=nmc, imin=imin))
    exe = standin.build_driver("pimd_ti", tmp_path)
    (tmp_path / "masses.dat").write_text("H %.17g\n" % c["mass"][0])
    for name, w in (("well1", m1), ("well2", m2)):
        (tmp_path / (name + ".dat")).write_text("%.17g %.17g\n" % tuple(w))
    (tmp_path / "pes.dat").write_text("\n".join("%.17g" % v for v in c["params"]) + "\n")
    (tmp_path / "path.xyz").write_text("".join(" 1\n frame %d\n H %.17g %.17g\n" % (i, *w) for i, w in
                                               enumerate((f1, f2))))
    text = ("&MCDATA n=%d, beta=%.17g, NMC=%d, dt=%.17g, imin=%d, tau=1.0, gamma=%.17g, nintegral=3,\n"
            " nrep=2, thermostat=2, ndim=2, natom=1, readpath=T, npath=2, instapath=T, centre=T,\n"
            " pes='2dtest', pes_params='pes.dat', precision='fp64', form='fused', init='path',\n"
            " init_sigma=%.17g, seed=0 /\n" % (P, c["beta"], nmc, c["dt"], imin, c["gamma"], c["init_sigma"]))
    r = subprocess.run([exe], input=text, capture_output=True, text=True, cwd=str(tmp_path), timeout=300)
    assert r.returncode == 0, r.stderr
    dA = float(__import__("re").search(r"final Delta A=\s*(\S+)", r.stdout).group(1))
    assert out["dA"] == pytest.approx(dA, rel=1e-12)


def test_run_ti_restart_files(oracle, run_job, tmp_path):
    """run_ti(restart=1) writes the restart_proc files the namelist driver writes
    for the same batch (same numbers, same layout); run_ti(restart=2) continues
    from them: 150 + 150 steps equal one 300-step run."""
    import re
    import standin
    c = dict(pgconfigs.load("c0"), imin=50, P=16)
    py_dir, cc_dir, one_dir = tmp_path / "py", tmp_path / "cc", tmp_path / "one"
    for d in (py_dir, cc_dir, one_dir):
        d.mkdir()
    run_job(dict(kind="ti_restart", nmc=150, restart=1, dir=str(py_dir)))
    exe = standin.build_driver("pimd_ti", tmp_path)
    (cc_dir / "masses.dat").write_text("H %.17g\n" % c["mass"][0])
    (cc_dir / "well1.dat").write_text("%.17g\n" % c["well1"][0])
    (cc_dir / "well2.dat").write_text("%.17g\n" % c["well2"][0])
    (cc_dir / "pes.dat").write_text("\n".join("%.17g" % v for v in c["params"]) + "\n")
    text = ("&MCDATA n=16, beta=%.17g, NMC=150, dt=%.17g, imin=50, tau=%.17g, gamma=%.17g, nintegral=%d,\n"
            " nrep=3, thermostat=2, ndim=1, natom=1, readpath=F, pes='1d', pes_params='pes.dat',\n"
            " precision='fp64', form='fused', init='well', init_sigma=%.17g, seed=0, restart=1, nproc=2 /\n"
            % (c["beta"], c["dt"], c["tau"], c["gamma"], c["nintegral"], c["init_sigma"]))
    r = subprocess.run([exe], input=text, capture_output=True, text=True, cwd=str(cc_dir), timeout=300)
    assert r.returncode == 0, r.stderr
    names = sorted(p.name for p in cc_dir.glob("restart_proc*.xyz"))
    assert names == sorted(p.name for p in py_dir.glob("restart_proc*.xyz")) and len(names) == 3 * c["nintegral"]
    for name in names:
        a, b = (cc_dir / name).read_text().split(), (py_dir / name).read_text().split()
        assert len(a) == len(b)
        for u, v in zip(a, b):
            if re.fullmatch(r"[A-Za-z]+", u):
                assert u == v
            else:
                # the namelist driver's end points come from a spline through the two wells,
                # the Python driver's from the straight line: round-off apart
                assert float(u) == pytest.approx(float(v), rel=1e-9, abs=1e-12)
    two_legs = run_job(dict(kind="ti_restart", nmc=150, restart=2, dir=str(cc_dir)))["dA"]
    one = run_job(dict(kind="ti_restart", nmc=300, restart=0, dir=str(one_dir)))["dA"]
    assert two_legs == pytest.approx(one, rel=1e-8)


def test_run_ti_resumes_after_a_failed_run(oracle, run_job, tmp_path):
    """run_ti(restart=1) with noutput = 100 writes the restart files before steps
    100 and 200; a run that fails at step 250 (injected on the host through the
    stand-in) resumes from them (restart=2) and matches an uninterrupted run."""
    run_dir, ref_dir = tmp_path / "run", tmp_path / "ref"
    run_dir.mkdir()
    ref_dir.mkdir()
    with pytest.raises(AssertionError, match="pg_ti_advance|pimdgpu error"):
        run_job(dict(kind="ti_restart", nmc=300, restart=1, noutput=100, dir=str(run_dir)),
                env=dict(PG_STANDIN_FAIL_AT="250"))
    lines = (run_dir / "restart_proc0_1.xyz").read_text().split("\n")
    assert lines[16 * 3 + 1].strip() == "199"
    resumed = run_job(dict(kind="ti_restart", nmc=101, restart=2, noutput=100, dir=str(run_dir)))["dA"]
    whole = run_job(dict(kind="ti_restart", nmc=300, restart=0, dir=str(ref_dir)))["dA"]
    assert resumed == pytest.approx(whole, rel=1e-8)


def test_run_ti_reports_a_nan_ring(oracle, run_job):
    """A NaN written into ring 1's start (lambda point 0, replica 1) on the host:
    run_ti reports it and its lambda point's mean is that of the other ring."""
    clean = run_job(dict(kind="ti", nmc=300))
    out = run_job(dict(kind="ti", nmc=300), env=dict(PG_STANDIN_NAN_RING="1"))
    assert clean["nan_rings"] == 0 and out["nan_rings"] == 1
    assert out["mean"][1:] == clean["mean"][1:]
    c = dict(pgconfigs.load("c0"), imin=50)
    ti = pgconfigs.TiInputs(dict(c, nrep=2, seeds=[0, 1]), gauleg=oracle.gauleg)
    pes = oracle.Pes(c["pes_id"], 1, 1, c["params"])
    prm = oracle.TiParams(ti.P, c["beta"], c["dt"], tau=c["tau"], gamma=c["gamma"], thermostat=2,
                          nm_resident=True, imin=50, init_sigma=c["init_sigma"])
    x, p = oracle.ring_init(pes, c["mass"], prm, ti.xref[0], 0, 0, a=ti.a, b=ti.b[0])
    res = oracle.ring_propagate(pes, c["mass"], prm, ti.a, ti.b[0], ti.dbdl[0], ti.xref[0], 0, 0, 0, 300, x, p)
    assert out["mean"][0] == pytest.approx(res.dhdr_sum / res.nsamples / ti.betan ** 2, rel=1e-12)


@pytest.mark.parametrize("cfg,npts", [("c3", 2), ("c1", 4)])
def test_run_rpi_angular_matches_the_namelist_driver(oracle, run_job, tmp_path, cfg, npts):
    """run_rpi_angular and rpi.cpp with angular = T give the same angularI.dat
    rows (3-D: c3's 9-atom surface; 2-D: c1), both through the stand-in."""
    import standin
    c = pgconfigs.load(cfg)
    n, beta, ct, cp = 4, 40.0, 1.0, 0.5
    out = run_job(dict(kind="angular", cfg=cfg, N=n, beta=beta, npoints=npts, ct=ct, cp=cp))
    exe = standin.build_driver("rpi", tmp_path)
    natom, ndim = c["natom"], c["ndim"]
    (tmp_path / "masses.dat").write_text("".join("X%d %.17g\n" % (j, mm) for j, mm in enumerate(c["mass"])))
    for name in ("well1", "well2"):
        w = np.array(c[name]).reshape(natom, ndim)
        (tmp_path / (name + ".dat")).write_text("".join(" ".join("%.17g" % v for v in row) + "\n" for row in w))
    (tmp_path / "pes.dat").write_text("\n".join("%.17g" % v for v in c["params"]) + "\n")
    text = ("&RPIDATA n=%d, beta=%.17g, ndim=%d, natom=%d, readpath=.false., pes='%s', pes_params='pes.dat',\n"
            " angular=.true., npoints=%d, cutofftheta=%.17g, cutoffphi=%.17g /\n"
            % (n, beta, ndim, natom, "synth9" if cfg == "c3" else "2dtest", npts, ct, cp))
    r = subprocess.run([exe], input=text, capture_output=True, text=True, cwd=str(tmp_path), timeout=300)
    assert r.returncode == 0, r.stderr
    rows = np.loadtxt(str(tmp_path / "angularI.dat"))
    np.testing.assert_allclose(np.array(out["rows"]), rows, rtol=1e-12, atol=1e-300)
