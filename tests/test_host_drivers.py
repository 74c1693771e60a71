"""The C++ namelist drivers (pimd_par.f90 / rpi_ser.f90 front ends).

CPU: namelist parsing in the reference's syntax and the loud failure without a
GPU.  GPU: the drivers reproduce the Python driver on the same inputs."""
import json
import os
import re
import subprocess

import numpy as np
import pytest

import pgconfigs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "pimd-tunneling_gb300", "lib")


@pytest.fixture(scope="module")
def drivers_built(pg):
    return LIB


def _run(exe, text, cwd=None, args=()):
    return subprocess.run([os.path.join(LIB, exe)] + list(args), input=text, capture_output=True, text=True,
                          cwd=cwd, timeout=600)


def test_mcdata_namelist_parsing(drivers_built):
    text = ("&MCDATA n=32, beta=538.47d0, NMC=2e4, Noutput=1e5, dt=2.76D-2, iprint=.false., imin=1000,\n"
            " tau=1.0, gamma=0.36, nintegral=11, nrep=1, thermostat=2, ndim=1, natom=1,\n"
            " readpath=F, cayley=.TRUE., pes='1d', precision='fp64' ! comment\n/\n")
    r = _run("pimd_ti", text, args=["--parse-only"])
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout)
    assert d["n"] == 32 and d["NMC"] == 20000 and d["Noutput"] == 100000
    assert abs(d["beta"] - 538.47) < 1e-12 and abs(d["dt"] - 0.0276) < 1e-15
    assert d["readpath"] is False and d["cayley"] is True and d["thermostat"] == 2
    assert d["pes"] == "1d" and d["precision"] == "fp64" and d["imin"] == 1000
    assert d["tune"] == "" and d["readhess"] is False
    r = _run("pimd_ti", "&MCDATA n=16, tune='tune.jsonl' /", args=["--parse-only"])
    assert json.loads(r.stdout)["tune"] == "tune.jsonl"
    # reference defaults (pimd_par.f90:60-88) for keys not given
    r = _run("pimd_ti", "&MCDATA /", args=["--parse-only"])
    d = json.loads(r.stdout)
    assert d["n"] == 100 and d["NMC"] == 5000000 and d["thermostat"] == 1 and d["ndim"] == 3


def test_readhess_size_limit_of_the_namelist_driver(drivers_built, tmp_path):
    """readhess diagonalises the polymer Hessian on the host (Jacobi): larger
    polymers are refused before any device work, pointing to the Python driver."""
    r = _run("pimd_ti", "&MCDATA n=1000, ndim=3, natom=9, readhess=.true. /", cwd=str(tmp_path))
    assert r.returncode == 1
    assert "readhess" in r.stderr and "Python driver" in r.stderr


def test_rpidata_namelist_parsing(drivers_built):
    r = _run("rpi", "&RPIDATA n=512, beta=3157.75, ndim=3, natom=9, readpath=.false., pes='synth9', m=10 /",
             args=["--parse-only"])
    d = json.loads(r.stdout)
    assert d["n"] == 512 and d["natom"] == 9 and d["readpath"] is False and d["m"] == 10
    assert d["pgtol"] == 1e-5 and d["factr"] == 1e6
    assert d["checkhess"] is False and d["output_instanton"] is False and d["alignwell"] is False


def test_namelist_errors_stop_the_run(drivers_built):
    """As a Fortran namelist read does: an unknown key or a value that does not
    convert stops the program before any work; '&end' also closes a group, and
    the reference keys without effect here are accepted."""
    r = _run("pimd_ti", "&MCDATA n=8, NMCC=100 /", args=["--parse-only"])
    assert r.returncode == 1 and "unknown key 'nmcc'" in r.stderr
    r = _run("pimd_ti", "&MCDATA n=8, beta=1.0x /", args=["--parse-only"])
    assert r.returncode == 1 and "beta" in r.stderr and "not a number" in r.stderr
    r = _run("pimd_ti", "&MCDATA cayley=yes /", args=["--parse-only"])
    assert r.returncode == 1 and "not a logical" in r.stderr
    r = _run("pimd_ti", "&MCDATA n=12, use_mkl=.false., basename='w' &end", args=["--parse-only"])
    assert r.returncode == 0, r.stderr
    assert json.loads(r.stdout)["n"] == 12
    r = _run("rpi", "&RPIDATA n=12, alignpath=.true., fixedends=.false. /", args=["--parse-only"])
    assert r.returncode == 0, r.stderr
    assert json.loads(r.stdout)["fixedends"] is False
    r = _run("rpi", "&RPIDATA fixedends=.false., angular=.true. /", args=["--parse-only"])
    assert json.loads(r.stdout)["fixedends"] is True  # rpi_ser.f90:53
    r = _run("crossover", "&CROSSDATA ndim=2, natom=1, nmc=3 /", args=["--parse-only"])
    assert r.returncode == 1 and "unknown key 'nmc'" in r.stderr
    # values out of range stop the programs with every problem named
    r = _run("pimd_ti", "&MCDATA n=1, dt=-0.1, thermostat=3 /", args=["--parse-only"])
    assert r.returncode == 1
    assert all(w in r.stderr for w in ("n (beads)", "dt must be positive", "thermostat must be"))
    r = _run("rpi", "&RPIDATA n=100, beta=0 /", args=["--parse-only"])
    assert r.returncode == 1 and "beta must be positive" in r.stderr


def test_driver_fails_loudly_without_gpu(drivers_built, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    (tmp_path / "masses.dat").write_text("H 1836.15\n")
    (tmp_path / "well1.dat").write_text("-1.0\n")
    (tmp_path / "well2.dat").write_text("1.0\n")
    r = _run("pimd_ti", "&MCDATA n=8, ndim=1, natom=1, nintegral=2, NMC=10, pes='1d' /", cwd=str(tmp_path))
    assert r.returncode == 2
    assert "no CPU fallback" in r.stderr


def _write_inputs(tmp_path, c, labels):
    nd = c["ndim"]
    (tmp_path / "masses.dat").write_text("".join("%s %.17g\n" % (l, m) for l, m in zip(labels, c["mass"])))
    for name in ("well1", "well2"):
        w = np.array(c[name]).reshape(c["natom"], nd)
        (tmp_path / (name + ".dat")).write_text("".join(" ".join("%.17g" % v for v in row) + "\n" for row in w))
    (tmp_path / "pes.dat").write_text("\n".join("%.17g" % v for v in c["params"]) + "\n")


@pytest.mark.gpu
def test_pimd_ti_driver_matches_python_driver(drivers_built, tmp_path):
    import drivers
    import pimdgpu as pg
    c = dict(pgconfigs.load("c0"))
    _write_inputs(tmp_path, c, ["H"])
    text = ("&MCDATA n=%d, beta=%.17g, NMC=2000, dt=%.17g, imin=%d, tau=%.17g, gamma=%.17g, nintegral=%d,\n"
            " nrep=1, thermostat=2, ndim=1, natom=1, readpath=F, pes='1d', pes_params='pes.dat',\n"
            " precision='fp64', form='fused', init='well', init_sigma=%.17g, seed=0 /\n"
            % (c["P"], c["beta"], c["dt"], c["imin"], c["tau"], c["gamma"], c["nintegral"], c["init_sigma"]))
    r = _run("pimd_ti", text, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    dA = float(re.search(r"final Delta A=\s*(\S+)", r.stdout).group(1))
    ref = drivers.run_ti(c, precision=pg.PG_FP64, form=pg.PG_FORM_FUSED, nmc=2000)
    assert abs(dA - ref["dA"]) <= 1e-12 * abs(ref["dA"])


@pytest.mark.gpu
def test_rpi_driver_matches_python_driver(drivers_built, tmp_path):
    import drivers
    c = dict(pgconfigs.load("c3"))
    _write_inputs(tmp_path, c, ["O", "O", "C", "C", "C", "H", "H", "H", "H"])
    beta = c["betas"][5]
    text = ("&RPIDATA n=64, beta=%.17g, ndim=3, natom=9, readpath=.false., pes='synth9', pes_params='pes.dat',\n"
            " m=10, pgtol=1d-8, factr=1d2 /\n" % beta)
    r = _run("rpi", text, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    S = float(re.search(r"s_kink=\s*(\S+)", r.stdout).group(1))
    ref = drivers.run_rpi(c, N=64, betas=[beta], m=10, factr=1e2, pgtol=1e-8)["results"][0]
    assert abs(S - ref["S"]) <= 1e-10 * abs(ref["S"])


@pytest.mark.gpu
def test_rpi_driver_free_ends_match_python_driver_and_scipy(drivers_built, tmp_path, oracle):
    """fixedends = .false. (rpi_ser.f90:39, 370-374): both front ends optimise the
    free-ended action (instanton(xtilde)) and report S = betan UM(xtilde); they
    agree to round-off, and S matches scipy L-BFGS-B on the oracle's free-ended
    action from the same linear start to 1e-8."""
    import drivers
    c = dict(pgconfigs.load("c3"))
    _write_inputs(tmp_path, c, ["O", "O", "C", "C", "C", "H", "H", "H", "H"])
    beta, n = c["betas"][5], 32
    text = ("&RPIDATA n=%d, beta=%.17g, ndim=3, natom=9, readpath=.false., pes='synth9', pes_params='pes.dat',\n"
            " m=10, pgtol=1d-9, factr=1d2, fixedends=.false. /\n" % (n, beta))
    r = _run("rpi", text, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    S = float(re.search(r"s_kink=\s*(\S+)", r.stdout).group(1))
    ref = drivers.run_rpi(c, N=n, betas=[beta], m=10, factr=1e2, pgtol=1e-9, fixedends=False)
    assert abs(S - ref["results"][0]["S"]) <= 1e-12 * abs(S)
    assert ref["results"][0]["status"] == 0
    fixed = drivers.run_rpi(c, N=n, betas=[beta], m=10, factr=1e2, pgtol=1e-9)["results"][0]["S"]
    pes = oracle.Pes(c["pes_id"], c["ndim"], c["natom"], c["params"], V0=c["V0"])
    w1, w2 = np.array(c["well1"]), np.array(c["well2"])
    k = np.arange(1, n + 1)
    x0 = np.concatenate([((n - k) * w1[d] + (k - 1) * w2[d]) / (n - 1) for d in range(len(w1))])
    _, fo, _ = oracle.instanton_lbfgs(pes, np.array(c["mass"]), n, beta / n, x0, None, None, m=10, factr=1e2,
                                      pgtol=1e-9, maxiter=200000, fixedends=False)
    vmin = min(float(np.min(ref["vpath"])), 0.0)
    assert abs(S - (beta / n) * (fo - n * vmin)) <= 1e-8 * abs(S)
    # the free-ended optimum differs from the fixed-ended one (no end springs)
    assert S != fixed


@pytest.mark.gpu
def test_rpi_driver_side_outputs(drivers_built, tmp_path):
    """checkhess (hessian_well1.dat and the mass-weighted eigenvalues,
    rpi_ser.f90:105-129), instanton.xyz with the bead energies and
    instantonpathenergy.csv (rpi_ser.f90:180-218).  Both front ends set
    V0 = V(well1) on the device (rpi_ser.f90:95), so they hand the optimiser
    bit-identical inputs and reach the same path: the bead energies agree to
    round-off, and the checkhess branch leaves the instanton unchanged (byte-
    identical instanton.xyz with and without it)."""
    import drivers
    import pimdgpu as pg
    c = dict(pgconfigs.load("c3"))
    _write_inputs(tmp_path, c, ["O", "O", "C", "C", "C", "H", "H", "H", "H"])
    beta, n, nd = c["betas"][5], 64, 27
    text = ("&RPIDATA n=%d, beta=%.17g, ndim=3, natom=9, readpath=.false., pes='synth9', pes_params='pes.dat',\n"
            " m=10, pgtol=1d-8, factr=1d2, checkhess=.true. /\n" % (n, beta))
    r = _run("rpi", text, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    w1 = np.array(c["well1"])
    ctx = pg.Context(0)
    try:
        ctx.set_system(c["ndim"], c["natom"], c["mass"], c["pes_id"], c["params"], c["V0"])
        H = ctx.pes_hessian(w1)[0]
    finally:
        ctx.close()
    Hf = np.loadtxt(str(tmp_path / "hessian_well1.dat"))
    np.testing.assert_allclose(Hf, H, rtol=1e-14, atol=1e-16)
    s = 1.0 / np.sqrt(np.repeat(c["mass"], 3))
    eta = np.linalg.eigvalsh(H * s[:, None] * s[None, :]) * 219475.0
    modes = re.search(r"normal modes:\n((?:\s*\d+\s+\S+\n){%d})" % nd, r.stdout).group(1).split()
    np.testing.assert_allclose(np.array(modes[1::2], float), eta, rtol=0, atol=1e-10 * np.max(np.abs(eta)))
    ref = drivers.run_rpi(c, N=n, betas=[beta], m=10, factr=1e2, pgtol=1e-8)
    lines = (tmp_path / "instanton.xyz").read_text().split("\n")
    assert len([l for l in lines if l.strip()]) == n * (2 + 9)
    energies = np.array([float(lines[b * 11 + 1].split()[-1]) for b in range(n)])
    np.testing.assert_allclose(energies, ref["vpath"][0], rtol=1e-12, atol=1e-20)
    lam, vp = np.loadtxt(str(tmp_path / "instantonpathenergy.csv"), unpack=True)
    assert lam[0] == 0.0 and lam[-1] == pytest.approx(1.0) and np.all(np.diff(lam) > 0)
    np.testing.assert_allclose(vp, energies, rtol=1e-15, atol=0)
    plain = tmp_path / "no_checkhess"
    plain.mkdir()
    _write_inputs(plain, c, ["O", "O", "C", "C", "C", "H", "H", "H", "H"])
    r2 = _run("rpi", text.replace(", checkhess=.true.", ""), cwd=str(plain))
    assert r2.returncode == 0, r2.stderr
    assert (plain / "instanton.xyz").read_bytes() == (tmp_path / "instanton.xyz").read_bytes()


@pytest.mark.gpu
def test_pimd_ti_restart_files_roundtrip(drivers_built, tmp_path):
    """restart = 1 writes the reference's restart_proc<iproc>_<ii>.xyz files (two
    ranks' worth here); restart = 2 without restart.ckpt reads them back: with
    NMC = 0 the answer is unchanged, and 200 + 200 steps through the files match
    one 400-step run."""
    c = dict(pgconfigs.load("c0"))
    _write_inputs(tmp_path, c, ["H"])

    def text(nmc, restart):
        return ("&MCDATA n=16, beta=%.17g, NMC=%d, dt=%.17g, imin=50, tau=1.0, gamma=%.17g, nintegral=2,\n"
                " nrep=3, thermostat=2, ndim=1, natom=1, readpath=F, pes='1d', pes_params='pes.dat',\n"
                " precision='fp64', form='fused', init='well', init_sigma=0.01, seed=0, restart=%d, nproc=2 /\n"
                % (c["beta"], nmc, c["dt"], c["gamma"], restart))

    def dA(out):
        return float(re.search(r"final Delta A=\s*(\S+)", out).group(1))

    r = _run("pimd_ti", text(200, 1), cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    names = sorted(p.name for p in tmp_path.glob("restart_proc*.xyz"))
    assert names == ["restart_proc0_1.xyz", "restart_proc0_2.xyz", "restart_proc0_3.xyz",
                     "restart_proc1_1.xyz", "restart_proc1_2.xyz", "restart_proc1_3.xyz"]
    lines = (tmp_path / "restart_proc0_1.xyz").read_text().split("\n")
    assert lines[0].strip() == "1" and lines[2].split()[0] == "H" and len(lines) == 2 * 16 * 3 + 1
    assert lines[16 * 3 + 1].strip() == "200"  # step count of the momentum block
    first = dA(r.stdout)
    (tmp_path / "restart.ckpt").unlink()
    r = _run("pimd_ti", text(0, 2), cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    assert abs(dA(r.stdout) - first) <= 1e-14 * abs(first)
    (tmp_path / "restart.ckpt").unlink()
    r = _run("pimd_ti", text(200, 2), cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    two_legs = dA(r.stdout)
    other = tmp_path / "one"
    other.mkdir()
    _write_inputs(other, c, ["H"])
    r = _run("pimd_ti", text(400, 0), cwd=str(other))
    assert r.returncode == 0, r.stderr
    assert abs(two_legs - dA(r.stdout)) <= 1e-8 * abs(dA(r.stdout))


@pytest.mark.gpu
def test_pimd_ti_instanton_path_and_centre(drivers_built, tmp_path):
    """readpath + instapath + centre (instantonmod.f90:895-1004) on the 2-D
    surface: the instanton between adjacent wells is optimised on the GPU,
    written to instanton.xyz, and the path is centred on its barrier top, which
    the reflection symmetry of the surface puts at lambda = 1/2."""
    c = dict(pgconfigs.load("c1"))
    _write_inputs(tmp_path, c, ["H"])
    w1, w2 = np.array(c["well1"]), np.array(c["well2"])
    (tmp_path / "path.xyz").write_text("".join(" 1\n frame %d\n H %.17g %.17g\n" % (i, *w) for i, w in
                                               enumerate((w1, w2))))
    n = 24
    text = ("&MCDATA n=%d, beta=%.17g, NMC=100, dt=%.17g, imin=10, tau=1.0, gamma=%.17g, nintegral=3,\n"
            " nrep=2, thermostat=2, ndim=2, natom=1, readpath=T, npath=2, instapath=T, centre=T,\n"
            " pes='2dtest', pes_params='pes.dat', precision='fp64', form='fused', init='path', seed=0 /\n"
            % (n, c["beta"], c["dt"], c["gamma"]))
    r = _run("pimd_ti", text, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    assert "Found instanton" in r.stdout
    lines = (tmp_path / "instanton.xyz").read_text().strip().split("\n")
    assert len(lines) == 3 * n
    beads = np.array([[float(v) for v in lines[3 * i + 2].split()[1:]] for i in range(n)]) / 0.529177
    # the optimised path is mirror-symmetric: bead i and bead n-1-i reflect into each other
    mid = 0.5 * (w1 + w2)
    u = (w2 - w1) / np.linalg.norm(w2 - w1)
    refl = beads - 2.0 * np.outer((beads - mid) @ u, u)
    assert np.max(np.abs(refl[::-1] - beads)) < 1e-4
    xm = float(re.search(r"Centred,\s*\S+\s+\S+\s+(\S+)", r.stdout).group(1))
    assert abs(xm - 0.5) < 1e-4
    assert np.isfinite(float(re.search(r"final Delta A=\s*(\S+)", r.stdout).group(1)))


@pytest.mark.gpu
def test_rpi_angular_grid_batch_matches_single_solves(drivers_built, tmp_path):
    """angular = T (rpi_ser.f90:241-348) on the 2-D surface: every orientation of
    well 2 is re-optimised in one batched call; each row of angularI.dat equals an
    independent single-orientation solve through the Python binding."""
    import drivers
    import pimdgpu as pg
    c = dict(pgconfigs.load("c1"))
    _write_inputs(tmp_path, c, ["H"])
    N, npts = 16, 3
    beta = c["beta"]
    text = ("&RPIDATA n=%d, beta=%.17g, ndim=2, natom=1, readpath=.false., pes='2dtest', pes_params='pes.dat',\n"
            " angular=.true., npoints=%d /\n" % (N, beta, npts))
    r = _run("rpi", text, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    rows = np.loadtxt(tmp_path / "angularI.dat")
    assert rows.shape == (npts, 3)
    assert abs(rows[:, 1].sum() - 2.0 * 3.14159265358979) < 1e-12
    betan = beta / N
    w1, w2 = np.array(c["well1"]), np.array(c["well2"])
    with pg.Context(0) as ctx:
        ctx.set_system(c["ndim"], c["natom"], c["mass"], c["pes_id"], c["params"], c["V0"])
        kw = dict(m=8, factr=1e6, pgtol=1e-5, maxiter=200000)
        x, _, _, _ = ctx.instanton_optimize(N, drivers.linear_guess(w1, w2, N), w1, w2, [betan], **kw)
        ld0, _, _ = ctx.instanton_logdet(N, np.repeat(w1, N), [betan], singlewell=True, skip_lowest=False)
        eta, _ = pg.gauleg(0.0, 2.0 * 3.14159265358979, npts)
        for k in range(npts):
            cth, sth = np.cos(eta[k]), np.sin(eta[k])
            b = np.array([cth * w2[0] + sth * w2[1], -sth * w2[0] + cth * w2[1]])
            xk, UM, _, st = ctx.instanton_optimize(N, x, w1, b, [betan], **kw)
            ld, _, _ = ctx.instanton_logdet(N, xk, [betan], singlewell=False, skip_lowest=True)
            S, om, _ = pg.rpi_assemble(betan, UM[0], ld[0], ld0[0])
            assert abs(rows[k, 0] - eta[k]) < 1e-14
            np.testing.assert_allclose(rows[k, 2], np.tanh(om * N), rtol=1e-9, atol=1e-300)


def test_rpi_driver_host_logic_on_the_oracle(oracle, tmp_path):
    """rpi.cpp end to end on the CPU, linked against the oracle-backed stand-in
    for its C-ABI calls (tests/standin; its optimiser returns the start path
    unchanged): checkhess output, instanton.xyz / instantonpathenergy.csv, and
    the action after V0 moves to the lowest bead (rpi_ser.f90:105-129, 180-218,
    368-381).  Well 1 lies 0.3 bohr beyond a minimum of the 2-D surface, so the
    straight start path passes below it."""
    import standin
    exe = standin.build_driver("rpi", tmp_path)
    c = pgconfigs.load("c1")
    m1, m2 = np.array(c["well1"]), np.array(c["well2"])
    u = (m1 - m2) / np.linalg.norm(m1 - m2)
    w1, w2 = m1 + 0.3 * u, m2
    cc = dict(c, well1=list(w1), well2=list(w2))
    _write_inputs(tmp_path, cc, ["H"])
    n, beta = 8, c["beta"] / 16
    text = ("&RPIDATA n=%d, beta=%.17g, ndim=2, natom=1, readpath=.false., pes='2dtest', pes_params='pes.dat',\n"
            " checkhess=.true. /\n" % (n, beta))
    r = subprocess.run([exe], input=text, capture_output=True, text=True, cwd=str(tmp_path), timeout=120)
    assert r.returncode == 0, r.stderr
    v0 = oracle.Pes(oracle.PES_2DTEST, 2, 1, c["params"]).V(w1)
    pes = oracle.Pes(oracle.PES_2DTEST, 2, 1, c["params"], V0=v0)
    k = np.arange(1, n + 1)
    x = np.concatenate([((n - k) * w1[d] + (k - 1) * w2[d]) / (n - 1) for d in range(2)])  # rpi_ser.f90:157-163
    vpath = np.array([pes.V(x.reshape(2, n)[:, b]) for b in range(n)])
    vmin = vpath.min()
    assert vmin < 0
    assert float(re.search(r"New V0=\s*(\S+)", r.stdout).group(1)) == pytest.approx(v0 + vmin, rel=1e-12)
    betan, mass = beta / n, c["mass"]
    UM = oracle.UM(pes, mass, n, betan, x, w1, w2) - n * vmin
    ld0 = oracle.logdet_band(oracle.UMhessian(pes, mass, n, betan, np.repeat(w1, n), singlewell=True), False)[0]
    ld = oracle.logdet_band(oracle.UMhessian(pes, mass, n, betan, x), True)[0]
    S = betan * UM
    om = betan * np.exp(-S) * np.sqrt(S / (2 * oracle.PI_REF)) / np.exp(0.5 * (ld - ld0))
    assert float(re.search(r"s_kink=\s*(\S+)", r.stdout).group(1)) == pytest.approx(S, rel=1e-12)
    delta = re.search(r"RPI delta=\s*(\S+)", r.stdout).group(1)
    assert float(delta) == pytest.approx(2 * om / betan, rel=1e-8)
    # instanton.xyz (Angstrom, padded to three coordinates) and instantonpathenergy.csv
    lines = (tmp_path / "instanton.xyz").read_text().split("\n")
    energies = np.array([float(lines[3 * b + 1].split()[-1]) for b in range(n)])
    np.testing.assert_allclose(energies, vpath, rtol=1e-14, atol=1e-16)
    xyz = np.array([list(map(float, lines[3 * b + 2].split()[1:])) for b in range(n)])
    np.testing.assert_allclose(xyz[:, :2] / 0.529177, x.reshape(2, n).T, rtol=1e-14)
    assert np.all(xyz[:, 2] == 0.0)
    lam, vp = np.loadtxt(str(tmp_path / "instantonpathenergy.csv"), unpack=True)
    np.testing.assert_allclose(lam, (k - 1) / (n - 1), atol=1e-14)  # equally spaced straight path
    np.testing.assert_array_equal(vp, energies)
    # aligned.xyz: the linear start path (rpi_ser.f90:164-172)
    al = (tmp_path / "aligned.xyz").read_text().strip().split("\n")
    assert al[1].strip() == "Energy of minimum 1"
    np.testing.assert_allclose(np.array([[float(v) for v in al[3 * b + 2].split()[1:]] for b in range(n)]) / 0.529177,
                               x.reshape(2, n).T, rtol=1e-14)
    # checkhess: the Hessian at well 1 and its mass-weighted eigenvalues times 219475
    H = pes.Vdoubleprime(w1)
    np.testing.assert_allclose(np.loadtxt(str(tmp_path / "hessian_well1.dat")), H, rtol=1e-14)
    modes = re.search(r"normal modes:\n\s*1\s+(\S+)\n\s*2\s+(\S+)\n", r.stdout).groups()
    np.testing.assert_allclose(np.array(modes, float), np.linalg.eigvalsh(H / mass[0]) * 219475.0, rtol=1e-10)
    # fixedends = F: the action without the end-point springs (rpi_ser.f90:370-374)
    r = subprocess.run([exe], input=text.replace("checkhess=.true.", "fixedends=.false."), capture_output=True,
                       text=True, cwd=str(tmp_path), timeout=120)
    assert r.returncode == 0, r.stderr
    UMf = oracle.UM(pes, mass, n, betan, x, w1, w2, fixedends=False) - n * vmin
    assert float(re.search(r"s_kink=\s*(\S+)", r.stdout).group(1)) == pytest.approx(betan * UMf, rel=1e-12)


def _oracle_ti(oracle, c, nmc, nm_resident=True, thermostat=2, noutput=100000, dhdr_limit=-1.0):
    """Delta A of the TI batch the driver sets up for c (all beads at well 1,
    seeds 0.., stream = lambda point), by the oracle ring by ring."""
    ti = pgconfigs.TiInputs(c, gauleg=oracle.gauleg)
    pes = oracle.Pes(c["pes_id"], c["ndim"], c["natom"], c["params"])
    prm = oracle.TiParams(ti.P, c["beta"], c["dt"], tau=c["tau"], gamma=c["gamma"], thermostat=thermostat,
                          nm_resident=nm_resident, imin=c["imin"], init_sigma=c["init_sigma"], noutput=noutput,
                          dhdr_limit=dhdr_limit)
    ints = np.zeros(ti.nrings)
    for r in range(ti.nrings):
        li = int(ti.ring_lambda[r])
        x, p = oracle.ring_init(pes, c["mass"], prm, ti.xref[li], int(ti.ring_seed[r]), int(ti.ring_stream[r]),
                                a=ti.a, b=ti.b[li])
        res = oracle.ring_propagate(pes, c["mass"], prm, ti.a, ti.b[li], ti.dbdl[li], ti.xref[li],
                                    int(ti.ring_seed[r]), int(ti.ring_stream[r]), 0, nmc, x, p)
        ints[r] = res.dhdr_sum / res.nsamples / ti.betan ** 2
    mean = np.array([ints[ti.ring_lambda == i].mean() for i in range(ti.nint)])
    return float(np.dot(ti.w, mean))


def _ti_text(c, nmc, nrep, extra=""):
    return ("&MCDATA n=%d, beta=%.17g, NMC=%d, dt=%.17g, imin=%d, tau=%.17g, gamma=%.17g, nintegral=%d,\n"
            " nrep=%d, thermostat=2, ndim=1, natom=1, readpath=F, pes='1d', pes_params='pes.dat',\n"
            " precision='fp64', form='fused', init='well', init_sigma=%.17g, seed=0 %s/\n"
            % (c["P"], c["beta"], nmc, c["dt"], c["imin"], c["tau"], c["gamma"], c["nintegral"], nrep,
               c["init_sigma"], extra))


def test_pimd_ti_driver_host_logic_on_the_oracle(oracle, tmp_path):
    """pimd_ti.cpp end to end on the CPU against the oracle-backed stand-in for
    its C-ABI calls (tests/standin): the lambda points, end points, start
    positions, seeds and streams it sets up, and its assembly of Delta A, agree
    with the oracle run ring by ring on the inputs the Python driver builds."""
    import standin
    exe = standin.build_driver("pimd_ti", tmp_path)
    c = dict(pgconfigs.load("c0"), imin=50)
    _write_inputs(tmp_path, c, ["H"])
    r = subprocess.run([exe], input=_ti_text(c, 300, 2), capture_output=True, text=True, cwd=str(tmp_path),
                       timeout=300)
    assert r.returncode == 0, r.stderr
    dA = float(re.search(r"final Delta A=\s*(\S+)", r.stdout).group(1))
    ref = _oracle_ti(oracle, dict(c, nrep=2, seeds=[0, 1]), 300)
    assert dA == pytest.approx(ref, rel=1e-12)


@pytest.mark.parametrize("extra,kw", [("thermostat=1, Noutput=25 ", dict(thermostat=1, noutput=25)),
                                      ("dHdrlimit=0.02 ", dict(dhdr_limit=0.02))])
def test_pimd_ti_thermostat_keys_on_the_oracle(oracle, tmp_path, extra, kw):
    """The namelist keys thermostat / Noutput (Andersen) and dHdrlimit reach the
    batch: pimd_ti.cpp through the stand-in against the oracle ring by ring."""
    import standin
    exe = standin.build_driver("pimd_ti", tmp_path)
    c = dict(pgconfigs.load("c0"), imin=50)
    _write_inputs(tmp_path, c, ["H"])
    text = _ti_text(c, 300, 2, extra).replace("thermostat=2, ", "" if "thermostat" in extra else "thermostat=2, ")
    r = subprocess.run([exe], input=text, capture_output=True, text=True, cwd=str(tmp_path), timeout=300)
    assert r.returncode == 0, r.stderr
    dA = float(re.search(r"final Delta A=\s*(\S+)", r.stdout).group(1))
    ref = _oracle_ti(oracle, dict(c, nrep=2, seeds=[0, 1]), 300, **kw)
    assert dA == pytest.approx(ref, rel=1e-12)
    assert ref != pytest.approx(_oracle_ti(oracle, dict(c, nrep=2, seeds=[0, 1]), 300), rel=1e-9)  # keys matter


def test_pimd_ti_restart_files_on_the_oracle(oracle, tmp_path):
    """restart = 1 writes restart_proc<iproc>_<ii>.xyz; restart = 2 reads them
    (no checkpoint file in the stand-in) and continues: 150 + 150 steps match
    one 300-step run."""
    import standin
    exe = standin.build_driver("pimd_ti", tmp_path)
    c = dict(pgconfigs.load("c0"), imin=50, P=16)
    _write_inputs(tmp_path, c, ["H"])

    def run(nmc, restart, cwd):
        r = subprocess.run([exe], input=_ti_text(c, nmc, 3, "restart=%d, nproc=2 " % restart),
                           capture_output=True, text=True, cwd=str(cwd), timeout=300)
        assert r.returncode == 0, r.stderr
        return float(re.search(r"final Delta A=\s*(\S+)", r.stdout).group(1))

    run(150, 1, tmp_path)
    names = {p.name for p in tmp_path.glob("restart_proc*.xyz")}
    ntask = c["nintegral"] * 3  # two ranks of ceil(ntask / 2) tasks (pimd_par.f90:109-110)
    assert len(names) == ntask and {"restart_proc0_1.xyz", "restart_proc1_1.xyz"} <= names
    assert "restart_proc0_%d.xyz" % ((ntask + 1) // 2) in names
    two_legs = run(150, 2, tmp_path)
    other = tmp_path / "one"
    other.mkdir()
    _write_inputs(other, c, ["H"])
    one = run(300, 0, other)
    assert two_legs == pytest.approx(one, rel=1e-8)  # the files carry 17 significant digits


def test_pimd_ti_readhess_on_the_oracle(oracle, tmp_path):
    """readhess in the namelist driver (verletmodule.f90:49-88, host Jacobi
    eigensolver), end to end on the CPU against the stand-in: every start
    displacement lies in the span of the positive modes of the polymer Hessian
    at the path beads other than the lowest, with N(0, 1/beta) coefficients,
    and depends only on the ring's seed and stream."""
    import standin
    exe = standin.build_driver("pimd_ti", tmp_path)
    c = pgconfigs.load("c1")
    _write_inputs(tmp_path, c, ["H"])
    n, nint, nrep = 8, 2, 3
    text = ("&MCDATA n=%d, beta=%.17g, NMC=4, dt=%.17g, imin=0, tau=1.0, gamma=%.17g, nintegral=%d, nrep=%d,\n"
            " thermostat=2, ndim=2, natom=1, readpath=F, pes='2dtest', pes_params='pes.dat', precision='fp64',\n"
            " form='fused', init='path', seed=5, readhess=.true. /\n" % (n, c["beta"], c["dt"], c["gamma"], nint, nrep))
    env = dict(os.environ, PG_STANDIN_X0=str(tmp_path / "x0.txt"))
    r = subprocess.run([exe], input=text, capture_output=True, text=True, cwd=str(tmp_path), timeout=300, env=env)
    assert r.returncode == 0, r.stderr
    x0 = np.loadtxt(str(tmp_path / "x0.txt")).reshape(nint * nrep, 2, n)
    ti = pgconfigs.TiInputs(dict(c, P=n, nintegral=nint, nrep=nrep), init="path", gauleg=oracle.gauleg)
    pes = oracle.Pes(oracle.PES_2DTEST, 2, 1, c["params"], V0=c["V0"])
    betan, m = c["beta"] / (n + 1), c["mass"][0]
    coefs = []
    for ring in range(nint * nrep):
        li = ring // nrep
        xref = ti.xref[li].reshape(2, n)
        band = oracle.UMhessian(pes, c["mass"], n, betan, ti.xref[li])
        tot = 2 * n
        H = np.zeros((tot, tot))
        for rr in range(3):
            for col in range(tot - rr):
                H[col + rr, col] = H[col, col + rr] = band[rr, col]
        w, V = np.linalg.eigh(H)
        d = (x0[ring] - xref).T.ravel()  # UMhessian order: bead-major, dimension fastest
        t = np.sqrt(np.clip(w, 0.0, None) * m) * (V.T @ d)
        assert abs(V[:, 0] @ d) < 1e-9 * np.linalg.norm(d)  # the lowest mode is left out
        np.testing.assert_allclose(V[:, w <= 0].T @ d, 0.0, atol=1e-9 * np.linalg.norm(d))
        coefs.append(t[1:][w[1:] > 0] * np.sqrt(c["beta"]))
    z = np.concatenate(coefs)
    assert np.all(np.abs(z) < 6.0) and 0.6 < z.std() < 1.4 and abs(z.mean()) < 0.5
    # the same seeds and streams give the same displacements; rings of one lambda point differ
    r2 = subprocess.run([exe], input=text, capture_output=True, text=True, cwd=str(tmp_path), timeout=300,
                        env=dict(env, PG_STANDIN_X0=str(tmp_path / "x0b.txt")))
    assert r2.returncode == 0, r2.stderr
    np.testing.assert_array_equal(np.loadtxt(str(tmp_path / "x0b.txt")), x0.ravel())
    assert not np.allclose(x0[0], x0[1])


def test_pimd_ti_path_and_centre_on_the_oracle(oracle, tmp_path):
    """readpath + instapath + centre through pimd_ti.cpp on the CPU against the
    stand-in, whose optimiser keeps the spline path: here the straight segment
    between points 10 % inside two adjacent wells (an optimised path's end
    beads also sit off the wells, which the path [well 1, beads, well 2] needs,
    instantonmod.f90:961-966).  instanton.xyz holds the n beads and the
    centring finds the barrier top at 1/2 by the mirror symmetry."""
    import standin
    exe = standin.build_driver("pimd_ti", tmp_path)
    c = dict(pgconfigs.load("c1"))
    _write_inputs(tmp_path, c, ["H"])
    m1, m2 = np.array(c["well1"]), np.array(c["well2"])
    w1, w2 = m1 + 0.1 * (m2 - m1), m2 - 0.1 * (m2 - m1)
    (tmp_path / "path.xyz").write_text("".join(" 1\n frame %d\n H %.17g %.17g\n" % (i, *w) for i, w in
                                               enumerate((w1, w2))))
    n = 24
    text = ("&MCDATA n=%d, beta=%.17g, NMC=20, dt=%.17g, imin=10, tau=1.0, gamma=%.17g, nintegral=3,\n"
            " nrep=2, thermostat=2, ndim=2, natom=1, readpath=T, npath=2, instapath=T, centre=T,\n"
            " pes='2dtest', pes_params='pes.dat', precision='fp64', form='fused', init='path', seed=0 /\n"
            % (n, c["beta"], c["dt"], c["gamma"]))
    r = subprocess.run([exe], input=text, capture_output=True, text=True, cwd=str(tmp_path), timeout=300)
    assert r.returncode == 0, r.stderr
    lines = (tmp_path / "instanton.xyz").read_text().strip().split("\n")
    assert len(lines) == 3 * n
    beads = np.array([[float(v) for v in lines[3 * i + 2].split()[1:]] for i in range(n)]) / 0.529177
    k = np.arange(n)[:, None] / (n - 1)
    np.testing.assert_allclose(beads, (1 - k) * w1 + k * w2, atol=1e-12)
    xm = float(re.search(r"Centred,\s*\S+\s+\S+\s+(\S+)", r.stdout).group(1))
    assert abs(xm - 0.5) < 1e-6
    assert np.isfinite(float(re.search(r"final Delta A=\s*(\S+)", r.stdout).group(1)))
    # read_path's side files: the instanton beads under the alignment angles (0 in 2-D), and one row of
    # spline second derivatives per coordinate over the n + 2 points [well 1, beads, well 2]
    al = (tmp_path / "aligned.xyz").read_text().strip().split("\n")
    assert al[1].split()[:2] == ["rotation", "angles:"] and [float(v) for v in al[1].split()[2:]] == [0.0] * 3
    np.testing.assert_allclose(np.array([[float(v) for v in al[3 * i + 2].split()[1:]] for i in range(n)]) / 0.529177,
                               beads, rtol=0, atol=1e-12)
    ts = [l.split() for l in (tmp_path / "testspline.csv").read_text().strip().split("\n")]
    assert [t[:2] for t in ts] == [["1", "1"], ["2", "1"]] and all(len(t) == 2 + n + 2 for t in ts)


def test_rpi_angular_grid_on_the_oracle(oracle, tmp_path):
    """angular = T for a 3-D system through rpi.cpp on the CPU against the
    stand-in (its optimiser keeps the start path): the Gauss-Legendre angles and
    weights, well 2 turned by R_x(theta) R_z(phi) R_x(eta) in the reference's
    rotation convention (rpi_ser.f90:245-257, instantonmod.f90:346-376), and
    I = tanh(Omega N) per row of angularI.dat (rpi_ser.f90:273-296; 0 here,
    since the unoptimised path's action is large)."""
    import align
    import standin
    exe = standin.build_driver("rpi", tmp_path)
    c = pgconfigs.load("c3")
    _write_inputs(tmp_path, c, ["O", "O", "C", "C", "C", "H", "H", "H", "H"])
    n, npts, beta = 4, 2, 40.0
    text = ("&RPIDATA n=%d, beta=%.17g, ndim=3, natom=9, readpath=.false., pes='synth9', pes_params='pes.dat',\n"
            " angular=.true., npoints=%d, cutofftheta=1.0, cutoffphi=0.5 /\n" % (n, beta, npts))
    env = dict(os.environ, PG_STANDIN_ENDS=str(tmp_path / "ends.txt"))
    r = subprocess.run([exe], input=text, capture_output=True, text=True, cwd=str(tmp_path), timeout=300, env=env)
    assert r.returncode == 0, r.stderr
    rows = np.loadtxt(str(tmp_path / "angularI.dat"))
    ends = np.loadtxt(str(tmp_path / "ends.txt")).reshape(npts ** 3, 27)
    assert rows.shape == (npts ** 3, 5)
    w1, w2, mass = np.array(c["well1"]), np.array(c["well2"]), c["mass"]
    pes0 = oracle.Pes(c["pes_id"], 3, 9, c["params"])
    pes = oracle.Pes(c["pes_id"], 3, 9, c["params"], V0=pes0.V(w1))
    betan, nd = beta / n, 27
    k = np.arange(1, n + 1)
    x = np.concatenate([((n - k) * w1[d] + (k - 1) * w2[d]) / (n - 1) for d in range(nd)])
    vshift = min(0.0, min(pes.V(x.reshape(nd, n)[:, b]) for b in range(n)))
    ld0 = oracle.logdet_band(oracle.UMhessian(pes, mass, n, betan, np.repeat(w1, n), singlewell=True), False)[0]
    ld = oracle.logdet_band(oracle.UMhessian(pes, mass, n, betan, x), True)[0]
    th, wth = oracle.gauleg(0.0, 1.0, npts)
    ph, wph = oracle.gauleg(0.0, 0.5, npts)
    q = 0
    for ii in range(npts):
        for jj in range(npts):
            for kk in range(npts):
                wr = w2.reshape(9, 3)
                wr = align.rotate_atoms(wr, 1, th[kk])  # eta shares theta's range
                wr = align.rotate_atoms(wr, 3, ph[jj])
                wr = align.rotate_atoms(wr, 1, th[ii])
                np.testing.assert_allclose(ends[q], wr.ravel(), rtol=0, atol=1e-13)
                UM = oracle.UM(pes, mass, n, betan, x, w1, wr.ravel()) - n * vshift
                S = betan * UM
                om = betan * np.exp(-S) * np.sqrt(S / (2 * oracle.PI_REF)) / np.exp(0.5 * (ld - ld0))
                ib = 1.0 if om * n > 1.0 else np.tanh(om * n)
                np.testing.assert_allclose(rows[q, :3], [th[ii], ph[jj], th[kk]], rtol=1e-15)
                assert rows[q, 3] == pytest.approx(wth[ii] * wph[jj] * wth[kk], rel=1e-14)
                assert rows[q, 4] == pytest.approx(ib, rel=1e-8, abs=1e-300)
                q += 1


def test_pimd_ti_resumes_after_a_failed_run(oracle, tmp_path):
    """Restart files every Noutput steps (verletmodule.f90:389-395): a run that
    fails at step 250 (injected on the host: the stand-in's advance refuses to
    pass it) has left the files of its state after 199 steps; restart = 2 from
    them runs to step 300 and matches an uninterrupted run."""
    import standin
    exe = standin.build_driver("pimd_ti", tmp_path)
    c = dict(pgconfigs.load("c0"), imin=50, P=16)
    run_dir, ref_dir = tmp_path / "run", tmp_path / "ref"
    for d in (run_dir, ref_dir):
        d.mkdir()
        _write_inputs(d, c, ["H"])

    def text(nmc, restart):
        return _ti_text(c, nmc, 2, "restart=%d, Noutput=100, chunk=30 " % restart)

    r = subprocess.run([exe], input=text(300, 1), capture_output=True, text=True, cwd=str(run_dir), timeout=300,
                       env=dict(os.environ, PG_STANDIN_FAIL_AT="250"))
    assert r.returncode == 2 and "pg_ti_advance" in r.stderr
    lines = (run_dir / "restart_proc0_1.xyz").read_text().split("\n")
    assert lines[16 * 3 + 1].strip() == "199"  # written before step 200 (the second write)
    r = subprocess.run([exe], input=text(101, 2), capture_output=True, text=True, cwd=str(run_dir), timeout=300)
    assert r.returncode == 0, r.stderr
    resumed = float(re.search(r"final Delta A=\s*(\S+)", r.stdout).group(1))
    r = subprocess.run([exe], input=text(300, 0), capture_output=True, text=True, cwd=str(ref_dir), timeout=300)
    assert r.returncode == 0, r.stderr
    whole = float(re.search(r"final Delta A=\s*(\S+)", r.stdout).group(1))
    assert resumed == pytest.approx(whole, rel=1e-8)


def test_pimd_ti_rejects_corrupted_restart_files(oracle, tmp_path):
    """Corrupted restart files stop restart = 2 with a message naming the file:
    a truncated file, a wrong atom count, step counts that disagree."""
    import standin
    exe = standin.build_driver("pimd_ti", tmp_path)
    c = dict(pgconfigs.load("c0"), imin=50, P=16)
    _write_inputs(tmp_path, c, ["H"])
    r = subprocess.run([exe], input=_ti_text(c, 60, 2, "restart=1 "), capture_output=True, text=True,
                       cwd=str(tmp_path), timeout=300)
    assert r.returncode == 0, r.stderr
    good = {p.name: p.read_text() for p in tmp_path.glob("restart_proc*.xyz")}
    f = tmp_path / "restart_proc0_3.xyz"

    def resume():
        return subprocess.run([exe], input=_ti_text(c, 10, 2, "restart=2 "), capture_output=True, text=True,
                              cwd=str(tmp_path), timeout=300)

    f.write_text(good[f.name][: len(good[f.name]) // 2])  # truncated
    r = resume()
    assert r.returncode == 1 and "restart_proc0_3.xyz" in r.stderr
    f.write_text(good[f.name].replace(" 1\n", " 2\n", 1))  # natom 2 in the first frame
    r = resume()
    assert r.returncode == 1 and "restart_proc0_3.xyz" in r.stderr
    lines = good[f.name].split("\n")
    lines[16 * 3 + 1] = " 61"  # two step counts in one file
    f.write_text("\n".join(lines))
    r = resume()
    assert r.returncode == 1 and "restart_proc0_3.xyz" in r.stderr
    for b in range(16):
        lines[(16 + b) * 3 + 1] = " 61"  # another step count than the other files
    f.write_text("\n".join(lines))
    r = resume()
    assert r.returncode == 1 and "disagree" in r.stderr
    f.write_text(good[f.name])
    r = resume()
    assert r.returncode == 0, r.stderr


def test_rpi_path_xyz_on_the_oracle(oracle, tmp_path):
    """readpath for a 3-D system through rpi.cpp on the CPU against the stand-in:
    the frames of path.xyz aligned by the first frame's angles, splined against
    arc length, n start beads; aligned.xyz carries them under those angles and
    testspline.csv the spline's second derivatives (instantonmod.f90:916-1031)."""
    import align
    import standin
    exe = standin.build_driver("rpi", tmp_path)
    c = pgconfigs.load("c3")
    labels = ["O", "O", "C", "C", "C", "H", "H", "H", "H"]
    _write_inputs(tmp_path, c, labels)
    w1, w2 = np.array(c["well1"]), np.array(c["well2"])
    rng = np.random.default_rng(3)
    frames = [w1 + 0.02 * rng.normal(size=27), 0.5 * (w1 + w2) + 0.05 * rng.normal(size=27), w2]
    (tmp_path / "path.xyz").write_text("".join(
        " 9\n frame %d\n" % i + "".join(" %s %.17g %.17g %.17g\n" % (labels[j], *(f.reshape(9, 3)[j] * 0.529177))
                                         for j in range(9)) for i, f in enumerate(frames)))
    n = 6
    text = ("&RPIDATA n=%d, beta=%.17g, ndim=3, natom=9, xunit=2, readpath=.true., npath=3, pes='synth9',\n"
            " pes_params='pes.dat' /\n" % (n, c["betas"][2]))
    (tmp_path / "well1.dat").write_text("\n".join("%.17g" % v for v in w1 * 0.529177) + "\n")
    (tmp_path / "well2.dat").write_text("\n".join("%.17g" % v for v in w2 * 0.529177) + "\n")
    r = subprocess.run([exe], input=text, capture_output=True, text=True, cwd=str(tmp_path), timeout=300)
    assert r.returncode == 0, r.stderr
    fa = np.array(align.align_frames(frames))
    lam = np.concatenate([[0.0], np.cumsum(np.linalg.norm(np.diff(fa, axis=0), axis=1))])
    lam /= lam[-1]
    y2 = [oracle.spline(lam, fa[:, d]) for d in range(27)]
    x = np.array([[oracle.splint(lam, fa[:, d], y2[d], b / (n - 1)) for d in range(27)] for b in range(n)])
    al = (tmp_path / "aligned.xyz").read_text().strip().split("\n")
    np.testing.assert_allclose([float(v) for v in al[1].split()[2:]], align.get_align(frames[0]), atol=1e-12)
    got = np.array([[float(v) for j in range(9) for v in al[11 * b + 2 + j].split()[1:]] for b in range(n)])
    np.testing.assert_allclose(got / 0.529177, x, rtol=0, atol=1e-10)
    ts = [l.split() for l in (tmp_path / "testspline.csv").read_text().strip().split("\n")]
    assert [(int(t[0]), int(t[1])) for t in ts] == [(d, j) for d in (1, 2, 3) for j in range(1, 10)]
    for t in ts:
        d, j = int(t[0]) - 1, int(t[1]) - 1
        np.testing.assert_allclose([float(v) for v in t[2:]], y2[j * 3 + d], rtol=1e-10, atol=1e-10)
