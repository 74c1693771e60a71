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
    # reference defaults (pimd_par.f90:60-88) for keys not given
    r = _run("pimd_ti", "&MCDATA /", args=["--parse-only"])
    d = json.loads(r.stdout)
    assert d["n"] == 100 and d["NMC"] == 5000000 and d["thermostat"] == 1 and d["ndim"] == 3


def test_rpidata_namelist_parsing(drivers_built):
    r = _run("rpi", "&RPIDATA n=512, beta=3157.75, ndim=3, natom=9, readpath=.false., pes='synth9', m=10 /",
             args=["--parse-only"])
    d = json.loads(r.stdout)
    assert d["n"] == 512 and d["natom"] == 9 and d["readpath"] is False and d["m"] == 10
    assert d["pgtol"] == 1e-5 and d["factr"] == 1e6


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
