"""Crossover inverse temperature of a transition state (crossover.f90:1-73):
beta_c = 2 pi / sqrt(-eta^2_min) of the mass-weighted Hessian.

CPU: the oracle against the closed forms (mcmod_1d barrier top; the c0 / c1
configurations' beta_c), the C++ header of the namelist driver
(host/crossover.hpp) against the oracle, the driver's namelist and file
parsing and its loud failure without a GPU.  GPU: the driver and the Python
function, with the library's Hessian, against the oracle."""
import json
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

import pgconfigs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "pimd-tunneling_gb300", "lib")
MP = 1836.15


def test_oracle_known_answers(oracle):
    # mcmod_1d barrier top x = 0: V'' = -4 H / x0^2, beta_c = 2 pi / sqrt(4 H / (m x0^2))
    for H, x0, m in [(1.0, 1.0, MP), (0.3, 1.7, 2.5 * MP)]:
        pes = oracle.Pes(oracle.PES_1D, 1, 1, [H, x0])
        b, eta2 = oracle.crossover_beta(pes, [m], [0.0])
        assert eta2[0] == pytest.approx(-4 * H / (m * x0 * x0), rel=1e-7)
        assert b == pytest.approx(2 * oracle.PI_REF / np.sqrt(4 * H / (m * x0 * x0)), rel=1e-7)
    c0 = pgconfigs.load("c0")
    b, _ = oracle.crossover_beta(oracle.Pes(oracle.PES_1D, 1, 1, c0["params"]), c0["mass"], [0.0])
    assert b == pytest.approx(c0["beta_c"], rel=1e-7)
    # c1: the transition state between two of the six wells of mcmod_2dtest
    c1 = pgconfigs.load("c1")
    pes = oracle.Pes(oracle.PES_2DTEST, 2, 1, c1["params"])
    b, eta2 = oracle.crossover_beta(pes, c1["mass"], c1["ts"])
    assert eta2[0] < 0 < eta2[1]
    assert b == pytest.approx(c1["beta_c"], rel=1e-6)  # the configuration took a finite-difference Hessian


HARNESS = r'''
#include <cstdio>
#include <vector>
#include "crossover.hpp"
int main() {
    int ndim, natom;
    if (std::scanf("%d %d", &ndim, &natom) != 2) return 2;
    const int nd = ndim * natom;
    std::vector<double> mass(natom), h((size_t)nd * nd), eta2;
    for (auto &m : mass)
        if (std::scanf("%lf", &m) != 1) return 2;
    for (auto &x : h)
        if (std::scanf("%lf", &x) != 1) return 2;
    const double b = pgh::crossover_beta(ndim, natom, h, mass, eta2);
    std::printf("%.17g\n", b);
    for (double e : eta2) std::printf("%.17g\n", e);
    return 0;
}
'''


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if not cxx:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("crossover")
    src = d / "harness.cpp"
    src.write_text(HARNESS)
    exe = d / "harness"
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "pimd-tunneling_gb300", "host"), str(src),
                    "-o", str(exe)], check=True)
    return str(exe)


def _harness(exe, ndim, natom, mass, H):
    text = "%d %d\n" % (ndim, natom) + "\n".join("%.17g" % v for v in np.concatenate([mass, np.ravel(H)]))
    out = np.array(subprocess.run([exe], input=text, capture_output=True, text=True, check=True).stdout.split(),
                   dtype=float)
    return out[0], out[1:]


def _saddles(oracle):
    c1 = pgconfigs.load("c1")
    yield oracle.Pes(oracle.PES_2DTEST, 2, 1, c1["params"]), c1["mass"], np.array(c1["ts"])
    c3 = pgconfigs.load("c3")
    pes = oracle.Pes(c3["pes_id"], c3["ndim"], c3["natom"], c3["params"])
    # midpoint of the two wells of the 9-atom surface: a configuration with negative curvature
    yield pes, c3["mass"], 0.5 * (np.array(c3["well1"]) + np.array(c3["well2"]))


def test_header_matches_oracle(oracle, harness):
    for pes, mass, ts in _saddles(oracle):
        b_ref, eta_ref = oracle.crossover_beta(pes, mass, ts)
        H = pes.Vdoubleprime(ts)
        b, eta = _harness(harness, pes.ndim, pes.natom, mass, H)
        scale = np.max(np.abs(eta_ref))
        np.testing.assert_allclose(eta, eta_ref, rtol=0, atol=1e-12 * scale)
        assert b == pytest.approx(b_ref, rel=1e-10)


def test_header_rejects_a_minimum(oracle, harness):
    c1 = pgconfigs.load("c1")
    pes = oracle.Pes(oracle.PES_2DTEST, 2, 1, c1["params"])
    b, eta = _harness(harness, 2, 1, c1["mass"], pes.Vdoubleprime(np.array(c1["well1"])))
    assert np.isnan(b) and eta[0] > 0


def _run(text, cwd, args=()):
    path = os.path.join(LIB, "crossover")
    if not os.path.exists(path):
        pytest.skip("drivers not built")
    return subprocess.run([path] + list(args), input=text, capture_output=True, text=True, cwd=cwd, timeout=300)


def _write_inputs(d, labels, mass, ts, ndim, params, angstrom=True):
    natom = len(labels)
    (d / "masses.dat").write_text("".join("%s %.17g\n" % (l, m) for l, m in zip(labels, mass)))
    x = np.asarray(ts, float).reshape(natom, ndim) * (0.529177 if angstrom else 1.0)
    (d / "transition.xyz").write_text(" %d\n TS\n" % natom + "".join(
        " %s " % l + " ".join("%.17g" % v for v in row) + "\n" for l, row in zip(labels, x)))
    (d / "pes.dat").write_text("\n".join("%.17g" % v for v in params) + "\n")


def test_driver_parse_only(pg, tmp_path):
    r = _run("&CROSSDATA ndim=2, natom=1 /", str(tmp_path), ["--parse-only"])
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout)
    assert d == {"ndim": 2, "natom": 1, "xunit": 2, "pes": "1d", "quirks": 0}  # crossover.f90:16-18 defaults
    r = _run("&CROSSDATA /", str(tmp_path), ["--parse-only"])
    assert json.loads(r.stdout)["ndim"] == 3


def test_driver_reads_inputs_then_fails_loudly_without_gpu(pg, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    c1 = pgconfigs.load("c1")
    r = _run("&CROSSDATA ndim=2, natom=1, pes='2dtest', pes_params='pes.dat' /", str(tmp_path))
    assert r.returncode == 1 and "masses.dat" in r.stderr  # inputs are read before the device is opened
    _write_inputs(tmp_path, ["H"], c1["mass"], c1["ts"], 2, c1["params"])
    r = _run("&CROSSDATA ndim=2, natom=1, pes='2dtest', pes_params='pes.dat' /", str(tmp_path))
    assert r.returncode == 2
    assert "no CPU fallback" in r.stderr


@pytest.fixture(scope="module")
def driver_on_oracle(oracle, tmp_path_factory):
    """The driver's host logic end to end on the CPU: crossover.cpp linked
    against the oracle-backed stand-in for its C-ABI calls (tests/standin)."""
    import standin
    return standin.build_driver("crossover", tmp_path_factory.mktemp("xdrv"))


@pytest.mark.parametrize("case", ["c1", "synth9"])
def test_driver_host_logic_on_the_oracle(oracle, driver_on_oracle, tmp_path, case):
    if case == "c1":
        c = pgconfigs.load("c1")
        pes, mass, ts, labels = oracle.Pes(oracle.PES_2DTEST, 2, 1, c["params"]), c["mass"], c["ts"], ["H"]
        text = "&CROSSDATA ndim=2, natom=1, pes='2dtest', pes_params='pes.dat' /"
    else:
        c = pgconfigs.load("c3")
        pes = oracle.Pes(c["pes_id"], 3, 9, c["params"])
        mass, labels = c["mass"], ["O", "O", "C", "C", "C", "H", "H", "H", "H"]
        ts = 0.5 * (np.array(c["well1"]) + np.array(c["well2"]))
        text = "&CROSSDATA ndim=3, natom=9, xunit=2, pes='synth9', pes_params='pes.dat' /"
    _write_inputs(tmp_path, labels, mass, ts, pes.ndim, c["params"])
    r = subprocess.run([driver_on_oracle], input=text, capture_output=True, text=True, cwd=str(tmp_path),
                       timeout=120)
    assert r.returncode == 0, r.stderr
    b = float(re.search(r"Crossover beta=\s*(\S+)", r.stdout).group(1))
    eta = np.array(r.stdout.split("Crossover")[0].split(), dtype=float)
    b_ref, eta_ref = oracle.crossover_beta(pes, mass, ts)
    assert b == pytest.approx(b_ref, rel=1e-9)
    np.testing.assert_allclose(eta, eta_ref, rtol=0, atol=1e-10 * np.max(np.abs(eta_ref)))


@pytest.mark.gpu
def test_driver_matches_oracle(pg, oracle, tmp_path):
    c1 = pgconfigs.load("c1")
    _write_inputs(tmp_path, ["H"], c1["mass"], c1["ts"], 2, c1["params"])
    r = _run("&CROSSDATA ndim=2, natom=1, xunit=2, pes='2dtest', pes_params='pes.dat' /", str(tmp_path))
    assert r.returncode == 0, r.stderr
    b = float(re.search(r"Crossover beta=\s*(\S+)", r.stdout).group(1))
    pes = oracle.Pes(oracle.PES_2DTEST, 2, 1, c1["params"])
    b_ref, _ = oracle.crossover_beta(pes, c1["mass"], c1["ts"])
    assert b == pytest.approx(b_ref, rel=1e-9)
    assert b == pytest.approx(c1["beta_c"], rel=1e-6)


@pytest.mark.gpu
def test_python_function_matches_oracle(ctx, oracle):
    import drivers
    for pes, mass, ts in _saddles(oracle):
        ctx.set_system(pes.ndim, pes.natom, mass, pes.id, pes.params, 0.0)
        b, eta = drivers.crossover_beta(ctx, ts, mass)
        b_ref, eta_ref = oracle.crossover_beta(pes, mass, ts)
        np.testing.assert_allclose(eta, eta_ref, rtol=0, atol=1e-10 * np.max(np.abs(eta_ref)))
        assert b == pytest.approx(b_ref, rel=1e-9)
