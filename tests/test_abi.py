"""C-ABI checks that need no GPU: the library loads, exports every symbol that
include/pimdgpu.h declares, its host-side assembly helpers match the oracle,
and context creation fails loudly (no CPU fallback) when no GPU is visible."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import pgconfigs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_functions():
    txt = open(os.path.join(ROOT, "include", "pimdgpu.h")).read()
    return sorted(set(re.findall(r"\b(pg_[a-z0-9_]+)\s*\(", txt)))


def test_exports_every_declared_symbol(pg):
    L = pg.lib()
    declared = _header_functions()
    assert len(declared) >= 25
    for name in declared:
        assert hasattr(L, name), name
    assert sorted(pg.EXPORTS) == declared
    assert L.pg_version() >= 10000


def test_host_gauleg_matches_oracle(pg, oracle):
    for n in (5, 11, 12, 16):
        x, w = pg.gauleg(0.0, 1.0, n)
        xo, wo = oracle.gauleg(0.0, 1.0, n)
        np.testing.assert_array_equal(x, xo)
        np.testing.assert_array_equal(w, wo)


def test_host_spline_matches_oracle(pg, oracle):
    xa = np.cumsum(np.random.RandomState(0).rand(17))
    xa /= xa[-1]
    ya = np.cos(4 * xa)
    y2 = pg.spline(xa, ya)
    np.testing.assert_array_equal(y2, oracle.spline(xa, ya))
    for t in (0.0, 0.31, 0.5, 0.999, 1.0):
        y, g = pg.splint(xa, ya, y2, t)
        assert y == oracle.splint(xa, ya, y2, t)
        assert g == oracle.splin_grad(xa, ya, y2, t)


def test_host_assembly_matches_oracle(pg, oracle):
    w = np.array([0.1, 0.4, 0.5])
    vals = np.random.RandomState(3).randn(3 * 5)
    m = vals.reshape(3, 5).mean(1)
    v = (vals.reshape(3, 5) ** 2).mean(1) - m ** 2
    dA, sA, q = pg.ti_assemble(w, m, v, 1.7)
    dAo, sAo, qo = oracle.ti_assemble(w, vals, 5, 1.7)
    assert abs(dA - dAo) < 1e-14 and abs(sA - sAo) < 1e-14 and abs(q - qo) < 1e-14
    d = pg.splitting_from_ratio(100.0, 0.25)
    assert abs(d - 2 * np.arctanh(0.25) / 100.0) < 1e-16
    S, om, de = pg.rpi_assemble(2.0, 3.0, 1.0, 0.5)
    assert abs(S - 6.0) < 1e-15
    assert abs(de - 2 * om / 2.0) < 1e-18
    with pytest.raises(pg.PgError):
        pg.splitting_from_ratio(100.0, 1.5)


def test_argument_errors_are_reported(pg):
    with pytest.raises(pg.PgError) as e:
        pg.gauleg(0.0, 1.0, 0)
    assert e.value.code == pg.PG_ERR_ARG
    assert "gauleg" in pg.lib().pg_last_error().decode()


def test_no_cpu_fallback_without_gpu(pg):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    h = C.c_void_p()
    rc = pg.lib().pg_create(C.byref(h), 0)
    assert rc == pg.PG_ERR_CUDA
    assert "no CPU fallback" in pg.lib().pg_last_error().decode()


def test_config_inputs_are_consistent(oracle):
    """The committed well files are stationary points of the oracle surfaces and
    the two wells of each symmetric surface are degenerate."""
    for name, pid in (("c1", oracle.PES_2DTEST), ("c2", oracle.PES_SYNTH9), ("c4", oracle.PES_SYNTH18)):
        c = pgconfigs.load(name)
        pes = oracle.Pes(pid, c["ndim"], c["natom"], c["params"], V0=c["V0"])
        for w in ("well1", "well2"):
            g = pes.Vprime(np.array(c[w]))
            assert np.max(np.abs(g)) < 1e-5, (name, w, np.max(np.abs(g)))
        assert abs(pes.V(np.array(c["well1"])) - pes.V(np.array(c["well2"]))) < 1e-10
        assert abs(pes.V(np.array(c["well1"]))) < 1e-10


def test_ti_inputs_layout():
    c = pgconfigs.load("c1")
    ti = pgconfigs.TiInputs(c, nrep=3, nintegral=4)
    assert ti.nrings == 12
    assert list(ti.ring_lambda) == [0, 0, 0, 1, 1, 1, 2, 2, 2, 3, 3, 3]
    assert list(ti.ring_seed[:4]) == [0, 1, 2, 0]
    assert ti.b.shape == (4, 2) and ti.xref.shape == (4, 2 * c["P"])


def _header_constants():
    txt = open(os.path.join(ROOT, "include", "pimdgpu.h")).read()
    return {k: int(v) for k, v in re.findall(r"^#define (PG_[A-Z0-9_]+) (-?\d+)\b", txt, flags=re.M)}


def test_constants_agree_across_header_python_and_fortran(pg):
    """Every numeric constant of include/pimdgpu.h has the same value in the
    Python binding and, where the Fortran module declares it, in pimdgpu_mod.f90."""
    h = _header_constants()
    assert len(h) >= 20
    for k, v in h.items():
        assert getattr(pg, k) == v, k
    ftxt = open(os.path.join(ROOT, "pimd-tunneling_gb300", "fortran", "pimdgpu_mod.f90")).read()
    fortran = {k: int(v) for k, v in re.findall(r"\b(PG_[A-Z0-9_]+)\s*=\s*(-?\d+)", ftxt)}
    assert len(fortran) >= 15
    for k, v in fortran.items():
        assert h[k] == v, k


def test_fortran_module_binds_every_function():
    """pimdgpu_mod.f90 has a bind(c) interface for every function of the header,
    each interface body is closed by its own end function, and no line passes the
    132 characters of free-form Fortran (no Fortran compiler is available here)."""
    ftxt = open(os.path.join(ROOT, "pimd-tunneling_gb300", "fortran", "pimdgpu_mod.f90")).read()
    bound = set(re.findall(r'bind\(c, name="(pg_[a-z0-9_]+)"\)', ftxt))
    assert set(_header_functions()) <= bound
    opened = re.findall(r"^\s*(?:[a-z_]+\([a-z0-9_]+\)\s+)?function\s+(pg_[a-z0-9_]+)\s*\(", ftxt, flags=re.M)
    closed = re.findall(r"^\s*end function\s+(pg_[a-z0-9_]+)\s*$", ftxt, flags=re.M)
    assert opened == closed
    for line in ftxt.splitlines():
        assert len(line) <= 132, line
