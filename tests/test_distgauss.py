"""The distance-Gaussian surface (pes_id 6): the functional form of
pes_malonaldehyde.f90 with the term tables as parameters.

CPU: the oracle's restatement, with tables extracted from the reference's own
source by configs/distgauss_from_fortran.py, is zero with zero gradient at the
published minimum structure (the file's header) -- run when the environment
variable PG_MALONALDEHYDE_F90 names the user's copy of pes_malonaldehyde.f90 --
and its gradient matches finite differences.  GPU: device surface,
Hessian and TI propagation against the oracle on seeded synthetic tables."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SRC = os.environ.get("PG_MALONALDEHYDE_F90", "")
sys.path.insert(0, os.path.join(ROOT, "pimd-tunneling_gb300", "configs"))

# minimum structure in the header of pes_malonaldehyde.f90 (angstrom; C C O C O H H H H)
MALON_MIN = np.array([[0.0035239647, 0.0, -1.1379095138], [1.1859410623, 0.0, -0.4671627095],
                      [1.2951373352, 0.0, 0.8494123252], [-1.2326642069, 0.0, -0.3950488380],
                      [-1.2836327508, 0.0, 0.8382056815], [-0.0071493753, 0.0, -2.2163348766],
                      [0.3688205810, 0.0, 1.1962401614], [-2.1703435327, 0.0, -0.9688628849],
                      [2.1404514581, 0.0, -0.9796660170]]) / 0.529177


def synthetic_distgauss(natom=6, seed=3):
    """A smooth distance-Gaussian surface and a start geometry (bohr)."""
    rs = np.random.RandomState(seed)
    ang = 2 * np.pi * np.arange(natom) / natom
    x0 = np.stack([2.4 * np.cos(ang), 2.4 * np.sin(ang), 0.3 * rs.randn(natom)], axis=1)
    pairs = [(i, j) for i in range(1, natom) for j in range(i)]
    r0 = np.array([np.linalg.norm(x0[i] - x0[j]) for i, j in pairs])
    npair = len(pairs)
    p = [natom, -0.01]
    morse = [(k, r0[k], rs.uniform(1.0, 2.0), rs.uniform(0.2, 0.5)) for k in rs.choice(npair, 5, replace=False)]
    g1 = [(k, r0[k] + 0.2 * rs.randn(), rs.uniform(1, 4), 0.01 * rs.randn(), 0.0) for k in rs.choice(npair, 8)]
    g2 = [tuple(rs.choice(npair, 2, replace=False)) for _ in range(12)]
    g2 = [(a, b, r0[a] + 0.2 * rs.randn(), r0[b] + 0.2 * rs.randn(), rs.uniform(1, 4), rs.uniform(1, 4),
           0.01 * rs.randn(), 0.1 * rs.rand()) for a, b in g2]
    g3 = [tuple(rs.choice(npair, 3, replace=False)) for _ in range(10)]
    g3 = [(a, b, c, r0[a], r0[b], r0[c], rs.uniform(1, 3), rs.uniform(1, 3), rs.uniform(1, 3),
           0.01 * rs.randn(), 0.0) for a, b, c in g3]
    p += [len(morse), len(g1), len(g2), len(g3)]
    for t in morse + g1 + g2 + g3:
        p += [float(v) for v in t]
    return [float(v) for v in p], x0.ravel()


def test_distgauss_gradient_matches_finite_differences(oracle):
    p, x0 = synthetic_distgauss()
    pes = oracle.Pes(6, 3, 6, p)
    rs = np.random.RandomState(1)
    x = x0 + 0.05 * rs.randn(x0.size)
    g = pes.Vprime(x)
    h = 1e-5
    fd = np.array([(pes.V(x + h * e) - pes.V(x - h * e)) / (2 * h) for e in np.eye(x.size)])
    np.testing.assert_allclose(g, fd, rtol=1e-6, atol=1e-9)


@pytest.mark.skipif(not (REF_SRC and os.path.exists(REF_SRC)),
                    reason="PG_MALONALDEHYDE_F90 does not name a copy of pes_malonaldehyde.f90")
def test_malonaldehyde_tables_zero_at_published_minimum(oracle):
    import distgauss_from_fortran as D
    p = D.parameters(open(REF_SRC).read())
    assert p[0] == 9 and p[2:6] == [9, 80, 1728, 1741] and len(p) == 33417
    pes = oracle.Pes(6, 3, 9, p)
    x = MALON_MIN.ravel()
    assert abs(pes.V(x)) < 1e-9
    assert np.max(np.abs(pes.Vprime(x))) < 1e-5


def _set(ctx, p, natom, mass=None):
    mass = mass if mass is not None else [12.0 * 1822.888486] * natom
    ctx.set_system(3, natom, mass, 6, p, 0.0)


@pytest.mark.gpu
def test_distgauss_device_surface_and_hessian_match_oracle(ctx, pg, oracle):
    p, x0 = synthetic_distgauss()
    _set(ctx, p, 6)
    pes = oracle.Pes(6, 3, 6, p)
    rs = np.random.RandomState(2)
    X = np.array([x0 + 0.05 * rs.randn(x0.size) for _ in range(16)])
    V, G = ctx.pes_eval(X.ravel(), pg.PG_FP64)
    for i in range(len(X)):
        assert abs(V[i] - pes.V(X[i])) <= 1e-13 * max(1.0, abs(pes.V(X[i])))
        np.testing.assert_allclose(G[i], pes.Vprime(X[i]), rtol=1e-11, atol=1e-13)
    Vf, Gf = ctx.pes_eval(X.ravel(), pg.PG_MIXED)
    assert np.max(np.abs(Gf - G)) < 2e-5 * np.max(np.abs(G)) + 1e-6
    H = ctx.pes_hessian(X[:4].ravel())
    for i in range(4):
        np.testing.assert_allclose(H[i], pes.Vdoubleprime(X[i]), rtol=1e-7, atol=1e-9)


@pytest.mark.gpu
def test_distgauss_ti_fp64_matches_oracle_and_tensor_tracks(ctx, pg, oracle):
    """Fused FP64 TI on the synthetic surface against the oracle's NM-resident
    step; the blocked tensor form (P = 64) tracks the FP32 SIMT form."""
    import pgconfigs
    p, x0 = synthetic_distgauss()
    rs = np.random.RandomState(4)
    mass = list(1822.888486 * rs.choice([1.0, 12.0, 16.0], 6))
    c = dict(ndim=3, natom=6, mass=mass, pes_id=6, params=p, V0=0.0, beta=2000.0, dt=0.05, tau=1.0,
             gamma=0.2, thermostat=2, well1=list(x0), well2=list(x0 + 0.1 * rs.randn(x0.size)),
             init_sigma=0.01, imin=3, P=16)
    ti = pgconfigs.TiInputs(c, nrep=2, nintegral=2)
    _set(ctx, p, 6, mass)
    nsteps = 30
    cfg = ti.ti_config(pg, pg.PG_FP64, pg.PG_FORM_FUSED)
    ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
    ctx.ti_advance(nsteps)
    x, _ = ctx.ti_state()
    s, n, _, st = ctx.ti_results()
    pes = oracle.Pes(6, 3, 6, p)
    prm = oracle.TiParams(ti.P, c["beta"], c["dt"], tau=1.0, gamma=c["gamma"], thermostat=2, nm_resident=True,
                          imin=3, init_sigma=c["init_sigma"])
    for r in range(ti.nrings):
        li = ti.ring_lambda[r]
        xo, po = oracle.ring_init(pes, np.array(mass), prm, ti.xref[li], int(ti.ring_seed[r]),
                                  int(ti.ring_stream[r]), a=ti.a, b=ti.b[li])
        res = oracle.ring_propagate(pes, np.array(mass), prm, ti.a, ti.b[li], ti.dbdl[li], ti.xref[li],
                                    int(ti.ring_seed[r]), int(ti.ring_stream[r]), 0, nsteps, xo, po)
        np.testing.assert_allclose(x[r * ti.nd * ti.P:(r + 1) * ti.nd * ti.P], xo, rtol=0, atol=1e-9)
        assert abs(s[r] - res.dhdr_sum) <= 1e-9 * abs(res.dhdr_sum) + 1e-12
    assert np.all(st == 0)
    c["P"] = 64
    ti = pgconfigs.TiInputs(c, nrep=3, nintegral=2)
    out = []
    for form in (pg.PG_FORM_FUSED, pg.PG_FORM_TENSOR):
        cfg = ti.ti_config(pg, pg.PG_MIXED, form)
        ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
        assert ctx.ti_form(1)[0] == form
        ctx.ti_advance(20)
        out.append((ctx.ti_state()[0], ctx.ti_results()[0]))
    assert np.max(np.abs(out[0][0] - out[1][0])) < 2e-3
    np.testing.assert_allclose(out[1][1], out[0][1], rtol=2e-4, atol=1e-6)
