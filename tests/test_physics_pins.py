"""Physics pins of the oracle beyond its unit checks (the reference ships no
tests, so these tie the restatement to known results):

* the mass-weighted Hessian of a fixed-end harmonic ring polymer has the
  closed-form spectrum (2 / betan^2)(1 - cos(j pi / (N + 1))) + k / m, so the
  log-determinant of detJ (instantonmod.f90:782-827) is a closed-form sum;
* Langevin sampling gives normal-mode equipartition <pi_j^2 / m~_j> = 1 / betan
  for every mode (verletmodule.f90:634-667), in the reference step order and in
  the normal-mode-resident order;
* the ring-polymer-instanton splitting of rpi_ser.f90:222-237, 354-381 (S,
  Gamma~, Omega, Delta = 2 Omega / betan) approaches the exact ground-state
  splitting of a 1-D double well from a sinc discrete-variable representation
  (Colbert and Miller, J. Chem. Phys. 96, 1982 (1992)), with the error of
  instanton theory, which falls like 1 / S.
CPU only."""
import numpy as np
import pytest

MP = 1836.15


def test_harmonic_polymer_logdet_closed_form(oracle):
    k, m, N, betan = 0.37, 3.0, 40, 2.1
    pes = oracle.Pes(oracle.PES_HARMONIC, 1, 1, [k])
    x = np.random.default_rng(0).normal(size=N)  # the Hessian of a harmonic surface is the same everywhere
    j = np.arange(1, N + 1)
    eta2 = (2.0 / betan ** 2) * (1.0 - np.cos(j * np.pi / (N + 1))) + k / m
    band = oracle.UMhessian(pes, np.array([m]), N, betan, x)
    np.testing.assert_allclose(oracle.band_eigvals(band), np.sort(eta2), rtol=1e-12)
    ld, nsk, w0 = oracle.logdet_band(band, False)
    assert ld == pytest.approx(np.sum(np.log(eta2)), rel=1e-12) and nsk == 0
    ld1, _, _ = oracle.logdet_band(band, True)  # the lowest eigenvalue left out (rpi_ser.f90:227)
    assert ld1 == pytest.approx(np.sum(np.log(eta2)) - np.log(eta2.min()), rel=1e-12)


@pytest.mark.parametrize("nm_resident", [False, True])
def test_normal_mode_equipartition(oracle, nm_resident):
    P, m, k, betan = 8, 2.0, 0.5, 1.4
    pes = oracle.Pes(oracle.PES_HARMONIC, 1, 1, [k])
    mass = np.array([m])
    a, b = np.array([-0.4]), np.array([0.6])
    dt = 0.2
    prm = oracle.TiParams(P, betan * (P + 1), dt, tau=1.0, gamma=1.0 / (10 * dt), thermostat=2,
                          nm_resident=nm_resident)
    T, _, bm, _ = oracle.init_nm(P, 1, 1, mass, prm.betan, prm.tau, a, b)
    xref = np.repeat(a, P)
    x, p = oracle.ring_init(pes, mass, prm, xref, seed=5, stream=0, a=a, b=b)
    dbdl = b - a
    acc = np.zeros(P)
    nblk, step = 3000, 0
    for _ in range(nblk):
        oracle.ring_propagate(pes, mass, prm, a, b, dbdl, xref, 5, 0, step, 20, x, p)
        step += 20
        pi = T @ p
        acc += pi ** 2 / bm[0]
    mode_avg = acc / nblk
    np.testing.assert_allclose(mode_avg * prm.betan, 1.0, rtol=0.12)
    assert np.mean(mode_avg) * prm.betan == pytest.approx(1.0, rel=0.04)


def _dvr_splitting(m, H, x0, L=3.0, n=801):
    """Lowest two levels of -1/(2m) d2/dx2 + H ((x/x0)^2 - 1)^2 on a sinc DVR grid."""
    x = np.linspace(-L, L, n)
    dx = x[1] - x[0]
    d = np.arange(n)[:, None] - np.arange(n)[None, :]
    kin = np.where(d == 0, np.pi ** 2 / 3, 2.0 / np.where(d == 0, 1, d) ** 2) * (-1.0) ** d / (2 * m * dx * dx)
    E = np.linalg.eigvalsh(kin + np.diag(H * ((x / x0) ** 2 - 1) ** 2))
    return E[1] - E[0]


def _rpi_splitting(oracle, m, H, x0, beta, N):
    """rpi_ser.f90 for mcmod_1d: instanton by L-BFGS between the wells, log-dets
    at well 1 (every eigenvalue) and at the instanton (the lowest left out),
    then S, Omega and Delta."""
    pes = oracle.Pes(oracle.PES_1D, 1, 1, [H, x0])
    mass = np.array([m])
    betan = beta / N
    a, b = np.array([-x0]), np.array([x0])
    k = np.arange(1, N + 1)
    guess = ((N - k) * a[0] + (k - 1) * b[0]) / (N - 1)
    xi, UM, _ = oracle.instanton_lbfgs(pes, mass, N, betan, guess, a, b, m=8, factr=1e2, pgtol=1e-9)
    S = betan * UM
    ld0 = oracle.logdet_band(oracle.UMhessian(pes, mass, N, betan, np.repeat(a, N), singlewell=True), False)[0]
    ld = oracle.logdet_band(oracle.UMhessian(pes, mass, N, betan, xi), True)[0]
    omega = betan * np.exp(-S) * np.sqrt(S / (2 * oracle.PI_REF)) / np.exp(0.5 * (ld - ld0))
    return 2.0 * omega / betan, S


def test_rpi_splitting_approaches_the_exact_one(oracle):
    ratios = []
    for H in (0.0153, 0.05):
        exact = _dvr_splitting(MP, H, 1.0)
        rpi, S = _rpi_splitting(oracle, MP, H, 1.0, beta=4000.0, N=256)
        ratio = rpi / exact
        assert 1.0 < ratio < 1.0 + 1.5 / S  # instanton theory overestimates by O(1/S)
        ratios.append(ratio)
    assert ratios[1] < ratios[0]  # and comes closer for the deeper barrier
    # converged in the bead number and the temperature
    r2, _ = _rpi_splitting(oracle, MP, 0.0153, 1.0, beta=8000.0, N=512)
    r1, _ = _rpi_splitting(oracle, MP, 0.0153, 1.0, beta=4000.0, N=256)
    assert r2 == pytest.approx(r1, rel=1e-5)
