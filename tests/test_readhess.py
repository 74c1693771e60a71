"""readhess start displacements (verletmodule.f90:49-88) of the Python driver,
on the oracle's polymer Hessian (CPU): a direct restatement of the reference's
loops gives the same displacements, the lowest mode and the negative modes do
not enter, and the displacement of a mode scales as 1/sqrt(eta^2 m)."""
import numpy as np
import pytest

import pgconfigs


def _reference_loops(band, P, ndim, natom, mass, beta, z):
    # the loops of verletmodule.f90:72-84 on the eigendecomposition of the band
    nd = ndim * natom
    n = P * nd
    H = np.zeros((n, n))
    for r in range(nd + 1):
        for c in range(n - r):
            H[c + r, c] = H[c, c + r] = band[r, c]
    eta2, vec = np.linalg.eigh(H)
    tempx = z * np.sqrt(1.0 / beta)
    dx = np.zeros(n)
    for idof1 in range(1, n):  # idof1 = 2 .. totdof
        if eta2[idof1] < 0.0:
            continue
        for i2 in range(P):
            for j2 in range(ndim):
                for k2 in range(natom):
                    idof2 = natom * (j2 + ndim * i2) + k2
                    dx[(k2 * ndim + j2) * P + i2] += (np.sqrt(1.0 / (eta2[idof1] * mass[k2])) * tempx[idof1]
                                                      * vec[idof2, idof1])
    return dx


@pytest.mark.parametrize("name,P", [("c1", 12), ("c2", 3)])
def test_readhess_matches_reference_loops(oracle, name, P):
    import drivers
    c = pgconfigs.load(name)
    pes = oracle.Pes(c["pes_id"], c["ndim"], c["natom"], c["params"], V0=c["V0"])
    mass = np.array(c["mass"])
    nd = c["ndim"] * c["natom"]
    w1, w2 = np.array(c["well1"]), np.array(c["well2"])
    x = np.concatenate([np.linspace(a, b, P) for a, b in zip(w1, w2)])  # a straight path, ring layout
    betan = c["beta"] / (P + 1)
    band = oracle.UMhessian(pes, mass, P, betan, x, singlewell=False)
    z = np.random.RandomState(5).randn(2, P * nd)
    dx = drivers.readhess_displacements(band, P, c["ndim"], c["natom"], mass, c["beta"], z)
    for r in range(2):
        np.testing.assert_allclose(dx[r], _reference_loops(band, P, c["ndim"], c["natom"], mass, c["beta"], z[r]),
                                   rtol=1e-10, atol=1e-12 * np.max(np.abs(dx[r])))


def test_readhess_modes_that_enter(oracle):
    import drivers
    c = pgconfigs.load("c1")
    pes = oracle.Pes(c["pes_id"], c["ndim"], c["natom"], c["params"], V0=c["V0"])
    mass = np.array(c["mass"])
    P, nd = 10, 2
    x = np.concatenate([np.linspace(a, b, P) for a, b in zip(c["well1"], c["well2"])])
    band = oracle.UMhessian(pes, mass, P, c["beta"] / (P + 1), x, singlewell=False)
    n = P * nd
    H = np.zeros((n, n))
    for r in range(nd + 1):
        i = np.arange(n - r)
        H[i + r, i] = band[r, :n - r]
        H[i, i + r] = band[r, :n - r]
    eta2, vec = np.linalg.eigh(H)
    for m in range(n):  # one normal at a time: the displacement is that mode alone, or nothing
        z = np.zeros((1, n))
        z[0, m] = 1.0
        dx = drivers.readhess_displacements(band, P, 2, 1, mass, c["beta"], z)[0]
        u = np.concatenate([dx[b::P] for b in range(P)])  # back to the Hessian's bead-major order
        if m == 0 or eta2[m] <= 0.0:
            assert np.all(dx == 0.0)
        else:
            np.testing.assert_allclose(u, vec[:, m] / np.sqrt(eta2[m] * mass[0] * c["beta"]), rtol=1e-9,
                                       atol=1e-14)
