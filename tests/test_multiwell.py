"""Splitting assembly beyond the single-temperature form, CPU only (host
functions of the C-ABI): the two-temperature splitting and offset
(python_utils/multiwell_waterdimer.py:6-16) and the per-representation
level ratios of a multi-well system (multiwell_waterdimer.py:65-84), against
closed forms and a loop-by-loop transcription of the script's arithmetic."""
import math

import numpy as np
import pytest


def _ratios_loops(c, rho):
    """multiwell_waterdimer.py:67-75."""
    out = []
    for i in range(len(c)):
        em = ep = 0.0
        for j in range(len(rho)):
            em += (1.0 - c[i][j]) * rho[j]
            ep += (1.0 + c[i][j]) * rho[j]
        out.append(em / ep)
    return out


def test_two_beta_recovers_splitting_and_offset(pg):
    for delta, bbar, b1, b2 in [(1e-4, 300.0, 12000.0, 20000.0), (3e-3, -50.0, 400.0, 900.0)]:
        r1, r2 = math.tanh(delta * (b1 - bbar) / 2), math.tanh(delta * (b2 - bbar) / 2)
        d, bb = pg.splitting_two_beta(b1, r1, b2, r2)
        assert d == pytest.approx(delta, rel=1e-9)
        assert bb == pytest.approx(bbar, rel=1e-6, abs=1e-6)
    # zero offset: the same splitting as the single-temperature form at either beta
    d, bb = pg.splitting_two_beta(1000.0, math.tanh(0.5), 3000.0, math.tanh(1.5))
    assert d == pytest.approx(pg.splitting_from_ratio(1000.0, math.tanh(0.5)), rel=1e-12)
    assert bb == pytest.approx(0.0, abs=1e-9)


def test_two_beta_rejects_bad_input(pg):
    with pytest.raises(pg.PgError):
        pg.splitting_two_beta(100.0, 0.2, 100.0, 0.3)
    with pytest.raises(pg.PgError):
        pg.splitting_two_beta(100.0, 1.2, 200.0, 0.3)
    _, bb = pg.splitting_two_beta(100.0, 0.3, 200.0, 0.3)
    assert math.isnan(bb)


def test_irrep_ratios(pg):
    # two wells, operations (E, swap): the antisymmetric representation gives rho itself
    c2 = np.array([[1.0, 1.0], [1.0, -1.0]])
    np.testing.assert_allclose(pg.irrep_ratios(c2, [1.0, 0.3]), [0.0, 0.3], rtol=0, atol=1e-16)
    rng = np.random.default_rng(2)
    chars = rng.choice([-1.0, 0.0, 1.0], size=(6, 8))
    chars[:, 0] = 1.0
    rho = np.concatenate([[1.0], rng.uniform(0, 0.2, 7)])
    np.testing.assert_allclose(pg.irrep_ratios(chars, rho), _ratios_loops(chars.tolist(), rho.tolist()),
                               rtol=1e-15)
    with pytest.raises(ValueError):
        pg.irrep_ratios(chars, rho[:5])


def test_multiwell_levels(pg):
    import drivers
    c2 = np.array([[1.0, 1.0], [1.0, -1.0]])
    delta, b1, b2 = 2e-4, 10000.0, 16000.0
    rho1, rho2 = [1.0, math.tanh(delta * b1 / 2)], [1.0, math.tanh(delta * b2 / 2)]
    d, bb, I1, I2 = drivers.multiwell_levels(c2, rho1, rho2, b1, b2)
    assert d[0] == 0.0 and math.isnan(bb[0])  # symmetric level: ratio 0 at both temperatures
    assert d[1] == pytest.approx(delta, rel=1e-10) and bb[1] == pytest.approx(0.0, abs=1e-6)
    np.testing.assert_allclose(I2, [0.0, rho2[1]], atol=1e-16)
