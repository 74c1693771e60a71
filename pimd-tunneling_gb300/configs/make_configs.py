"""Generate the inputs of the five benchmark configurations (JSON, committed).

The reference reads masses.dat / well1.dat / well2.dat and namelists; these
configurations are synthetic and new, so their inputs are produced here from
stated seeds with numpy/scipy (no GPU needed) and written next to this script.
Run:  python make_configs.py   (rewrites c0..c4 *.json)

Choices recorded in each JSON (the configuration texts leave them open):
  * masses: proton 1836.15 m_e for the 1-D and 2-D surfaces; 1/12/16 amu;
  * beta for c0/c1: 4 * beta_c, beta_c = 2 pi / sqrt(-eta^2_min) at the barrier
    (crossover.f90:49-71);
  * dt = (1/20) of the shortest normal-mode period of the ring at the well,
    2 pi tau / sqrt(1 + eta^2_max / lam_1^2) with tau = 1 (the free-polymer
    modes all have period 2 pi tau, verletmodule.f90:315,519; the PES curvature
    stiffens the low modes); gamma = 1/(100 dt);
  * straight-line TI path between the wells, Gauss-Legendre points on [0, 1].
"""
import json
import os

import numpy as np
from scipy.optimize import minimize

HERE = os.path.dirname(os.path.abspath(__file__))
AMU = 1822.888486
KB = 3.166811563e-6
MP = 1836.15
PI_REF = 3.14159265358979


# ---------------------------------------------------------------- numpy surfaces
def v_2dtest(x, m=6, a0=2.0, b0=0.2, rho0=3.0):
    k = np.arange(1, m + 1)
    xk = rho0 * np.cos(k * 2.0 * PI_REF / m)
    yk = rho0 * np.sin(k * 2.0 * PI_REF / m)
    u = (x[0] - xk) ** 2 + (x[1] - yk) ** 2
    return float(np.sum(-0.5 * np.exp(-a0 * u) - 0.5 * np.exp(-b0 * u)))


def num_hess(f, x, h=1e-4):
    n = len(x)
    H = np.zeros((n, n))
    for i in range(n):
        for j in range(i, n):
            e_i = np.zeros(n)
            e_j = np.zeros(n)
            e_i[i] = h
            e_j[j] = h
            H[i, j] = (f(x + e_i + e_j) - f(x + e_i - e_j) - f(x - e_i + e_j) + f(x - e_i - e_j)) / (4 * h * h)
            H[j, i] = H[i, j]
    return H


def synth9_params(seed=7):
    """36 pair Morse terms drawn per orbit of the mirror permutation, plus the
    quartic double well (barrier 0.006 Eh) in s = r(H*,O1) - r(H*,O2).
    Atoms: 0 O1, 1 O2, 2 C1, 3 C2, 4 C3, 5 H* (transferring), 6 H(C1), 7 H(C2), 8 H(C3).
    Mirror pi: O1<->O2, C1<->C3, H(C1)<->H(C3); C2, H*, H(C2) fixed."""
    perm = [1, 0, 4, 3, 2, 5, 8, 7, 6]
    rng = np.random.RandomState(seed)
    pairs = [(i, j) for i in range(9) for j in range(i + 1, 9)]
    seen = {}
    out = []
    for (i, j) in pairs:
        key = tuple(sorted((i, j)))
        img = tuple(sorted((perm[i], perm[j])))
        orb = min(key, img)
        if orb not in seen:
            seen[orb] = (rng.uniform(0.05, 0.15), rng.uniform(1.0, 2.0), rng.uniform(1.8, 2.8))
        D, a, r0 = seen[orb]
        out.append((i, j, D, a, r0))
    B, s0 = 0.006, 1.0
    params = [len(out)]
    for t in out:
        params += list(t)
    params += [5, 0, 1, B, s0]
    return np.array(params, dtype=float), perm


def v_synth9(x, params):
    npair = int(params[0])
    X = x.reshape(9, 3)
    v = 0.0
    for q in range(npair):
        i, j, D, a, r0 = params[1 + 5 * q: 6 + 5 * q]
        r = np.linalg.norm(X[int(i)] - X[int(j)])
        v += D * (1 - np.exp(-a * (r - r0))) ** 2
    iH, iO1, iO2, B, s0 = params[1 + 5 * npair: 6 + 5 * npair]
    s = np.linalg.norm(X[int(iH)] - X[int(iO1)]) - np.linalg.norm(X[int(iH)] - X[int(iO2)])
    return v + B * ((s / s0) ** 2 - 1) ** 2


def synth18_params():
    return np.array([6, 0.5, 1.81, 0.16, np.deg2rad(104.52), 2.4e-4, 5.96, -0.82, 0.41])


def v_synth18(x, p):
    nmol = int(p[0])
    kr, re, kth, the, eps, sig, qO, qH = p[1:9]
    X = x.reshape(3 * nmol, 3)
    v = 0.0
    for m in range(nmol):
        O, H1, H2 = X[3 * m], X[3 * m + 1], X[3 * m + 2]
        u1, u2 = H1 - O, H2 - O
        r1, r2 = np.linalg.norm(u1), np.linalg.norm(u2)
        ct = np.clip(u1 @ u2 / (r1 * r2), -1, 1)
        v += 0.5 * kr * ((r1 - re) ** 2 + (r2 - re) ** 2) + 0.5 * kth * (np.arccos(ct) - the) ** 2
    q = np.array([qO, qH, qH] * nmol)
    mol = np.repeat(np.arange(nmol), 3)
    for i in range(3 * nmol):
        for j in range(i + 1, 3 * nmol):
            if mol[i] == mol[j]:
                continue
            r = np.linalg.norm(X[i] - X[j])
            v += q[i] * q[j] / r
            if i % 3 == 0 and j % 3 == 0:
                v += 4 * eps * ((sig / r) ** 12 - (sig / r) ** 6)
    return v


def g_synth18(x, p):
    """Analytic gradient of v_synth18 (for tight well minimisation)."""
    nmol = int(p[0])
    kr, re, kth, the, eps, sig, qO, qH = p[1:9]
    X = x.reshape(3 * nmol, 3)
    G = np.zeros_like(X)
    for m in range(nmol):
        iO, i1, i2 = 3 * m, 3 * m + 1, 3 * m + 2
        u1, u2 = X[i1] - X[iO], X[i2] - X[iO]
        r1, r2 = np.linalg.norm(u1), np.linalg.norm(u2)
        n1, n2 = u1 / r1, u2 / r2
        ct = np.clip(n1 @ n2, -1, 1)
        st = max(np.sqrt(1 - ct * ct), 1e-12)
        dth = kth * (np.arccos(ct) - the)
        g1 = kr * (r1 - re) * n1 - dth * (n2 - ct * n1) / (r1 * st)
        g2 = kr * (r2 - re) * n2 - dth * (n1 - ct * n2) / (r2 * st)
        G[i1] += g1
        G[i2] += g2
        G[iO] -= g1 + g2
    q = np.array([qO, qH, qH] * nmol)
    mol = np.repeat(np.arange(nmol), 3)
    for i in range(3 * nmol):
        for j in range(i + 1, 3 * nmol):
            if mol[i] == mol[j]:
                continue
            d = X[i] - X[j]
            r2 = d @ d
            r = np.sqrt(r2)
            dv = -q[i] * q[j] / (r2 * r)
            if i % 3 == 0 and j % 3 == 0:
                sr6 = (sig * sig / r2) ** 3
                dv += 4 * eps * (-12 * sr6 * sr6 + 6 * sr6) / r2
            G[i] += dv * d
            G[j] -= dv * d
    return G.ravel()


def g_synth9(x, params):
    """Analytic gradient of v_synth9."""
    npair = int(params[0])
    X = x.reshape(9, 3)
    G = np.zeros_like(X)
    for q in range(npair):
        i, j, D, a, r0 = params[1 + 5 * q: 6 + 5 * q]
        i, j = int(i), int(j)
        d = X[i] - X[j]
        r = np.linalg.norm(d)
        e = np.exp(-a * (r - r0))
        dv = 2 * D * a * (1 - e) * e / r
        G[i] += dv * d
        G[j] -= dv * d
    iH, iO1, iO2, B, s0 = params[1 + 5 * npair: 6 + 5 * npair]
    iH, iO1, iO2 = int(iH), int(iO1), int(iO2)
    e1, e2 = X[iH] - X[iO1], X[iH] - X[iO2]
    r1, r2 = np.linalg.norm(e1), np.linalg.norm(e2)
    s = r1 - r2
    dvds = 4 * B * ((s / s0) ** 2 - 1) * s / s0 ** 2
    G[iH] += dvds * (e1 / r1 - e2 / r2)
    G[iO1] -= dvds * e1 / r1
    G[iO2] += dvds * e2 / r2
    return G.ravel()


# ---------------------------------------------------------------- helpers
def ring_dt(eta2_max, P, betan, tau=1.0):
    lam1 = 2.0 * np.sin(PI_REF / (2 * P + 2)) / betan
    w = np.sqrt(1.0 + max(eta2_max, 0.0) / lam1 ** 2) / tau
    return float(2 * np.pi / w / 20.0)


def mass_weighted_eigs(H, masses_per_dof):
    s = 1.0 / np.sqrt(masses_per_dof)
    return np.linalg.eigvalsh(H * s[:, None] * s[None, :])


def write(name, d):
    with open(os.path.join(HERE, name + ".json"), "w") as f:
        json.dump(d, f, indent=1)


def gl_nodes(n):
    x, w = np.polynomial.legendre.leggauss(n)
    return list(0.5 * (x + 1)), list(0.5 * w)


# ---------------------------------------------------------------- configurations
def c0():
    m = MP
    H, x0 = 1.0, 1.0
    wb = np.sqrt(4 * H / (m * x0 * x0))
    beta_c = 2 * np.pi / wb
    beta = 4 * beta_c
    P = 32
    betan = beta / (P + 1)
    eta2_max = 8 * H / (x0 * x0) / m  # V''(+-x0) / m
    dt = ring_dt(eta2_max, P, betan)
    return dict(name="c0", description="mcmod_1d, 1 particle, FP64, P=32, beta = 4 beta_c, Langevin",
                pes_id=1, ndim=1, natom=1, mass=[m], params=[H, x0], V0=0.0, P=P, beta=beta,
                beta_c=beta_c, dt=dt, tau=1.0, gamma=1.0 / (100 * dt), thermostat=2, nmc=20000,
                imin=1000, nintegral=11, nrep=1, well1=[-1.0], well2=[1.0], init_sigma=0.01,
                seeds=[0], precision="fp64")


def c1():
    m = MP
    f = v_2dtest
    r = minimize(f, np.array([3.0, 0.0]), method="BFGS", options=dict(gtol=1e-12))
    w1 = r.x
    ang = 2 * PI_REF / 6
    w2 = np.array([np.cos(ang) * w1[0] - np.sin(ang) * w1[1], np.sin(ang) * w1[0] + np.cos(ang) * w1[1]])
    # transition state on the bisecting ray
    ray = np.array([np.cos(ang / 2), np.sin(ang / 2)])
    rr = minimize(lambda t: f(t[0] * ray), np.array([2.5]), method="Nelder-Mead",
                  options=dict(xatol=1e-12, fatol=1e-15)).x[0]
    ts = rr * ray
    eta_ts = mass_weighted_eigs(num_hess(f, ts), np.array([m, m]))
    beta_c = 2 * np.pi / np.sqrt(-eta_ts.min())
    beta = 4 * beta_c
    P = 128
    betan = beta / (P + 1)
    eta_w = mass_weighted_eigs(num_hess(f, w1), np.array([m, m]))
    dt = ring_dt(eta_w.max(), P, betan)
    V0 = f(w1)
    return dict(name="c1", description="mcmod_2dtest, P=128, 1024 traj x 16 lambda, 50000 steps",
                pes_id=2, ndim=2, natom=1, mass=[m], params=[6, 2.0, 0.2, 3.0], V0=V0, P=P,
                beta=beta, beta_c=beta_c, dt=dt, tau=1.0, gamma=1.0 / (100 * dt), thermostat=2,
                nmc=50000, imin=2000, nintegral=16, nrep=1024, well1=list(w1), well2=list(w2),
                ts=list(ts), barrier=f(ts) - V0, init_sigma=0.02, seeds=list(range(1024)),
                precision="mixed")


def c2():
    """Synthetic 9-atom surface.  The drawn Morse network alone holds the
    transferring proton H* midway between O1 and O2 (s = 0); the quartic term
    B ((s/s0)^2 - 1)^2 (B = 0.006 Eh) turns that into a symmetric double well when
    its negative curvature at s = 0 beats the network's.  s0 is set from the
    network's curvature k along the O1 -> O2 axis at the symmetric minimum,
    s0 = sqrt(8 B / k), which makes the total curvature there -k."""
    params, perm = synth9_params(7)
    masses = np.array([16, 16, 12, 12, 12, 1, 1, 1, 1], dtype=float) * AMU
    X = np.array([[-2.3, 1.3, 0.0], [2.3, 1.3, 0.0], [-2.4, -1.0, 0.0], [0.0, -2.2, 0.0],
                  [2.4, -1.0, 0.0], [-0.9, 2.2, 0.0], [-4.3, -1.8, 0.0], [0.0, -4.2, 0.0],
                  [4.3, -1.8, 0.0]])
    X[:, 2] += 0.05 * np.random.RandomState(7).randn(9)
    npair = int(params[0])
    iB = 1 + 5 * npair + 3
    # 1) symmetric minimum of the network with the quartic switched off
    p0 = params.copy()
    p0[iB] = 0.0
    fg0 = lambda x: (v_synth9(x, p0), g_synth9(x, p0))
    xs = minimize(fg0, X.ravel(), jac=True, method="BFGS", options=dict(gtol=1e-11, maxiter=20000)).x.reshape(9, 3)
    # 2) curvature of the network along the O1 -> O2 axis for the proton
    e = xs[1] - xs[0]
    e /= np.linalg.norm(e)
    h = 1e-4

    def vdelta(dl):
        y = xs.copy()
        y[5] = y[5] + dl * e
        return v_synth9(y.ravel(), p0)

    k = (vdelta(h) - 2 * vdelta(0.0) + vdelta(-h)) / (h * h)
    s0 = float(np.sqrt(8.0 * 0.006 / k))
    params[iB + 1] = s0
    f = lambda x: v_synth9(x, params)
    fg = lambda x: (v_synth9(x, params), g_synth9(x, params))
    # 3) well 1: proton displaced towards O1 (s < 0), relaxed
    y = xs.copy()
    y[5] = y[5] - 0.5 * s0 * e
    w1 = minimize(fg, y.ravel(), jac=True, method="BFGS", options=dict(gtol=1e-11, maxiter=20000)).x.reshape(9, 3)
    w1 = w1 - (masses[:, None] * w1).sum(0) / masses.sum()
    # 4) well 2: mirror-permuted copy aligned onto well 1 (Kabsch, reflection allowed), relaxed
    B = w1[perm]
    Hm = B.T @ (w1 * masses[:, None])
    U, S, Vt = np.linalg.svd(Hm)
    Rm = (U @ Vt).T
    w2 = B @ Rm.T
    w2 = minimize(fg, w2.ravel(), jac=True, method="BFGS", options=dict(gtol=1e-11, maxiter=20000)).x.reshape(9, 3)
    # barrier: relaxed symmetric (s = 0) geometry
    xts = minimize(lambda x: (v_synth9(x, params) + 50.0 * (np.linalg.norm(x.reshape(9, 3)[5] - x.reshape(9, 3)[0])
                                                            - np.linalg.norm(x.reshape(9, 3)[5] - x.reshape(9, 3)[1])) ** 2),
                   xs.ravel(), method="BFGS", options=dict(gtol=1e-10, maxiter=20000)).x
    V0 = f(w1.ravel())
    dofm = np.repeat(masses, 3)
    eta = mass_weighted_eigs(num_hess(f, w1.ravel(), 1e-4), dofm)
    T = 50.0
    beta = 1.0 / (KB * T)
    P = 256
    betan = beta / (P + 1)
    dt = ring_dt(eta.max(), P, betan)
    sfun = lambda w: float(np.linalg.norm(w[5] - w[0]) - np.linalg.norm(w[5] - w[1]))
    return dict(name="c2", description="synthetic 9-atom Morse network + proton-transfer well, P=256, "
                "256 traj x 12 lambda, T=50 K", pes_id=3, ndim=3, natom=9, mass=list(masses),
                params=list(params), V0=V0, P=P, beta=beta, dt=dt, tau=1.0, gamma=1.0 / (100 * dt),
                thermostat=2, nmc=20000, imin=1000, nintegral=12, nrep=256, well1=list(w1.ravel()),
                well2=list(w2.ravel()), Vwell2_minus_V0=f(w2.ravel()) - V0, s0=s0, network_curvature=k,
                s_well1=sfun(w1), s_well2=sfun(w2), well_separation=float(np.linalg.norm(w1 - w2)),
                barrier=f(xts) - V0, init_sigma=0.0, seeds=list(range(256)), precision="mixed",
                eta2_well=list(eta))


def c3(c2d):
    T = np.linspace(100.0, 20.0, 32)
    betas = list(1.0 / (KB * T))
    return dict(name="c3", description="instanton on the c2 surface, N=512, 32 beta values",
                pes_id=3, ndim=3, natom=9, mass=c2d["mass"], params=c2d["params"], V0=c2d["V0"],
                N=512, betas=betas, temperatures=list(T), lbfgs_m=10, well1=c2d["well1"],
                well2=c2d["well2"])


def c4():
    p = synth18_params()
    rng = np.random.RandomState(11)
    nmol = 6
    R = 5.3
    X = []
    for m in range(nmol):
        ang = 2 * np.pi * m / nmol
        O = np.array([R * np.cos(ang), R * np.sin(ang), 0.0]) + 0.2 * rng.randn(3)
        # water in its own frame, one H pointing to the next molecule
        th = np.deg2rad(104.52)
        t = np.array([-np.sin(ang), np.cos(ang), 0.0])
        n = np.array([np.cos(ang), np.sin(ang), 0.0])
        z = np.array([0.0, 0.0, 1.0])
        rot = rng.randn(3) * 0.2
        h1 = 1.81 * (np.cos(0.0) * t + rot)
        h1 = 1.81 * h1 / np.linalg.norm(h1)
        h2dir = np.cos(th) * t + np.sin(th) * (0.5 * n + 0.87 * z)
        h2 = 1.81 * h2dir / np.linalg.norm(h2dir)
        X += [O, O + h1, O + h2]
    X = np.array(X)
    f = lambda x: v_synth18(x, p)
    fg = lambda x: (v_synth18(x, p), g_synth18(x, p))
    r = minimize(fg, X.ravel(), jac=True, method="BFGS", options=dict(maxiter=50000, gtol=1e-11))
    w1 = r.x.reshape(-1, 3)
    masses = np.array([16, 1, 1] * nmol, dtype=float) * AMU
    w1 = w1 - (masses[:, None] * w1).sum(0) / masses.sum()
    w2 = w1.copy()
    w2[[1, 2]] = w2[[2, 1]]  # swap the H labels of molecule 0
    V0 = f(w1.ravel())
    T = 100.0
    beta = 1.0 / (KB * T)
    dofm = np.repeat(masses, 3)
    eta = mass_weighted_eigs(num_hess(f, w1.ravel(), 1e-4), dofm)
    Ps = [64, 128, 256, 512]
    dts = {str(P): ring_dt(eta.max(), P, beta / (P + 1)) for P in Ps}
    dt = min(dts.values())
    nring = 4096
    Pring = list(np.random.RandomState(11).choice(Ps, size=nring).astype(int).tolist())
    return dict(name="c4", description="synthetic 18-atom water hexamer, 4096 rings with P in "
                "{64,128,256,512}", pes_id=4, ndim=3, natom=18, mass=list(masses), params=list(p),
                V0=V0, Ps=Ps, P_per_ring=Pring, beta=beta, dt=dt, dt_per_P=dts, tau=1.0,
                gamma=1.0 / (100 * dt), thermostat=2, nmc=5000, imin=500, nintegral=8,
                well1=list(w1.ravel()), well2=list(w2.ravel()), init_sigma=0.0,
                precision="mixed", eta2_well_max=float(eta.max()))


if __name__ == "__main__":
    d0 = c0()
    write("c0", d0)
    d1 = c1()
    write("c1", d1)
    d2 = c2()
    write("c2", d2)
    write("c3", c3(d2))
    write("c4", c4())
    print("c0 beta=%.4f dt=%.5f" % (d0["beta"], d0["dt"]))
    print("c1 beta=%.4f dt=%.5f barrier=%.5f" % (d1["beta"], d1["dt"], d1["barrier"]))
    print("c2 dt=%.6f V(w2)-V0=%.3e s0=%.4f s1=%.4f s2=%.4f |w1-w2|=%.4f barrier=%.5f" % (
        d2["dt"], d2["Vwell2_minus_V0"], d2["s0"], d2["s_well1"], d2["s_well2"], d2["well_separation"],
        d2["barrier"]))
