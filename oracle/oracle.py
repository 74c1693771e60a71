"""ctypes wrapper around liboracle.so, plus the scipy-based pieces of the oracle.

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU legs of ``bench.py``; the product library never uses it.

Parity unpinned: the reference (Fortran + MKL + MPI) cannot be built here and
ships no golden vectors; the oracle is pinned to analytic known answers.

Scipy pieces:
  * ``instanton_lbfgs`` drives scipy's L-BFGS-B (v3.0, the algorithm vendored as
    lbfgsb.f in the reference) on the C action/gradient, with the reference's
    settings m, factr=1e6, pgtol=eps2 (instantonmod.f90:715-724);
  * ``logdet_band`` calls LAPACK dsbevd through scipy on the lower band storage,
    as detJ does (instantonmod.f90:782-827).
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

PES_1D, PES_2DTEST, PES_SYNTH9, PES_SYNTH18, PES_HARMONIC, PES_DISTGAUSS = 1, 2, 3, 4, 5, 6
PI_REF = 3.14159265358979


class _Pes(C.Structure):
    _fields_ = [("id", C.c_int32), ("ndim", C.c_int32), ("natom", C.c_int32),
                ("nparams", C.c_int32), ("V0", C.c_double), ("params", C.POINTER(C.c_double))]


class _TiParams(C.Structure):
    _fields_ = [("P", C.c_int64), ("beta", C.c_double), ("betan", C.c_double),
                ("dt", C.c_double), ("tau", C.c_double), ("gamma", C.c_double),
                ("thermostat", C.c_int32), ("cayley", C.c_int32), ("nm_resident", C.c_int32),
                ("pad", C.c_int32), ("imin", C.c_int64), ("noutput", C.c_int64),
                ("dhdr_limit", C.c_double), ("init_sigma", C.c_double)]


class RingResult(C.Structure):
    _fields_ = [("dhdr_sum", C.c_double), ("nsamples", C.c_int64), ("nreinit", C.c_int64),
                ("and_count", C.c_int64), ("and_rkick", C.c_int64), ("status", C.c_int32),
                ("pad", C.c_int32)]


def build():
    """Compile liboracle.so with the committed Makefile (gcc, portable flags)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        src = os.path.join(_HERE, "oracle.c")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            build()
        _LIB = C.CDLL(path)
        _declare(_LIB)
    return _LIB


def _declare(L):
    D, I64, I32, U32, U64, P = C.c_double, C.c_int64, C.c_int32, C.c_uint32, C.c_uint64, C.c_void_p
    L.or_V.restype = D
    L.or_V.argtypes = [P, P]
    L.or_Vprime.argtypes = [P, P, P]
    L.or_potforce.restype = D
    L.or_potforce.argtypes = [P, P, P]
    L.or_Vdoubleprime.argtypes = [P, P, P, C.c_int]
    L.or_philox4x32_10.argtypes = [P, P, P]
    L.or_normal.restype = D
    L.or_normal.argtypes = [U64, U32, U32, U32, U32]
    L.or_uniform.restype = D
    L.or_uniform.argtypes = [U64, U32, U32, U32, U32]
    L.or_poisson.restype = I64
    L.or_poisson.argtypes = [U64, U32, U32, U32, D]
    L.or_init_nm.argtypes = [I64, I64, I64, P, D, D, P, P, P, P, P, P]
    L.or_nm_forward.argtypes = [I64, P, P, P, P]
    L.or_nm_backward.argtypes = [I64, P, P, P, P]
    L.or_ring_init.argtypes = [P, P, P, P, P, P, U64, U32, U32, U32, U32, P, P]
    L.or_ring_propagate.argtypes = [P, P, P, P, P, P, P, U64, U32, I64, I64, P, P, P]
    L.or_ti_run_batch.restype = C.c_int
    L.or_ti_run_batch.argtypes = [P, P, P, I64, P, P, P, P, P, P, P, I64, I32, P, P, P]
    L.or_UM.restype = D
    L.or_UM.argtypes = [P, P, I64, D, P, P, P, C.c_int]
    L.or_UMprime.argtypes = [P, P, I64, D, P, P, P, C.c_int, P]
    L.or_UMforceenergy.restype = D
    L.or_UMforceenergy.argtypes = [P, P, I64, D, P, P, P, C.c_int, P]
    L.or_UMhessian.argtypes = [P, P, I64, D, P, C.c_int, C.c_int, P]
    L.or_gauleg.argtypes = [D, D, P, P, I64]
    L.or_spline.argtypes = [P, P, I64, D, D, P]
    L.or_splint.restype = D
    L.or_splint.argtypes = [P, P, P, I64, D]
    L.or_splin_grad.restype = D
    L.or_splin_grad.argtypes = [P, P, P, I64, D]
    L.or_locate.restype = I64
    L.or_locate.argtypes = [P, I64, D]
    L.or_ti_assemble.argtypes = [I64, I64, P, P, D, P, P, P]


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Pes:
    """One PES (mcmod module) instance: id, shape, parameter vector, V0."""

    def __init__(self, pes_id, ndim, natom, params=(), V0=0.0):
        self.id, self.ndim, self.natom = int(pes_id), int(ndim), int(natom)
        self.params = _f64(np.asarray(params, dtype=np.float64).ravel())
        if self.params.size == 0:
            self.params = np.zeros(1)
            n = 0
        else:
            n = self.params.size
        self.V0 = float(V0)
        self._s = _Pes(self.id, self.ndim, self.natom, n, self.V0,
                       self.params.ctypes.data_as(C.POINTER(C.c_double)))

    @property
    def ndof(self):
        return self.ndim * self.natom

    def ref(self):
        return C.byref(self._s)

    def V(self, x):
        x = _f64(x)
        return lib().or_V(self.ref(), _p(x))

    def Vprime(self, x):
        x = _f64(x)
        g = np.zeros(self.ndof)
        lib().or_Vprime(self.ref(), _p(x), _p(g))
        return g

    def potforce(self, x):
        x = _f64(x)
        g = np.zeros(self.ndof)
        v = lib().or_potforce(self.ref(), _p(x), _p(g))
        return v, g

    def Vdoubleprime(self, x, quirks=False):
        """hess[a, b] = d grad_b / d x_a (reference memory order a + ndof*b)."""
        x = _f64(x)
        h = np.zeros(self.ndof * self.ndof)
        lib().or_Vdoubleprime(self.ref(), _p(x), _p(h), int(bool(quirks)))
        return h.reshape(self.ndof, self.ndof, order="F")


# ---------------------------------------------------------------- RNG
def philox(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    o = np.zeros(4, dtype=np.uint32)
    lib().or_philox4x32_10(_p(c), _p(k), _p(o))
    return o


def normal(seed, stream, step, purpose, n):
    return lib().or_normal(seed, stream, step, purpose, n)


def uniform(seed, stream, step, purpose, n):
    return lib().or_uniform(seed, stream, step, purpose, n)


def poisson(seed, stream, step, purpose, mean):
    return lib().or_poisson(seed, stream, step, purpose, mean)


# ---------------------------------------------------------------- normal modes
def init_nm(P, ndim, natom, mass, betan, tau, a, b):
    nd = ndim * natom
    T = np.zeros(P * P)
    lam = np.zeros(P)
    bm = np.zeros(natom * P)
    bv = np.zeros(P * nd)
    lib().or_init_nm(P, ndim, natom, _p(_f64(mass)), betan, tau, _p(_f64(a)), _p(_f64(b)),
                     _p(T), _p(lam), _p(bm), _p(bv))
    return (T.reshape(P, P, order="F"), lam, bm.reshape(natom, P, order="F"),
            bv.reshape(P, nd, order="F"))


def nm_forward(T, x, shift=None):
    P = T.shape[0]
    Tf = _f64(T.ravel(order="F"))
    q = np.zeros(P)
    s = _f64(shift) if shift is not None else None
    lib().or_nm_forward(P, _p(Tf), _p(_f64(x)), _p(q), _p(s) if s is not None else None)
    return q


def nm_backward(T, q, shift=None):
    P = T.shape[0]
    Tf = _f64(T.ravel(order="F"))
    x = np.zeros(P)
    s = _f64(shift) if shift is not None else None
    lib().or_nm_backward(P, _p(Tf), _p(_f64(q)), _p(x), _p(s) if s is not None else None)
    return x


# ---------------------------------------------------------------- TI
class TiParams:
    def __init__(self, P, beta, dt, tau=1.0, gamma=1.0, thermostat=2, cayley=False,
                 nm_resident=False, imin=0, noutput=100000, dhdr_limit=-1.0, init_sigma=0.0,
                 betan=None):
        self.P = int(P)
        self.beta = float(beta)
        self.betan = float(beta / (P + 1)) if betan is None else float(betan)
        self.dt, self.tau, self.gamma = float(dt), float(tau), float(gamma)
        self.thermostat, self.cayley, self.nm_resident = int(thermostat), int(cayley), int(nm_resident)
        self.imin, self.noutput = int(imin), int(noutput)
        self.dhdr_limit, self.init_sigma = float(dhdr_limit), float(init_sigma)

    def struct(self):
        return _TiParams(self.P, self.beta, self.betan, self.dt, self.tau, self.gamma,
                         self.thermostat, self.cayley, self.nm_resident, 0, self.imin,
                         self.noutput, self.dhdr_limit, self.init_sigma)


def new_result():
    r = RingResult()
    r.and_rkick = -1
    return r


def ring_init(pes, mass, prm, xref, seed, stream, step=0, purpose_x=2, purpose_p=1, a=None, b=None):
    nd = pes.ndof
    P = prm.P
    a = np.zeros(nd) if a is None else a
    b = np.zeros(nd) if b is None else b
    T, lam, bm, bv = init_nm(P, pes.ndim, pes.natom, mass, prm.betan, prm.tau, a, b)
    x = np.zeros(nd * P)
    p = np.zeros(nd * P)
    s = prm.struct()
    lib().or_ring_init(pes.ref(), _p(_f64(mass)), C.byref(s), _p(_f64(T.ravel(order="F"))),
                       _p(_f64(bm.ravel(order="F"))), _p(_f64(xref)), seed, stream, step,
                       purpose_x, purpose_p, _p(x), _p(p))
    return x, p


def ring_propagate(pes, mass, prm, a, b, dbdl, xref, seed, stream, step0, nsteps, x, p, res=None):
    """In-place propagation of one ring; returns the RingResult (accumulating)."""
    if res is None:
        res = new_result()
    s = prm.struct()
    assert x.dtype == np.float64 and x.flags.c_contiguous
    assert p.dtype == np.float64 and p.flags.c_contiguous
    lib().or_ring_propagate(pes.ref(), _p(_f64(mass)), C.byref(s), _p(_f64(a)), _p(_f64(b)),
                            _p(_f64(dbdl)), _p(_f64(xref)), seed, stream, step0, nsteps,
                            _p(x), _p(p), C.byref(res))
    return res


def ti_run_batch(pes, mass, prm, lam_index, seeds, streams, a, b, dbdl, xref, nsteps,
                 nthreads, x, p):
    nr = len(lam_index)
    res = (RingResult * nr)()
    li = np.ascontiguousarray(lam_index, dtype=np.int32)
    sd = np.ascontiguousarray(seeds, dtype=np.uint64)
    stv = np.ascontiguousarray(streams, dtype=np.uint32)
    s = prm.struct()
    lib().or_ti_run_batch(pes.ref(), _p(_f64(mass)), C.byref(s), nr, _p(li), _p(sd), _p(stv),
                          _p(_f64(a)), _p(_f64(b)), _p(_f64(dbdl)), _p(_f64(xref)), nsteps,
                          int(nthreads), _p(x), _p(p), res)
    return res


# ---------------------------------------------------------------- instanton
def UM(pes, mass, N, betan, x, a, b, fixedends=True):
    return lib().or_UM(pes.ref(), _p(_f64(mass)), N, betan, _p(_f64(x)), _p(_f64(a)),
                       _p(_f64(b)), int(fixedends))


def UMprime(pes, mass, N, betan, x, a, b, fixedends=True):
    g = np.zeros(N * pes.ndof)
    lib().or_UMprime(pes.ref(), _p(_f64(mass)), N, betan, _p(_f64(x)), _p(_f64(a)),
                     _p(_f64(b)), int(fixedends), _p(g))
    return g


def UMforceenergy(pes, mass, N, betan, x, a, b, fixedends=True):
    g = np.zeros(N * pes.ndof)
    v = lib().or_UMforceenergy(pes.ref(), _p(_f64(mass)), N, betan, _p(_f64(x)), _p(_f64(a)),
                               _p(_f64(b)), int(fixedends), _p(g))
    return v, g


def UMhessian(pes, mass, N, betan, x, singlewell=False, quirks=False):
    nd = pes.ndof
    band = np.zeros((nd + 1) * N * nd)
    lib().or_UMhessian(pes.ref(), _p(_f64(mass)), N, betan, _p(_f64(x)), int(singlewell),
                       int(quirks), _p(band))
    return band.reshape(nd + 1, N * nd, order="F")


def band_eigvals(band):
    """All eigenvalues of the lower-band matrix (dsbevd, as instantonmod.f90:823)."""
    from scipy.linalg import lapack
    w, _z, info = lapack.dsbevd(np.asfortranarray(band), compute_v=0, lower=1)
    if info != 0:
        raise RuntimeError("dsbevd info=%d" % info)
    return w


def logdet_band(band, skip_lowest):
    """Sum of log(eta^2) over eta^2 > 0 (rpi_ser.f90:227-236, 354-365); skip_lowest
    drops the first eigenvalue as rpi_ser does for the instanton."""
    w = band_eigvals(band)
    start = 1 if skip_lowest else 0
    ww = w[start:]
    pos = ww > 0.0
    return float(np.sum(np.log(ww[pos]))), int(np.sum(~pos)), float(w[0])


def instanton_lbfgs(pes, mass, N, betan, x0, a, b, m=8, factr=1.0e6, pgtol=1.0e-5, maxiter=15000,
                    fixedends=True):
    """scipy L-BFGS-B on UM, unbounded (instantonmod.f90:679-777); with
    fixedends False the action without the end-point springs (a, b unused)."""
    from scipy.optimize import minimize
    nd = pes.ndim * pes.natom
    if not fixedends:
        a = np.zeros(nd) if a is None else a
        b = np.zeros(nd) if b is None else b

    def fg(x):
        v, g = UMforceenergy(pes, mass, N, betan, x, a, b, fixedends)
        return v, g

    r = minimize(fg, _f64(x0), jac=True, method="L-BFGS-B",
                 options=dict(maxcor=m, ftol=factr * np.finfo(float).eps, gtol=pgtol,
                              maxiter=maxiter, maxfun=4 * maxiter))
    return r.x, r.fun, r


def crossover_beta(pes, mass, ts, quirks=False):
    """crossover.f90:49-71: eigenvalues of the mass-weighted Hessian at the
    transition state (dsyevd there, LAPACK syevd through numpy here) and
    beta_c = 2 pi / sqrt(-eta^2_min).  Every atom pair is mass-weighted (the
    reference's second atom loop stops at ndim, crossover.f90:56)."""
    H = pes.Vdoubleprime(_f64(ts), quirks=quirks)
    s = 1.0 / np.sqrt(np.repeat(_f64(mass), pes.ndim))
    eta2 = np.linalg.eigvalsh(H * s[:, None] * s[None, :])
    return 2.0 * PI_REF / np.sqrt(-eta2[0]), eta2


# ---------------------------------------------------------------- quadrature / splines
def gauleg(x1, x2, n):
    x = np.zeros(n)
    w = np.zeros(n)
    lib().or_gauleg(x1, x2, _p(x), _p(w), n)
    return x, w


def spline(x, y, yp1=1.0e31, ypn=1.0e31):
    n = len(x)
    y2 = np.zeros(n)
    lib().or_spline(_p(_f64(x)), _p(_f64(y)), n, yp1, ypn, _p(y2))
    return y2


def splint(xa, ya, y2a, x):
    return lib().or_splint(_p(_f64(xa)), _p(_f64(ya)), _p(_f64(y2a)), len(xa), x)


def splin_grad(xa, ya, y2a, x):
    return lib().or_splin_grad(_p(_f64(xa)), _p(_f64(ya)), _p(_f64(y2a)), len(xa), x)


def ti_assemble(weights, integrands, nrep, betan):
    nint = len(weights)
    dA = C.c_double()
    sA = C.c_double()
    q = C.c_double()
    lib().or_ti_assemble(nint, nrep, _p(_f64(weights)), _p(_f64(integrands)), betan,
                         C.byref(dA), C.byref(sA), C.byref(q))
    return dA.value, sA.value, q.value
