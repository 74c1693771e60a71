"""ctypes binding of libpimdgpu.so (include/pimdgpu.h).

This is the binding a Python caller (the tests, bench.py) uses; the Fortran
binding is ``fortran/pimdgpu_mod.f90`` and the C++ drivers link the library
directly.  Every call goes to the CUDA library; there is no CPU fallback and
loading fails loudly when the shared library has not been built.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_PKG = os.path.dirname(_HERE)
LIBPATH = os.path.join(_PKG, "lib", "libpimdgpu.so")

PG_OK, PG_ERR_ARG, PG_ERR_CUDA, PG_ERR_STATE, PG_ERR_UNSUPPORTED, PG_ERR_IO, PG_ERR_NUMERIC = range(7)
PG_PES_1D, PG_PES_2DTEST, PG_PES_SYNTH9, PG_PES_SYNTH18, PG_PES_HARMONIC, PG_PES_DISTGAUSS = 1, 2, 3, 4, 5, 6
PG_FP64, PG_MIXED = 0, 1
PG_FORM_AUTO, PG_FORM_PLAIN, PG_FORM_FUSED, PG_FORM_TENSOR = 0, 1, 2, 3
PG_TUNE_OFF, PG_TUNE_CACHE, PG_TUNE_ON = 0, 1, 2
PG_ANDERSEN, PG_LANGEVIN = 1, 2
PG_RING_NAN, PG_RING_TIMEOUT = 1, 2  # per-ring status bits

# Every symbol include/pimdgpu.h declares.
EXPORTS = [
    "pg_create", "pg_destroy", "pg_last_error", "pg_version", "pg_set_system", "pg_pes_eval",
    "pg_pes_hessian", "pg_nm_transform", "pg_ti_setup", "pg_ti_advance", "pg_ti_get_state",
    "pg_ti_get_results", "pg_ti_lambda_reduce", "pg_ti_get_step", "pg_ti_advance_timed", "pg_ti_get_form", "pg_ti_kernel_times", "pg_set_tuning", "pg_ti_get_tuning", "pg_ti_checkpoint_save",
    "pg_ti_checkpoint_load", "pg_ti_release", "pg_propagate_pimd", "pg_gauleg", "pg_spline",
    "pg_splint", "pg_ti_assemble", "pg_splitting_from_ratio", "pg_splitting_two_beta", "pg_irrep_ratios",
    "pg_set_fixedends", "pg_instanton_fg",
    "pg_instanton_optimize", "pg_um_hessian", "pg_instanton_logdet", "pg_rpi_assemble",
    "pg_nm_transform_noalloc", "pg_set_wait_limit", "pg_fp32_peak", "pg_ti_advance_group", "pg_ti_set_accumulators",
]


class TiConfig(C.Structure):
    _fields_ = [("nbeads", C.c_int64), ("beta", C.c_double), ("dt", C.c_double),
                ("tau", C.c_double), ("gamma", C.c_double), ("thermostat", C.c_int32),
                ("precision", C.c_int32), ("form", C.c_int32), ("cayley", C.c_int32),
                ("imin", C.c_int64), ("noutput", C.c_int64), ("dhdr_limit", C.c_double),
                ("init_sigma", C.c_double)]


class LbfgsOpts(C.Structure):
    _fields_ = [("m", C.c_int32), ("max_backtracks", C.c_int32), ("maxiter", C.c_int64),
                ("factr", C.c_double), ("pgtol", C.c_double), ("cluster_ctas", C.c_int32),
                ("reserved", C.c_int32)]


class PgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("pimdgpu error %d: %s" % (code, msg))
        self.code = code


_LIB = None


def lib():
    """Load libpimdgpu.so (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIBPATH):
            raise OSError("libpimdgpu.so not found at %s: run the build first" % LIBPATH)
        L = C.CDLL(LIBPATH)
        P, I64, I32, D = C.c_void_p, C.c_int64, C.c_int32, C.c_double
        L.pg_last_error.restype = C.c_char_p
        L.pg_version.restype = I32
        L.pg_create.argtypes = [C.POINTER(C.c_void_p), I32]
        L.pg_destroy.argtypes = [P]
        L.pg_set_system.argtypes = [P, I64, I64, P, I32, P, I64, D]
        L.pg_pes_eval.argtypes = [P, I64, P, P, P, I32]
        L.pg_pes_hessian.argtypes = [P, I64, P, P, I32]
        L.pg_nm_transform.argtypes = [P, I64, I64, P, P, I32]
        L.pg_nm_transform_noalloc.argtypes = [I64, I64, P, P, P]
        L.pg_set_wait_limit.argtypes = [P, I64]
        L.pg_fp32_peak.argtypes = [P, P]
        L.pg_ti_setup.argtypes = [P, P, I64, I64, P, P, P, P, P, P, P, P, P]
        L.pg_ti_advance.argtypes = [P, I64]
        L.pg_ti_advance_timed.argtypes = [P, I64, P]
        L.pg_ti_advance_group.argtypes = [P, I64, I64, P]
        L.pg_ti_set_accumulators.argtypes = [P, P, P, I64]
        L.pg_ti_get_state.argtypes = [P, P, P]
        L.pg_ti_get_results.argtypes = [P, P, P, P, P]
        L.pg_ti_lambda_reduce.argtypes = [P, P, P, P]
        L.pg_ti_get_step.argtypes = [P, P]
        L.pg_ti_get_form.argtypes = [P, I64, P, P]
        L.pg_set_tuning.argtypes = [P, C.c_char_p, I32]
        L.pg_ti_get_tuning.argtypes = [P, P, P, P]
        L.pg_ti_kernel_times.argtypes = [P, I64, P, P, P, P, P]
        L.pg_ti_checkpoint_save.argtypes = [P, C.c_char_p]
        L.pg_ti_checkpoint_load.argtypes = [P, C.c_char_p]
        L.pg_ti_release.argtypes = [P]
        L.pg_propagate_pimd.argtypes = [P, P, I64, I64, P, P, P, P, P, P, P, P, P]
        L.pg_gauleg.argtypes = [D, D, P, P, I64]
        L.pg_spline.argtypes = [P, P, I64, D, D, P]
        L.pg_splint.argtypes = [P, P, P, I64, D, P, P]
        L.pg_ti_assemble.argtypes = [I64, P, P, P, D, P, P, P]
        L.pg_splitting_from_ratio.argtypes = [D, D, P]
        L.pg_splitting_two_beta.argtypes = [D, D, D, D, P, P]
        L.pg_irrep_ratios.argtypes = [I64, I64, P, P, P]
        L.pg_set_fixedends.argtypes = [P, I32]
        L.pg_instanton_fg.argtypes = [P, I64, I64, P, P, P, P, P, P]
        L.pg_instanton_optimize.argtypes = [P, I64, I64, P, P, P, P, P, P, P, P]
        L.pg_um_hessian.argtypes = [P, I64, D, P, I32, I32, P]
        L.pg_instanton_logdet.argtypes = [P, I64, I64, P, P, I32, I32, I32, P, P, P]
        L.pg_rpi_assemble.argtypes = [D, D, D, D, P, P, P]
        _LIB = L
    return _LIB


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def check(rc):
    if rc != PG_OK:
        raise PgError(rc, lib().pg_last_error().decode())


# ---------------------------------------------------------------- host helpers (no context)
def gauleg(x1, x2, n):
    x = np.zeros(n)
    w = np.zeros(n)
    check(lib().pg_gauleg(x1, x2, _p(x), _p(w), n))
    return x, w


def spline(x, y, yp1=1.0e31, ypn=1.0e31):
    x, y = _f64(x), _f64(y)
    y2 = np.zeros(len(x))
    check(lib().pg_spline(_p(x), _p(y), len(x), yp1, ypn, _p(y2)))
    return y2


def splint(xa, ya, y2a, x):
    xa, ya, y2a = _f64(xa), _f64(ya), _f64(y2a)
    y = C.c_double()
    g = C.c_double()
    check(lib().pg_splint(_p(xa), _p(ya), _p(y2a), len(xa), x, C.byref(y), C.byref(g)))
    return y.value, g.value


def ti_assemble(weights, mean, var, betan):
    w, m, v = _f64(weights), _f64(mean), _f64(var)
    dA, sA, q = C.c_double(), C.c_double(), C.c_double()
    check(lib().pg_ti_assemble(len(w), _p(w), _p(m), _p(v), betan, C.byref(dA), C.byref(sA), C.byref(q)))
    return dA.value, sA.value, q.value


def splitting_from_ratio(beta, qratio):
    d = C.c_double()
    check(lib().pg_splitting_from_ratio(beta, qratio, C.byref(d)))
    return d.value


def splitting_two_beta(beta1, ratio1, beta2, ratio2):
    """(Delta, beta_bar) from ratios at two inverse temperatures."""
    d, b = C.c_double(), C.c_double()
    check(lib().pg_splitting_two_beta(beta1, ratio1, beta2, ratio2, C.byref(d), C.byref(b)))
    return d.value, b.value


def irrep_ratios(chars, rho):
    """Level-pair ratio per irreducible representation; chars: (nirrep, nop)."""
    ch = _f64(np.atleast_2d(chars))
    r = _f64(rho)
    if ch.shape[1] != r.size:
        raise ValueError("chars has %d columns for %d operations" % (ch.shape[1], r.size))
    out = np.zeros(ch.shape[0])
    check(lib().pg_irrep_ratios(ch.shape[0], ch.shape[1], _p(ch), _p(r), _p(out)))
    return out


def rpi_assemble(betan, UM, lndetJ, lndetJ0):
    S, om, de = C.c_double(), C.c_double(), C.c_double()
    check(lib().pg_rpi_assemble(betan, UM, lndetJ, lndetJ0, C.byref(S), C.byref(om), C.byref(de)))
    return S.value, om.value, de.value


# ---------------------------------------------------------------- context
class Context:
    """One pg_ctx on one device."""

    def __init__(self, device=0):
        h = C.c_void_p()
        check(lib().pg_create(C.byref(h), device))
        self.h = h
        self.ndim = self.natom = 0

    def close(self):
        if self.h:
            lib().pg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def ndof(self):
        return self.ndim * self.natom

    def set_system(self, ndim, natom, mass, pes_id, params=(), V0=0.0):
        m = _f64(mass)
        pr = _f64(np.asarray(params, dtype=np.float64).ravel())
        check(lib().pg_set_system(self.h, ndim, natom, _p(m), pes_id, _p(pr) if pr.size else None,
                                  pr.size, V0))
        self.ndim, self.natom = ndim, natom

    def pes_eval(self, x, precision=PG_FP64):
        x = _f64(x)
        n = x.size // self.ndof
        V = np.zeros(n)
        g = np.zeros(n * self.ndof)
        check(lib().pg_pes_eval(self.h, n, _p(x), _p(V), _p(g), precision))
        return V, g.reshape(n, self.ndof)

    def pes_hessian(self, x, quirks=False):
        x = _f64(x)
        n = x.size // self.ndof
        h = np.zeros(n * self.ndof * self.ndof)
        check(lib().pg_pes_hessian(self.h, n, _p(x), _p(h), int(quirks)))
        return h.reshape(n, self.ndof, self.ndof).transpose(0, 2, 1)  # [c, a, b] = d g_b / d x_a

    def nm_transform(self, P, cols, precision=PG_FP64):
        cols = _f64(cols)
        ncol = cols.size // P
        out = np.zeros_like(cols)
        check(lib().pg_nm_transform(self.h, P, ncol, _p(cols), _p(out), precision))
        return out

    # ---- TI
    def ti_setup(self, cfg, ring_lambda, ring_seed, ring_stream, a, b, dbdl, xref=None, x0=None, p0=None):
        lam = np.ascontiguousarray(ring_lambda, dtype=np.int32)
        seed = np.ascontiguousarray(ring_seed, dtype=np.uint64)
        stream = np.ascontiguousarray(ring_stream, dtype=np.uint32)
        a, b, dbdl, xref, x0, p0 = map(_f64, (a, b, dbdl, xref, x0, p0))
        nl = b.size // self.ndof
        self._ti = (cfg.nbeads, len(lam), nl)
        check(lib().pg_ti_setup(self.h, C.byref(cfg), len(lam), nl, _p(lam), _p(seed), _p(stream),
                                _p(a), _p(b), _p(dbdl), _p(xref), _p(x0), _p(p0)))

    def ti_advance(self, nsteps):
        check(lib().pg_ti_advance(self.h, nsteps))

    def ti_advance_timed(self, nsteps):
        """Advance and return the device milliseconds (CUDA events on the library stream)."""
        ms = C.c_double()
        check(lib().pg_ti_advance_timed(self.h, nsteps, C.byref(ms)))
        return ms.value

    @staticmethod
    def ti_advance_group(contexts, nsteps):
        """Advance several contexts (e.g. one per bead number) concurrently;
        returns the device milliseconds spanning all of them."""
        arr = (C.c_void_p * len(contexts))(*[c.h for c in contexts])
        ms = C.c_double()
        check(lib().pg_ti_advance_group(arr, len(contexts), nsteps, C.byref(ms)))
        return ms.value

    def ti_set_accumulators(self, dhdr_sum, nsamples, step):
        d = np.ascontiguousarray(dhdr_sum, dtype=np.float64)
        n = np.ascontiguousarray(nsamples, dtype=np.int64)
        check(lib().pg_ti_set_accumulators(self.h, _p(d), _p(n), int(step)))

    def ti_state(self):
        P, nr, _ = self._ti
        x = np.zeros(nr * self.ndof * P)
        p = np.zeros(nr * self.ndof * P)
        check(lib().pg_ti_get_state(self.h, _p(x), _p(p)))
        return x, p

    def ti_results(self):
        _, nr, _ = self._ti
        s = np.zeros(nr)
        n = np.zeros(nr, dtype=np.int64)
        ri = np.zeros(nr, dtype=np.int64)
        st = np.zeros(nr, dtype=np.int32)
        check(lib().pg_ti_get_results(self.h, _p(s), _p(n), _p(ri), _p(st)))
        return s, n, ri, st

    def ti_step(self):
        """MD steps the batch has taken (pg_ti_get_step)."""
        v = np.zeros(1, dtype=np.int64)
        check(lib().pg_ti_get_step(self.h, _p(v)))
        return int(v[0])

    def ti_lambda_reduce(self):
        _, _, nl = self._ti
        m = np.zeros(nl)
        v = np.zeros(nl)
        c = np.zeros(nl, dtype=np.int64)
        check(lib().pg_ti_lambda_reduce(self.h, _p(m), _p(v), _p(c)))
        return m, v, c

    def ti_step(self):
        s = np.zeros(1, dtype=np.int64)
        check(lib().pg_ti_get_step(self.h, _p(s)))
        return int(s[0])

    def ti_form(self, nsteps=1):
        """(resolved PG_FORM_*, kernel launches per pg_ti_advance(nsteps))."""
        f = np.zeros(1, dtype=np.int32)
        n = np.zeros(1, dtype=np.int64)
        check(lib().pg_ti_get_form(self.h, nsteps, _p(f), _p(n)))
        return int(f[0]), int(n[0])

    def set_tuning(self, cache_path, mode):
        """Autotuning of AUTO batches: mode PG_TUNE_OFF / PG_TUNE_CACHE / PG_TUNE_ON,
        records in the JSON-lines file cache_path."""
        check(lib().pg_set_tuning(self.h, None if cache_path is None else str(cache_path).encode(), int(mode)))

    def ti_tuning(self):
        """(form, SIMT threads per ring, MD steps per tensor-step launch) of the batch; 0 = built-in."""
        v = np.zeros(3, dtype=np.int32)
        check(lib().pg_ti_get_tuning(self.h, _p(v[0:1]), _p(v[1:2]), _p(v[2:3])))
        return int(v[0]), int(v[1]), int(v[2])

    def ti_kernel_times(self, nsteps):
        """[(name, mean ms per launch, launches, algorithmic bytes per launch)] over nsteps steps."""
        nk = C.c_int32()
        ms = np.zeros(4)
        cnt = np.zeros(4, dtype=np.int64)
        by = np.zeros(4)
        names = (C.c_char_p * 4)()
        check(lib().pg_ti_kernel_times(self.h, nsteps, C.byref(nk), _p(ms), _p(cnt), _p(by), names))
        return [(names[i].decode(), float(ms[i]), int(cnt[i]), float(by[i])) for i in range(nk.value)]

    def ti_checkpoint_save(self, path):
        check(lib().pg_ti_checkpoint_save(self.h, path.encode()))

    def ti_checkpoint_load(self, path):
        check(lib().pg_ti_checkpoint_load(self.h, path.encode()))

    def ti_release(self):
        check(lib().pg_ti_release(self.h))

    def propagate_pimd(self, cfg, nmc, a, b, dbdl, seed, stream, x, p, inplace=False):
        """A batch of propagate_pimd_pile / _nm calls.  inplace=True updates the
        caller's contiguous float64 x and p (the reference's inout arrays, and
        what the C-ABI does; pinned arrays then copy at full speed); otherwise
        copies are returned."""
        a, b, dbdl = map(_f64, (a, b, dbdl))
        if inplace:
            if not (isinstance(x, np.ndarray) and isinstance(p, np.ndarray) and x.dtype == np.float64
                    and p.dtype == np.float64 and x.flags.c_contiguous and p.flags.c_contiguous):
                raise ValueError("inplace=True needs contiguous float64 arrays")
        else:
            x = np.array(x, dtype=np.float64)
            p = np.array(p, dtype=np.float64)
        nt = b.size // self.ndof
        sd = np.ascontiguousarray(seed, dtype=np.uint64)
        stv = np.ascontiguousarray(stream, dtype=np.uint32)
        dh = np.zeros(nt)
        st = np.zeros(nt, dtype=np.int32)
        check(lib().pg_propagate_pimd(self.h, C.byref(cfg), nt, nmc, _p(a), _p(b), _p(dbdl), _p(sd),
                                      _p(stv), _p(x), _p(p), _p(dh), _p(st)))
        return x, p, dh, st

    # ---- instanton
    def fp32_peak(self):
        """Measured FP32 FMA throughput of this GPU, TFLOP/s (pg_fp32_peak)."""
        v = C.c_double(0.0)
        check(lib().pg_fp32_peak(self.h, C.byref(v)))
        return v.value

    def set_wait_limit(self, ns):
        """Wall-time bound (ns) of the tensor-core transform's device waits
        (pg_set_wait_limit); 2e9 by default."""
        check(lib().pg_set_wait_limit(self.h, int(ns)))

    def set_fixedends(self, fixedends):
        """instantonmod's fixedends: False drops the end-point springs of the
        action and its gradient (pg_set_fixedends)."""
        check(lib().pg_set_fixedends(self.h, int(bool(fixedends))))

    def instanton_fg(self, N, x, a, b, betan):
        x, betan = _f64(x), _f64(np.atleast_1d(betan))
        a = None if a is None else _f64(a)
        b = None if b is None else _f64(np.atleast_1d(b))
        nb = betan.size
        UM = np.zeros(nb)
        g = np.zeros(x.size)
        check(lib().pg_instanton_fg(self.h, nb, N, _p(x), _p(a), _p(b), _p(betan), _p(UM), _p(g)))
        return UM, g

    def instanton_optimize(self, N, x, a, b, betan, m=8, factr=1.0e6, pgtol=1.0e-5, maxiter=20000,
                           max_backtracks=40, cluster_ctas=0):
        x = np.array(x, dtype=np.float64)
        betan = _f64(np.atleast_1d(betan))
        a = None if a is None else _f64(a)
        b = None if b is None else _f64(np.atleast_1d(b))
        nb = betan.size
        o = LbfgsOpts(m, max_backtracks, maxiter, factr, pgtol, cluster_ctas, 0)
        UM = np.zeros(nb)
        it = np.zeros(nb, dtype=np.int64)
        st = np.zeros(nb, dtype=np.int32)
        check(lib().pg_instanton_optimize(self.h, nb, N, _p(x), _p(a), _p(b), _p(betan), C.byref(o),
                                          _p(UM), _p(it), _p(st)))
        return x, UM, it, st

    def um_hessian(self, N, betan, x, singlewell=False, quirks=False):
        x = _f64(x)
        nd = self.ndof
        band = np.zeros((nd + 1) * N * nd)
        check(lib().pg_um_hessian(self.h, N, betan, _p(x), int(singlewell), int(quirks), _p(band)))
        return band.reshape(nd + 1, N * nd, order="F")

    def instanton_logdet(self, N, x, betan, singlewell=False, skip_lowest=True, quirks=False):
        x, betan = _f64(x), _f64(np.atleast_1d(betan))
        nb = betan.size
        ld = np.zeros(nb)
        emin = np.zeros(nb)
        nsk = np.zeros(nb, dtype=np.int64)
        check(lib().pg_instanton_logdet(self.h, nb, N, _p(x), _p(betan), int(singlewell),
                                        int(skip_lowest), int(quirks), _p(ld), _p(emin), _p(nsk)))
        return ld, emin, nsk
