"""TI-PIMD and RPI drivers over the C-ABI (the pimd_par.f90 / rpi_ser.f90 flow).

run_ti   -- Gauss-Legendre points on the straight path between the wells, nrep
            replicas per point, one batched propagation of every ring, the
            per-point mean / variance of dHdr/betan^2 on the device, then
            dA = sum w_i I_i, sigma_A^2 = sum w_i^2 var_i, q/q0 = exp(-dA betan)
            (pimd_par.f90:212-221, 379-424) and Delta = (2/beta) artanh(q/q0).
run_ti_mixed -- a task list whose rings have different bead numbers P (one
            context per P, all advanced together by pg_ti_advance_group on
            concurrent streams); TI is assembled per P, since betan = beta/(P+1)
            and the estimate itself depend on P.
run_rpi  -- rpi_ser.f90:133-190, 222-237, 354-381 for a batch of beta values:
            linear-interpolation or path.xyz spline guess (path=frames),
            instanton by on-device L-BFGS (V0 moved
            to the lowest bead when one lies below well 1), log-det at
            the wells (single well, all eigenvalues) and at the instanton
            (lowest eigenvalue dropped), S = betan UM, Omega and Delta.
run_rpi_angular -- rpi_ser.f90:241-348: the solid-angle grid for one beta.
crossover_beta -- crossover.f90:49-71: beta_c of a transition state.
multiwell_levels -- python_utils/multiwell_waterdimer.py: splittings per
            irreducible representation from path ratios at two temperatures.
Every number is computed by libpimdgpu on the GPU; this module only sequences
the calls and assembles the scalars.
"""
import time

import numpy as np

import pgconfigs
import pimdgpu as pg


def set_system_at_well1(ctx, c):
    """Select the surface with V0 = V(well1) evaluated by the library in FP64,
    as both reference drivers set it (pimd_par.f90:166, rpi_ser.f90:95) and the
    namelist drivers do: every front end then hands the device the same energy
    zero, so the L-BFGS objective (and its stopping test) is bit-identical."""
    ctx.set_system(c["ndim"], c["natom"], c["mass"], c["pes_id"], c["params"], 0.0)
    v0 = float(ctx.pes_eval(np.asarray(c["well1"], float).reshape(1, -1))[0][0])
    ctx.set_system(c["ndim"], c["natom"], c["mass"], c["pes_id"], c["params"], v0)
    return v0


def _lambda_stderr2(w, var, cnt):
    """sum_i w_i^2 var_i / n_i over the rings each lambda point kept (the
    reference's sigmaA / nrep when every ring counts, pimd_par.f90:422); a point
    whose rings were all left out (NaN-flagged or without samples) has no
    estimate, and the run stops instead of integrating a zero."""
    cnt = np.asarray(cnt)
    if np.any(cnt <= 0):
        raise RuntimeError("integration point(s) %s have no valid ring (all NaN-flagged or without samples)"
                           % (np.nonzero(cnt <= 0)[0] + 1).tolist())
    return float(np.sum(np.asarray(w) ** 2 * np.asarray(var) / cnt))


def readhess_displacements(band, P, ndim, natom, mass, beta, z):
    """Bead displacements of init_path with readhess (verletmodule.f90:49-88).

    band: the (nd + 1) x (P nd) lower band of the polymer Hessian at the path
    beads (pg_um_hessian, singlewell false), whose full eigendecomposition is
    what detJ(x, etasquared, .false., interphess, eigvecs) returns
    (instantonmod.f90:782-827; the interpolated Hessian it is passed is not used).
    z: (nrep, P nd) standard normals, scaled here by sqrt(1/beta) (tempx).
    Every mode but the lowest with eta^2 > 0 displaces the beads by
    sqrt(1 / (eta^2 m_k)) tempx eigvec, reading the eigenvector component of
    bead i, dimension j, atom k at natom (j + ndim i) + k as the reference does
    (verletmodule.f90:75-83; for several atoms this differs from the Hessian's
    atom-major dof order, reference behaviour).  eta^2 = 0 is skipped (the
    reference divides by it).  Returns (nrep, nd P) in the ring layout
    dx[(k ndim + j) P + i]."""
    nd = ndim * natom
    n = P * nd
    band = np.asarray(band, dtype=float).reshape(nd + 1, n)
    H = np.zeros((n, n))
    for r in range(nd + 1):
        i = np.arange(n - r)
        H[i + r, i] = band[r, :n - r]
        H[i, i + r] = band[r, :n - r]
    w, v = np.linalg.eigh(H)
    sel = np.arange(n) >= 1
    sel &= w > 0.0
    z = np.atleast_2d(np.asarray(z, dtype=float)) * np.sqrt(1.0 / beta)
    u = (z[:, sel] / np.sqrt(w[sel])) @ v[:, sel].T  # (nrep, n): components in the eigenvector index
    bead = np.arange(P)
    dx = np.zeros((z.shape[0], n))
    for j in range(ndim):
        for k in range(natom):
            dx[:, (k * ndim + j) * P + bead] = u[:, bead * nd + j * natom + k] / np.sqrt(mass[k])
    return dx


def readhess_start(ctx, c, ti, quirks=False):
    """Start positions of every ring: the path at the ring's lambda point plus
    the readhess displacements, one eigendecomposition per lambda point and
    normals from each ring's own seed (numpy's Philox; the reference draws them
    with MKL VSL)."""
    nd, P = ti.nd, ti.P
    x0 = np.zeros((ti.nrings, nd * P))
    for lam in range(ti.nint):
        rings = np.nonzero(np.asarray(ti.ring_lambda) == lam)[0]
        if rings.size == 0:
            continue
        band = ctx.um_hessian(P, ti.betan, ti.xref[lam], singlewell=False, quirks=quirks)
        z = np.stack([np.random.Generator(np.random.Philox(key=int(ti.ring_seed[r]),
                                                           counter=[int(ti.ring_stream[r]), 49, 0, 0]))
                      .standard_normal(nd * P) for r in rings])
        x0[rings] = ti.xref[lam][None, :] + readhess_displacements(band, P, c["ndim"], c["natom"], c["mass"],
                                                                   c["beta"], z)
    return x0.ravel()


def _arc_length(frames):
    lam = np.concatenate([[0.0], np.cumsum(np.linalg.norm(np.diff(frames, axis=0), axis=1))])
    return lam / lam[-1]


def _bisect_top(dv, x1=0.3, x2=0.7, xacc=1.0e-6, jmax=40):
    """findmiddle (instantonmod.f90:832-871): bisection for the zero of dV/dlambda."""
    f1, f2 = dv(x1), dv(x2)
    if f1 * f2 >= 0.0:
        raise ValueError("centre: the barrier top is not bracketed in (%g, %g)" % (x1, x2))
    xm, dx = (x1, x2 - x1) if f1 < 0.0 else (x2, x1 - x2)
    for _ in range(jmax):
        dx *= 0.5
        xmid = xm + dx
        fm = dv(xmid)
        if fm <= 0.0:
            xm = xmid
        if abs(dx) < xacc or fm == 0.0:
            break
    return xm


def ti_path_inputs(ctx, c, ti, frames, instapath=False, centre=False, init="path", fixedends=True):
    """The read_path flow of pimd_par (instantonmod.f90:895-1004, pimd_par.f90:212-221)
    for the batch ti (modified in place): the frames of path.xyz (3-D frames
    aligned by the first frame's angles) splined against normalised arc length;
    with instapath the instanton of that path guess (n = P beads at
    (k-1)/(n-1), the driver's betan) replaces it: optimised with fixed ends at
    the wells as [well 1, beads, well 2], or free-ended (fixedends False) as the
    beads alone (instantonmod.f90:952-970); with centre the arc length is remapped so that the
    barrier top of V along the path sits at 1/2.  Then a = path(0), b_i =
    path(xi_i), dbdl_i = path'(xi_i) and the start beads at
    xi_eff = (k-1) xi_i / (P-1) (init 'path', verletmodule.f90:40-48) or at
    well 1 ('well').  Returns the centring's barrier top (or None)."""
    import align
    nd, P = ti.nd, ti.P
    w1, w2 = np.asarray(c["well1"], float), np.asarray(c["well2"], float)
    fr = [np.asarray(f, dtype=float) for f in frames]
    if align.supported(c["ndim"], c["natom"]):
        fr = align.align_frames(fr)
    fr = np.array(fr)
    lam = _arc_length(fr)

    def splines(lam, fr):
        return [pg.spline(lam, fr[:, d]) for d in range(nd)]

    if instapath:
        y2 = splines(lam, fr)
        t = np.arange(P) / (P - 1)
        xt = np.concatenate([[pg.splint(lam, fr[:, d], y2[d], v)[0] for v in t] for d in range(nd)])
        ctx.set_fixedends(fixedends)
        try:
            x, _, _, _ = ctx.instanton_optimize(P, xt, w1 if fixedends else None, w2 if fixedends else None,
                                                [ti.betan], m=8, factr=1.0e6, pgtol=1.0e-5, maxiter=200000)
        finally:
            ctx.set_fixedends(True)
        beads = np.asarray(x).reshape(nd, P).T
        fr = np.vstack([w1, beads, w2]) if fixedends else beads
        lam = _arc_length(fr)
    xm = None
    if centre:
        V = ctx.pes_eval(fr)[0]
        v2 = pg.spline(lam, V)
        xm = _bisect_top(lambda l: pg.splint(lam, V, v2, l)[1])
        ca, cb = 2.0 - 4.0 * xm, 4.0 * xm - 1.0  # instantonmod.f90:993-1004
        lam = 2.0 * lam / (cb + np.sqrt(cb * cb + 4.0 * ca * lam))
    y2 = splines(lam, fr)

    def at(v, d):
        return pg.splint(lam, fr[:, d], y2[d], v)

    ti.a = np.array([at(0.0, d)[0] for d in range(nd)])
    ti.b = np.array([[at(x, d)[0] for d in range(nd)] for x in ti.xi])
    ti.dbdl = np.array([[at(x, d)[1] for d in range(nd)] for x in ti.xi])
    if init == "path":
        ti.xref = np.array([np.concatenate([[at(k * x / (P - 1), d)[0] for k in range(P)] for d in range(nd)])
                            for x in ti.xi])
    else:
        ti.xref = np.array([np.repeat(w1, P) for _ in ti.xi])
    return xm


def restart_name(r, ntask, nproc=1):
    """restart_proc<iproc>_<ii>.xyz of task r: nproc contiguous blocks of
    ceil(ntask / nproc) tasks (pimd_par.f90:109-110, 352)."""
    ncalcs = -(-ntask // nproc)
    return "restart_proc%d_%d.xyz" % (r // ncalcs, r % ncalcs + 1)


def write_restart_files(ctx, c, labels=None, nproc=1, directory="."):
    """write_restart (verletmodule.f90:162-185) for every ring of the batch on
    ctx: per bead natom, the running dHdr sum, label x y z; then per bead natom,
    the step count, label px py pz (coordinates beyond ndim written as 0), in
    the files of restart_name."""
    import os
    ndim, natom = c["ndim"], c["natom"]
    labels = labels or ["X"] * natom
    x, p = ctx.ti_state()
    dsum = ctx.ti_results()[0]
    step = ctx.ti_step()
    nr = dsum.size
    P = x.size // (nr * ndim * natom)
    x = x.reshape(nr, natom, ndim, P)
    p = p.reshape(nr, natom, ndim, P)
    for r in range(nr):
        with open(os.path.join(directory, restart_name(r, nr, nproc)), "w") as f:
            for v, head in ((x[r], "%.17g" % dsum[r]), (p[r], "%d" % step)):
                for i in range(P):
                    f.write(" %d\n %s\n" % (natom, head))
                    for j in range(natom):
                        f.write(" %s %s\n" % (labels[j], " ".join("%.17g" % (v[j, d, i] if d < ndim else 0.0)
                                                                for d in range(3))))


def read_restart_files(c, nrings, P, nproc=1, directory="."):
    """The files of write_restart_files back: (x0, p0, dhdr_sum, step) in the ring
    layout x[r][(atom ndim + dim) P + bead]; the files must agree on the step."""
    import os
    ndim, natom = c["ndim"], c["natom"]
    x0 = np.zeros((nrings, natom, ndim, P))
    p0 = np.zeros((nrings, natom, ndim, P))
    dsum = np.zeros(nrings)
    steps = set()
    for r in range(nrings):
        name = restart_name(r, nrings, nproc)
        with open(os.path.join(directory, name)) as f:
            tok = f.read().split()
        k = 0
        try:
            for dest in (x0, p0):
                for i in range(P):
                    if int(tok[k]) != natom:
                        raise ValueError("natom mismatch")
                    head = tok[k + 1]
                    k += 2
                    if dest is x0:
                        dsum[r] = float(head)
                    else:
                        steps.add(int(head))
                    for j in range(natom):
                        vals = [float(v) for v in tok[k + 1:k + 4]]
                        if len(vals) != 3:
                            raise ValueError("short file")
                        dest[r, j, :, i] = vals[:ndim]
                        k += 4
        except (IndexError, ValueError) as e:
            raise ValueError("cannot read restart file %s (%s)" % (name, e)) from None
    if len(steps) != 1:
        raise ValueError("restart files disagree on the step count")
    return x0.reshape(nrings, -1), p0.reshape(nrings, -1), dsum, steps.pop()


def run_ti(cfg, precision=pg.PG_MIXED, form=pg.PG_FORM_AUTO, nmc=None, nrep=None, nintegral=None,
           seed_offset=0, chunk=2000, device=0, ctx=None, verbose=False, tune=None, readhess=False,
           frames=None, instapath=False, centre=False, init="well", restart=0, nproc=1, labels=None,
           directory=".", fixedends=True):
    c = dict(cfg)
    if nrep is not None:
        c["nrep"] = nrep
    nrep = c.get("nrep", 1)
    c["seeds"] = [seed_offset + s for s in range(nrep)] if "seeds" not in cfg or seed_offset else c["seeds"]
    ti = pgconfigs.TiInputs(c, nrep=nrep, nintegral=nintegral, gauleg=pg.gauleg, init=init)
    nmc = int(nmc if nmc is not None else c["nmc"])
    own = ctx is None
    if own:
        ctx = pg.Context(device)
    try:
        set_system_at_well1(ctx, c)
        if frames is not None or instapath or centre:  # path.xyz / instanton / centring
            ti_path_inputs(ctx, c, ti, frames if frames is not None else [c["well1"], c["well2"]],
                           instapath=instapath, centre=centre, init=init, fixedends=fixedends)
        tcfg = ti.ti_config(pg, precision, form)
        if tune:  # autotuner cache (AUTO form): tuned on the first batch of each shape
            ctx.set_tuning(tune, pg.PG_TUNE_ON)
        p0 = None
        if restart == 2:  # continue from the restart files, nmc further steps (pimd_par.f90:356-369)
            x0, p0, dsum, step0 = read_restart_files(c, ti.nrings, ti.P, nproc, directory)
        else:
            x0 = readhess_start(ctx, c, ti) if readhess else None
        ctx.ti_setup(tcfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref, x0=x0, p0=p0)
        done = 0
        if restart == 2:
            ctx.ti_set_accumulators(dsum, np.full(ti.nrings, max(0, step0 - int(c.get("imin", 0)))), step0)
            done = step0
        start, target = done, done + nmc
        # restart files every Noutput steps past imin (verletmodule.f90:389-395), as the namelist
        # driver writes them: the state before step ii of this run, labelled with its step count
        noutput = int(c.get("noutput", 100000))
        next_ii = max(noutput, int(c.get("imin", 0)) + 1) if restart >= 1 and noutput > 0 else None
        form_used, _ = ctx.ti_form(1)
        t0 = time.perf_counter()
        dev_ms = 0.0
        while done < target:
            at = start + next_ii - 1 if next_ii is not None else target
            n = min(chunk, min(target, at) - done)
            if n > 0:
                dev_ms += ctx.ti_advance_timed(n)
                done += n
                if verbose:
                    print("  %d / %d steps" % (done, target), flush=True)
            if next_ii is not None and done == at and done < target:
                write_restart_files(ctx, c, labels, nproc, directory)
                next_ii += noutput
        wall = time.perf_counter() - t0
        if restart >= 1:
            write_restart_files(ctx, c, labels, nproc, directory)
        mean, var, cnt = ctx.ti_lambda_reduce()
        _, _, _, status = ctx.ti_results()
    finally:
        if own:
            ctx.close()
    se2 = _lambda_stderr2(ti.w, var, cnt)
    dA, sigA, q = pg.ti_assemble(ti.w, mean, var, ti.betan)
    try:
        delta = pg.splitting_from_ratio(c["beta"], q)
    except pg.PgError:
        delta = float("nan")
    lnq = -dA * ti.betan
    lnq_err = ti.betan * np.sqrt(max(se2, 0.0))
    beads = ti.nrings * ti.P
    return dict(dA=dA, sigmaA=sigA, qratio=q, ln_qratio=lnq, ln_qratio_stderr=lnq_err, delta=delta,
                integrand_mean=list(mean), integrand_var=list(var), nrings=ti.nrings, P=ti.P, nmc=nmc,
                nrep=nrep, nintegral=ti.nint, betan=ti.betan, form=form_used, device_s=dev_ms / 1e3,
                wall_s=wall, bead_steps_per_s=beads * nmc / (dev_ms / 1e3), nan_rings=int(np.sum(status != 0)))


def run_ti_mixed(cfg, precision=pg.PG_MIXED, form=pg.PG_FORM_AUTO, nmc=None, chunk=1000, device=0,
                 verbose=False):
    """Rings r = i*nrep + j (lambda point i, replica j) with bead number
    cfg["P_per_ring"][r]; the time step of a group is cfg["dt_per_P"][P] when
    given.  Returns per-P TI results and the throughput of the whole batch."""
    c = dict(cfg)
    Pr = np.asarray(c["P_per_ring"], dtype=np.int64)
    nint = int(c["nintegral"])
    if len(Pr) % nint:
        raise ValueError("P_per_ring length is not a multiple of nintegral")
    nrep = len(Pr) // nint
    nmc = int(nmc if nmc is not None else c["nmc"])
    groups = []
    try:
        for P in sorted(set(int(v) for v in Pr)):
            idx = np.nonzero(Pr == P)[0]
            cg = dict(c, P=P)
            if "dt_per_P" in c:
                cg["dt"] = c["dt_per_P"][str(P)]
            ti = pgconfigs.TiInputs(cg, nrep=nrep, nintegral=nint, P=P, gauleg=pg.gauleg)
            ctx = pg.Context(device)
            groups.append((P, idx, ti, ctx))
            set_system_at_well1(ctx, c)
            ctx.ti_setup(ti.ti_config(pg, precision, form), ti.ring_lambda[idx], ti.ring_seed[idx],
                         ti.ring_stream[idx], ti.a, ti.b, ti.dbdl, ti.xref)
        t0 = time.perf_counter()
        dev_ms = 0.0
        done = 0
        ctxs = [g[3] for g in groups]
        while done < nmc:
            n = min(chunk, nmc - done)
            dev_ms += pg.Context.ti_advance_group(ctxs, n)
            done += n
            if verbose:
                print("  %d / %d steps" % (done, nmc), flush=True)
        wall = time.perf_counter() - t0
        per_P = []
        beads = 0
        for P, idx, ti, ctx in groups:
            mean, var, cnt = ctx.ti_lambda_reduce()
            _, _, _, status = ctx.ti_results()
            form_used, _ = ctx.ti_form(1)
            se2 = _lambda_stderr2(ti.w, var, cnt)
            dA, sigA, q = pg.ti_assemble(ti.w, mean, var, ti.betan)
            try:
                delta = pg.splitting_from_ratio(c["beta"], q)
            except pg.PgError:
                delta = float("nan")
            per_P.append(dict(P=P, nrings=int(len(idx)), dA=dA, sigmaA=sigA, qratio=q, ln_qratio=-dA * ti.betan,
                              ln_qratio_stderr=ti.betan * np.sqrt(max(se2, 0.0)), delta=delta,
                              betan=ti.betan, dt=ti.cfg["dt"], form=form_used,
                              nan_rings=int(np.sum(status != 0))))
            beads += len(idx) * P
    finally:
        for g in groups:
            g[3].close()
    return dict(per_P=per_P, nrings=int(len(Pr)), beads=int(beads), nmc=nmc, device_s=dev_ms / 1e3, wall_s=wall,
                bead_steps_per_s=beads * nmc / (dev_ms / 1e3))


def crossover_beta(ctx, ts, mass, quirks=False):
    """crossover.f90:49-71 for the system set on ctx (mass: per atom): the Hessian at the
    transition state ts from the library, the ascending eigenvalues eta^2 of its
    mass-weighted form (every atom pair; the reference's second atom loop stops
    at ndim, crossover.f90:56) and beta_c = 2 pi / sqrt(-eta^2_min), with the
    reference's pi.  Returns (beta_c, eta2); beta_c is NaN when no eigenvalue
    is negative."""
    ts = np.ascontiguousarray(ts, dtype=float)
    H = ctx.pes_hessian(ts, quirks=quirks)[0]
    s = 1.0 / np.sqrt(np.repeat(np.asarray(mass, float), ctx.ndim))
    eta2 = np.linalg.eigvalsh(H * s[:, None] * s[None, :])
    beta_c = 2.0 * 3.14159265358979 / np.sqrt(-eta2[0]) if eta2[0] < 0.0 else float("nan")
    return float(beta_c), eta2


def multiwell_levels(chars, rho1, rho2, beta1, beta2):
    """python_utils/multiwell_waterdimer.py:65-84: per irreducible
    representation (rows of chars, columns the operations g), the level-pair
    ratios I at two inverse temperatures from the path ratios rho_g (rho of
    the identity = 1), then Delta = 2 (artanh I2 - artanh I1) / (beta2 - beta1)
    in Hartree (the script prints 219475 Delta, cm^-1) and the offset beta_bar.
    Returns (delta, betabar, I1, I2)."""
    I1, I2 = pg.irrep_ratios(chars, rho1), pg.irrep_ratios(chars, rho2)
    out = [pg.splitting_two_beta(beta1, a, beta2, b) for a, b in zip(I1, I2)]
    return np.array([d for d, _ in out]), np.array([b for _, b in out]), I1, I2


def path_guess(frames, N, ndim=None, natom=None, atoms=(1, 2, 3)):
    """Start path from the frames of path.xyz (read_path, instantonmod.f90:916-950;
    rpi_ser.f90:133-146): three-dimensional frames aligned by the angles of the
    first (instantonmod.f90:926-932), normalised arc length between frames, a
    natural cubic spline per dof and N beads at (k-1)/(N-1).  frames: (npath, nd)
    arrays x[atom*ndim + dim]; returns the path x[dof*N + bead]."""
    import align
    fr = [np.asarray(f, dtype=float) for f in frames]
    if ndim is not None and natom is not None and align.supported(ndim, natom, atoms):
        fr = align.align_frames(fr, atoms)
    fr = np.array(fr)
    lam = np.concatenate([[0.0], np.cumsum(np.linalg.norm(np.diff(fr, axis=0), axis=1))])
    lam /= lam[-1]
    t = np.arange(N) / (N - 1)
    out = []
    for d in range(fr.shape[1]):
        y2 = pg.spline(lam, fr[:, d])
        out.append([pg.splint(lam, fr[:, d], y2, v)[0] for v in t])
    return np.concatenate(out)


def linear_guess(w1, w2, N):
    """rpi_ser.f90:157-163."""
    k = np.arange(1, N + 1)
    return np.concatenate([((N - k) * w1[d] + (k - 1) * w2[d]) / (N - 1) for d in range(len(w1))])


def run_rpi(cfg, N=None, betas=None, m=8, factr=1.0e6, pgtol=1.0e-5, maxiter=200000, quirks=False,
            device=0, ctx=None, fixedends=True, path=None):
    c = dict(cfg)
    N = int(N if N is not None else c["N"])
    betas = np.asarray(betas if betas is not None else c["betas"], dtype=float)
    nb = len(betas)
    betan = betas / N  # rpi_ser.f90:45
    w1, w2 = np.asarray(c["well1"], float), np.asarray(c["well2"], float)
    nd = len(w1)
    own = ctx is None
    if own:
        ctx = pg.Context(device)
    try:
        set_system_at_well1(ctx, c)
        guess = (linear_guess(w1, w2, N) if path is None
                 else path_guess(path, N, c["ndim"], c["natom"]))  # rpi_ser.f90:133-163
        x0 = np.concatenate([guess for _ in range(nb)])
        t0 = time.perf_counter()
        # fixedends False: the free-ended action, optimised without the end
        # points (instanton(xtilde), instantonmod.f90:724-762)
        ctx.set_fixedends(fixedends)
        try:
            x, UM, it, st = ctx.instanton_optimize(N, x0, w1 if fixedends else None,
                                                   np.tile(w2, nb) if fixedends else None, betan, m=m,
                                                   factr=factr, pgtol=pgtol, maxiter=maxiter)
        finally:
            ctx.set_fixedends(True)
        t_opt = time.perf_counter() - t0
        # V along each instanton: a bead below well 1 moves V0 to its energy,
        # which raises the action by -N min V (rpi_ser.f90:180-190)
        beads = np.asarray(x).reshape(nb, nd, N).transpose(0, 2, 1).reshape(nb * N, nd)
        vpath = ctx.pes_eval(beads)[0].reshape(nb, N)
        vshift = np.minimum(vpath.min(axis=1), 0.0)
        # S = betan UM(xtilde[, well1, well2]) (rpi_ser.f90:370-374): the action
        # as it was optimised, with or without the end springs
        UM = np.asarray(UM) - N * vshift
        xharm = np.concatenate([np.repeat(w1, N) for _ in range(nb)])
        t0 = time.perf_counter()
        ld0, _, _ = ctx.instanton_logdet(N, xharm, betan, singlewell=True, skip_lowest=False, quirks=quirks)
        ld, emin, nsk = ctx.instanton_logdet(N, x, betan, singlewell=False, skip_lowest=True, quirks=quirks)
        t_det = time.perf_counter() - t0
    finally:
        if own:
            ctx.close()
    out = []
    for k in range(nb):
        S, om, de = pg.rpi_assemble(betan[k], UM[k], ld[k], ld0[k])
        out.append(dict(beta=float(betas[k]), betan=float(betan[k]), UM=float(UM[k]), S=S, omega=om, delta=de,
                        lndetJ=float(ld[k]), lndetJ0=float(ld0[k]), eta2_min=float(emin[k]),
                        skipped=int(nsk[k]), iterations=int(it[k]), status=int(st[k])))
    return dict(N=N, results=out, x=x, vpath=vpath, optimize_s=t_opt, logdet_s=t_det)


def _rotate(w, ndim, axis, theta):
    """rotate_atoms (instantonmod.f90:346-376) on x[atom*ndim + dim]; in 2-D the
    rotation in the plane (axis 3)."""
    import align
    if ndim == 3:
        return align.rotate_atoms(np.asarray(w, float).reshape(-1, 3), axis, theta).ravel()
    if abs(theta) <= 1.0e-10:
        return np.asarray(w, float)
    v = np.asarray(w, float).reshape(-1, 2)
    c, s = np.cos(theta), np.sin(theta)
    return np.stack([c * v[:, 0] + s * v[:, 1], -s * v[:, 0] + c * v[:, 1]], axis=1).ravel()


def run_rpi_angular(cfg, N, beta, npoints, cutofftheta=2.0 * 3.14159265358979, cutoffphi=3.14159265358979,
                    m=8, factr=1.0e6, pgtol=1.0e-5, maxiter=200000, quirks=False, device=0, ctx=None, path=None):
    """The solid-angle grid of rpi_ser.f90:241-348 for one beta, as the namelist
    driver runs it: the instanton of run_rpi, then well 2 turned by
    R_x(theta) R_z(phi) R_x(eta) at Gauss-Legendre angles (3-D; in 2-D by eta in
    the plane), every orientation re-optimised from that instanton in one batched
    call, log-dets with the lowest eigenvalue left out, and per orientation
    I = tanh(Omega N) (3-D: 1 when Omega N > 1).  Returns the rows of
    angularI.dat: (theta, phi, eta, weight, I) in 3-D, (eta, weight, I) in 2-D."""
    c = dict(cfg)
    ndim = c["ndim"]
    if ndim not in (2, 3):
        raise ValueError("the angular grid needs ndim = 2 or 3")
    own = ctx is None
    if own:
        ctx = pg.Context(device)
    try:
        base = run_rpi(c, N=N, betas=[beta], m=m, factr=factr, pgtol=pgtol, maxiter=maxiter, quirks=quirks,
                       ctx=ctx, path=path)
        ld0 = base["results"][0]["lndetJ0"]
        vshift = min(float(np.min(base["vpath"])), 0.0)
        betan = beta / N
        w1, w2 = np.asarray(c["well1"], float), np.asarray(c["well2"], float)
        et, wet = pg.gauleg(0.0, min(2.0 * 3.14159265358979, cutofftheta), npoints)
        rows, ends = [], []
        if ndim == 3:
            th, wth = et, wet
            ph, wph = pg.gauleg(0.0, min(3.14159265358979, cutoffphi), npoints)
            for ii in range(npoints):
                for jj in range(npoints):
                    for kk in range(npoints):
                        w = _rotate(_rotate(_rotate(w2, 3, 1, et[kk]), 3, 3, ph[jj]), 3, 1, th[ii])
                        ends.append(w)
                        rows.append([th[ii], ph[jj], et[kk], wth[ii] * wph[jj] * wet[kk]])
        else:
            for kk in range(npoints):
                ends.append(_rotate(w2, 2, 3, et[kk]))
                rows.append([et[kk], wet[kk]])
        nb = len(ends)
        xs = np.tile(np.asarray(base["x"], float), nb)
        bn = np.full(nb, betan)
        xs, UM, _, _ = ctx.instanton_optimize(N, xs, w1, np.concatenate(ends), bn, m=m, factr=factr, pgtol=pgtol,
                                              maxiter=maxiter)
        ld, _, _ = ctx.instanton_logdet(N, xs, bn, singlewell=False, skip_lowest=True, quirks=quirks)
    finally:
        if own:
            ctx.close()
    out = []
    for q in range(nb):
        _, om, _ = pg.rpi_assemble(betan, UM[q] - N * vshift, ld[q], ld0)
        ib = np.tanh(om * N)
        if ndim == 3 and om * N > 1.0:
            ib = 1.0
        out.append(rows[q] + [float(ib)])
    return np.array(out)
