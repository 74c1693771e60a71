#!/usr/bin/env python
"""Throughput benchmark: bead-force-steps/s of batched TI-PIMD on one GB300.

Workload (one GPU): the 2-D six-well surface of mcmod_2dtest, P = 128 beads,
1024 trajectories x 16 Gauss-Legendre lambda points = 16,384 ring polymers,
Langevin thermostat, mixed precision (FP32 forces and state, split-BF16
tensor-core normal-mode transform, FP64 estimator accumulation).  One bench
"step" = MD_PER_STEP MD steps of every ring (one launch of the fused kernel).

  value   = (sum over rings of P) * MD steps / device seconds, all ranks
  e2e     = the same metric through pg_propagate_pimd (the reference-facing
            drop-in for propagate_pimd_pile) with host x/p buffers: H2D of the
            ring state, the MD steps, D2H of state and estimators, every step
  plain / fused FP64: the same rings through the FP64 forms (denominators)
  split_check: ln q/q0 and the splitting of the benchmarked mixed-precision
            batch against the FP64 form (itself parity-tested against the CPU
            oracle) on the same rings, seeds and number of MD steps
  roofline: compute-bound terms of the dominant kernel (tensor: the two NM
            transforms; SIMT: surface, operand splitting, update, normals;
            HBM: ncu DRAM bytes), the kernel timed inside the replayed advance
  instanton_c3 / uneven_p_c4: the instanton batch (32 beta, N = 512) and the
            uneven-P batch (4,096 rings, P in {64..512}) timed through the API
  cpu_baseline: the CPU restatement of the reference step (ten dense NM
            transforms per step, FP64) on all host cores, bounded sample

--impl reference times only that CPU restatement (the reference's own
Fortran/MKL/MPI build cannot be compiled on these machines).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "pimd-tunneling_gb300")
for _p in (os.path.join(PKG, "python"), PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "bead-force-steps/s, batched mixed-prec vs plain FP64 on 1 GB300 at <=1% split err"
UNIT = "bead-force-steps/s"
MD_PER_STEP = 500


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _workload(rank, name="c1"):
    import pgconfigs
    c = dict(pgconfigs.load(name))
    # weak scaling: every rank runs its own trajectories (distinct seeds)
    nrep = int(c.get("nrep", 1))
    c["seeds"] = [s + nrep * rank for s in range(nrep)]
    ti = pgconfigs.TiInputs(c)
    return c, ti


WORKLOADS = {
    "c1": "c1: mcmod_2dtest surface, P=128, 1024 traj x 16 lambda = 16384 rings per GPU",
    "c2": "c2: synthetic 9-atom surface (27 dof), P=256, 256 traj x 12 lambda = 3072 rings per GPU",
}


def _config(M, form, name="c1"):
    """The workload description shared by both arms."""
    return {"workload": WORKLOADS[name] + ", Langevin, %d MD steps per bench step" % M,
            "precision": "FP32 forces/state, split-BF16 NM transform, FP64 estimator",
            "l2": "flushed (256 MB write) between timed steps", "form": form}


def simt_flops_per_bead_step(c):
    """Algorithmic FP32 SIMT flops per bead-force-step of the mixed step kernels
    (MUFU exponentials count as one): the surface gradient per bead plus 28 per
    dof -- positions x = T q + x* (2), splitting the two BF16 operands (4), the
    kick / rotation / OU map of (q, pi) (16), the OU normal's Box-Muller share
    and scale (6).  Surface gradients: mcmod_2dtest 16 per well (offsets 2,
    u 3, two exponentials 4, coefficient 3, gradient 4); the 9-atom surface 30
    per Morse pair (distance, exponential, Morse value and its gradient through
    the B-matrix) for 36 pairs plus 20 for the quartic coordinate."""
    nd = c["ndim"] * c["natom"]
    pid = c["pes_id"]
    if pid == 2:
        fpes = 16.0 * c["params"][0]
    elif pid == 3:
        fpes = 30.0 * 36 + 20.0
    elif pid == 1:
        fpes = 8.0 * nd
    elif pid == 4:
        # 18-atom surface: per molecule two bonds and the angle with their
        # gradients (80); per site pair of different molecules the distance,
        # the Coulomb term and its gradient through the B-matrix (20), plus the
        # Lennard-Jones term of each O-O pair (15)
        nmol = int(c["params"][0])
        fpes = 80.0 * nmol + 20.0 * 9 * nmol * (nmol - 1) / 2 + 15.0 * nmol * (nmol - 1) / 2
    else:
        return None
    return fpes + 28.0 * nd


def roofline(ctx, pg, c, ti, beads, M, adv_ms, peaks, peak_kind, fp32_tflops):
    """The dominant kernel's place under its compute roofline.  Its time per
    launch inside the replayed advance is the advance time less the other
    kernels (timed alone) over its launches; achieved = algorithmic work per
    launch / that time, per term; the bound is the largest fraction."""
    kt = ctx.ti_kernel_times(M)  # per-kernel events, direct launches (advances the batch M steps)
    if not kt:
        return None
    try:
        with open(os.path.join(ROOT, "profiles", "tensor_kernels_traffic.json")) as f:
            tj = json.load(f)
    except Exception:
        tj = {}
    persistent = [i for i, t in enumerate(kt) if t[0].startswith(("k_tc_step", "k_tf_step ("))]
    if persistent:
        # a persistent step kernel does the whole MD step: it is the unit
        dom = persistent[0]
        name, kms_alone, kcount, kbytes = kt[dom]
        minor = sum(m * n for i, (_, m, n, _) in enumerate(kt) if i != dom)
        kms = (adv_ms - minor) / max(kcount, 1)
        traffic = tj.get(name.split()[0])
        per_md = tj.get(name.split()[0] + "_per_md_step")  # traffic that scales with the MD steps of a launch
        if traffic is None and per_md is not None:
            traffic = per_md * M / max(kcount, 1)
    else:
        # several kernels per MD step (blocked form): the MD step is the unit
        name = " + ".join(n.split()[0] for n, _, _, _ in kt) + " (one MD step)"
        kcount = M
        kms = adv_ms / M
        kms_alone = sum(m for _, m, _, _ in kt)
        kbytes = sum(b for _, _, _, b in kt)
        tr = [tj.get(n.split()[0]) for n, _, _, _ in kt]
        traffic = sum(tr) if all(t is not None for t in tr) else None
    md_per_launch = M / max(kcount, 1)  # MD steps one launch of the unit covers
    units = beads * md_per_launch        # bead-force-steps per launch
    secs = kms / 1e3
    terms = {}
    # tensor: two NM transforms per MD step (T q to positions, T F to modes), 2 P d flops per bead each
    tc_flops = 4.0 * ti.P * ti.nd * units
    terms["tensor"] = {"flops_per_bead_step": 4.0 * ti.P * ti.nd, "achieved": tc_flops / secs / 1e12,
                       "peak": peaks["bf16_tflops"], "unit": "TFLOP/s",
                       "peak_basis": "dense bf16 cuBLAS burst (%s)" % peak_kind}
    fs = simt_flops_per_bead_step(c)
    if fs is not None and fp32_tflops:
        terms["simt"] = {"flops_per_bead_step": fs, "achieved": fs * units / secs / 1e12, "peak": fp32_tflops,
                         "unit": "TFLOP/s", "peak_basis": "FP32 FMA chains measured live (pg_fp32_peak)"}
    if traffic:
        terms["hbm"] = {"bytes_per_launch": traffic, "achieved": traffic / secs / 1e9, "peak": peaks["hbm_gbs"],
                        "unit": "GB/s", "peak_basis": "STREAM copy (%s); bytes: ncu DRAM read + write of one "
                                                      "launch" % peak_kind}
    for t in terms.values():
        t["frac"] = t["achieved"] / t["peak"]
    bind = max(terms, key=lambda k: terms[k]["frac"])
    b = terms[bind]
    return {"bound": "compute", "binding_term": bind, "achieved": b["achieved"], "peak": b["peak"],
            "unit": b["unit"], "frac": b["frac"], "traffic": traffic, "peak_source": peak_kind,
            "kernel": name, "kernel_ms": kms, "kernel_ms_alone": kms_alone, "launches_per_bench_step": kcount,
            "bead_steps_per_launch": units, "algorithmic_bytes_per_launch": kbytes, "terms": terms,
            "kernels": [{"name": n, "ms_per_launch_alone": m, "launches_per_bench_step": k, "bytes_per_launch": by}
                        for (n, m, k, by) in kt]}


def split_check(ctx, pg, c, ti, nsteps, mixed, chunk=1000):
    """ln q/q0 and the splitting Delta = (2/beta) artanh(q/q0) of the mixed batch
    after nsteps MD steps (its per-lambda mean / var / count in mixed) against
    the FP64 fused form on the same rings, seeds and steps (pimd_par.f90:399-424)."""
    import drivers

    def assemble(mean, var, cnt):
        se2 = drivers._lambda_stderr2(ti.w, var, cnt)
        dA, _, q = pg.ti_assemble(ti.w, mean, var, ti.betan)
        try:
            delta = pg.splitting_from_ratio(c["beta"], q)
        except pg.PgError:
            delta = float("nan")
        return {"ln_qratio": -dA * ti.betan, "ln_qratio_stderr": ti.betan * float(np.sqrt(max(se2, 0.0))),
                "delta": delta}

    t0 = time.perf_counter()
    m = assemble(*mixed)
    cfg64 = ti.ti_config(pg, pg.PG_FP64, pg.PG_FORM_FUSED)
    ctx.ti_setup(cfg64, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
    done = 0
    while done < nsteps:
        k = min(chunk, nsteps - done)
        ctx.ti_advance(k)
        done += k
    r = assemble(*ctx.ti_lambda_reduce())
    _, _, _, st = ctx.ti_results()
    rel = abs(m["delta"] / r["delta"] - 1.0) if r["delta"] else float("nan")
    return {"md_steps": int(nsteps), "imin": int(ti.cfg["imin"]), "rings": int(ti.nrings), "mixed": m, "fp64": r,
            "delta_rel_err": rel, "ln_qratio_diff": m["ln_qratio"] - r["ln_qratio"], "within_1pct": bool(rel <= 0.01),
            "fp64_nan_rings": int(np.sum(st != 0)), "seconds": time.perf_counter() - t0,
            "fp64_form": "fused SIMT FP64 (parity-tested against the CPU oracle to 1e-9 per step)"}


def instanton_leg(pg, device):
    """The c3 instanton batch: 32 beta values, N = 512 beads of the 9-atom surface,
    one batched L-BFGS to pgtol 1e-8 from the rpi_ser linear path (thread-block
    clusters per polymer), then the log-determinants at the instantons."""
    import drivers
    import pgconfigs
    c = pgconfigs.load("c3")
    with pg.Context(device) as ctx:
        ctx.set_system(c["ndim"], c["natom"], c["mass"], c["pes_id"], c["params"], c["V0"])
        w1, w2 = np.array(c["well1"]), np.array(c["well2"])
        N, betas = c["N"], np.array(c["betas"])
        nb = len(betas)
        betan = betas / N
        x0 = np.tile(drivers.linear_guess(w1, w2, N), nb)
        t0 = time.perf_counter()
        x, UM, it, st = ctx.instanton_optimize(N, x0, w1, np.tile(w2, nb), betan, m=10, factr=1e2, pgtol=1e-8,
                                               maxiter=200000)
        t_opt = time.perf_counter() - t0
        t0 = time.perf_counter()
        ctx.instanton_logdet(N, x, betan, singlewell=False, skip_lowest=True)
        t_det = time.perf_counter() - t0
    return {"betas": nb, "N": N, "dofs": c["ndim"] * c["natom"], "optimize_s": t_opt, "logdet_s": t_det,
            "iterations_mean": float(np.mean(it)), "converged": int(np.sum(st == 0)),
            "note": "one batched L-BFGS, each polymer on a thread-block cluster; host-timed calls"}


def p256_leg(pg, device, peaks, peak_kind, fp32, M=100, K=3):
    """The c2 batch (3,072 rings of the 9-atom surface, P = 256) in the persistent
    folded step kernel: device time of K advances of M MD steps after one warm-up,
    L2 flushed before each, and its roofline terms."""
    import torch
    c, ti = _workload(0, "c2")
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    with pg.Context(device) as ctx:
        ctx.set_system(c["ndim"], c["natom"], c["mass"], c["pes_id"], c["params"], c["V0"])
        cfg = ti.ti_config(pg, pg.PG_MIXED, pg.PG_FORM_AUTO)
        ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
        ctx.ti_advance(M)
        dev_s = 0.0
        for _ in range(K):
            flush.add_(1.0)
            torch.cuda.synchronize()
            dev_s += ctx.ti_advance_timed(M) / 1e3
        form_used, launches = ctx.ti_form(M)
        roof = roofline(ctx, pg, c, ti, ti.nrings * ti.P, M, 1e3 * dev_s / K, peaks, peak_kind, fp32)
        _, _, _, st = ctx.ti_results()
    return {"value": ti.nrings * ti.P * M * K / dev_s, "unit": UNIT, "rings": ti.nrings, "P": ti.P,
            "md_steps": M * K, "device_s": dev_s, "launches_per_advance": launches, "roofline": roof,
            "nan_rings": int(np.sum(st != 0)),
            "note": "persistent folded step: T folded into two resident 128 x 128 halves, two warp groups per CTA"}


def uneven_p_leg(pg, peaks=None, fp32=None, nmc=200):
    """The c4 batch: 4,096 rings of the 18-atom surface with P in {64, 128, 256,
    512}, one context per P advanced together as one CUDA-graph launch; with
    the measured peaks, its roofline terms from algorithmic work per
    bead-force-step (the blocked form moves q and x (positions), x and F
    (forces), F, q, pi in and q, pi out (kick): 36 d bytes; two NM transforms
    of 2 P d flops each, P weighted by the beads of each bead number)."""
    import drivers
    import pgconfigs
    c = dict(pgconfigs.load("c4"), imin=0)
    r = drivers.run_ti_mixed(c, precision=pg.PG_MIXED, form=pg.PG_FORM_AUTO, nmc=nmc, chunk=nmc // 2)
    out = {"value": r["bead_steps_per_s"], "unit": UNIT, "rings": r["nrings"], "md_steps": nmc,
           "device_s": r["device_s"], "note": "pg_ti_advance_group: every P's step kernels in one graph launch"}
    if peaks:
        Pr = np.asarray(c["P_per_ring"], dtype=float)
        nd = c["ndim"] * c["natom"]
        rate = r["bead_steps_per_s"]
        p_eff = float(np.sum(Pr * Pr) / np.sum(Pr))  # bead-weighted P
        terms = {"tensor": {"flops_per_bead_step": 4.0 * p_eff * nd, "peak": peaks["bf16_tflops"],
                            "unit": "TFLOP/s"},
                 "hbm": {"bytes_per_bead_step": 36.0 * nd, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "basis": "algorithmic bytes (no capture of the group)"}}
        terms["tensor"]["achieved"] = terms["tensor"]["flops_per_bead_step"] * rate / 1e12
        terms["hbm"]["achieved"] = terms["hbm"]["bytes_per_bead_step"] * rate / 1e9
        fs = simt_flops_per_bead_step(c)
        if fs is not None and fp32:
            terms["simt"] = {"flops_per_bead_step": fs, "achieved": fs * rate / 1e12, "peak": fp32, "unit": "TFLOP/s"}
        for t in terms.values():
            t["frac"] = t["achieved"] / t["peak"]
        bind = max(terms, key=lambda k: terms[k]["frac"])
        out["roofline"] = {"binding_term": bind, "frac": terms[bind]["frac"], "p_bead_weighted": p_eff,
                           "terms": terms}
    return out


def cpu_reference_rate(c, ti, target_s=12.0, nthreads=None):
    """Bead-force-steps/s of the CPU restatement of the reference step on all host
    cores (one ring per thread at a time), on a bounded sample of the workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.lib()
    nthreads = nthreads or os.cpu_count() or 1
    pes = O.Pes(c["pes_id"], c["ndim"], c["natom"], c["params"], V0=c["V0"])
    mass = np.array(c["mass"])
    prm = O.TiParams(ti.P, c["beta"], c["dt"], tau=c["tau"], gamma=c["gamma"], thermostat=2,
                     nm_resident=False, imin=0, init_sigma=c["init_sigma"])
    nd, P = ti.nd, ti.P

    def run(nr, nsteps):
        idx = np.arange(nr) % ti.nrings
        lam = ti.ring_lambda[idx]
        x = np.zeros(nr * nd * P)
        p = np.zeros(nr * nd * P)
        for k, r in enumerate(idx):
            li = ti.ring_lambda[r]
            xx, pp = O.ring_init(pes, mass, prm, ti.xref[li], int(ti.ring_seed[r]), int(ti.ring_stream[r]),
                                 a=ti.a, b=ti.b[li])
            x[k * nd * P:(k + 1) * nd * P] = xx
            p[k * nd * P:(k + 1) * nd * P] = pp
        t0 = time.perf_counter()
        O.ti_run_batch(pes, mass, prm, lam, ti.ring_seed[idx], ti.ring_stream[idx], ti.a, ti.b, ti.dbdl,
                       ti.xref, nsteps, nthreads, x, p)
        return time.perf_counter() - t0

    nr = nthreads
    probe_steps = 20
    dt = run(nr, probe_steps)
    rate_ring_steps = nr * probe_steps / max(dt, 1e-9)
    nsteps = max(20, int(target_s * rate_ring_steps / nr))
    dt = run(nr, nsteps)
    value = nr * nsteps * P / dt
    sample = ("%d rings x %d MD steps of the workload (P=%d, %d dofs), reference step "
              "order (10 dense NM transforms per step), FP64, %d threads, %.1f s" % (nr, nsteps, P, nd, nthreads, dt))
    return value, nthreads, sample


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    c, ti = _workload(0, args.workload)
    vals = []
    for _ in range(max(args.warmup, 0)):
        cpu_reference_rate(c, ti, target_s=1.0)
    per = max(3.0, 20.0 / max(args.steps, 1))
    sample = ""
    cores = 1
    for _ in range(args.steps):
        v, cores, sample = cpu_reference_rate(c, ti, target_s=per)
        vals.append(v)
    value = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": _config(args.md_per_step, args.form, args.workload),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference Fortran/MKL/MPI build cannot be compiled here (no Fortran compiler, "
                    "no MKL); this arm times the CPU restatement of the reference step"}
    print(json.dumps(line), flush=True)
    return 0


def _extras(ctx, pg, cfg, ti, M, K, value, ws, beads, extras):
    import torch
    # e2e: the reference-facing drop-in with host buffers, copies inside the timed region
    x0, p0 = ctx.ti_state()
    xh = torch.from_numpy(x0).pin_memory().numpy()
    ph = torch.from_numpy(p0).pin_memory().numpy()
    bseq = ti.b
    dseq = ti.dbdl
    bl = np.ascontiguousarray(bseq[ti.ring_lambda])
    dl = np.ascontiguousarray(dseq[ti.ring_lambda])
    for _ in range(2):
        ctx.propagate_pimd(cfg, M, ti.a, bl, dl, ti.ring_seed, ti.ring_stream, xh, ph, inplace=True)
    te = []
    for _ in range(max(3, K // 2)):
        t0 = time.perf_counter()
        xo, po, dh, _ = ctx.propagate_pimd(cfg, M, ti.a, bl, dl, ti.ring_seed, ti.ring_stream, xh, ph,
                                           inplace=True)
        te.append(time.perf_counter() - t0)
    e2e_s = statistics.median(te)
    h2d = xh.nbytes + ph.nbytes
    d2h = xh.nbytes + ph.nbytes + dh.nbytes
    extras["e2e"] = {"value": beads * M / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                     "d2h_bytes_per_step": int(d2h), "call": "pg_propagate_pimd (host buffers)"}
    # FP64 denominators on the same rings
    for name, form64, md in (("plain_fp64", pg.PG_FORM_PLAIN, 20), ("fused_fp64", pg.PG_FORM_FUSED, 100)):
        cfg64 = ti.ti_config(pg, pg.PG_FP64, form64)
        ctx.ti_setup(cfg64, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
        ctx.ti_advance(md)
        ms = ctx.ti_advance_timed(md)
        extras[name] = {"value": beads * md / (ms / 1e3), "unit": UNIT, "md_steps": md}
    extras["speedup_vs_plain_fp64"] = value / ws / extras["plain_fp64"]["value"]
    extras["speedup_vs_fused_fp64"] = value / ws / extras["fused_fp64"]["value"]



def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--md-per-step", type=int, default=MD_PER_STEP)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-extras", action="store_true", help="skip the e2e and FP64 legs")
    ap.add_argument("--no-split-check", action="store_true",
                    help="skip the splitting check of the benchmarked batch against the FP64 form")
    ap.add_argument("--form", default="auto", choices=["auto", "fused", "tensor"])
    ap.add_argument("--workload", default="c1", choices=sorted(WORKLOADS),
                    help="c1 (the headline configuration) or c2 (27-dof surface, P = 256)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    ws, rank, local = _dist()
    import torch
    import torch.distributed as dist
    if ws > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)

    import build as B
    if rank == 0 or ws == 1:
        B.build()
    if ws > 1:
        dist.barrier()
    import pimdgpu as pg

    c, ti = _workload(rank, args.workload)
    ctx = pg.Context(local)
    ctx.set_system(c["ndim"], c["natom"], c["mass"], c["pes_id"], c["params"], c["V0"])
    form = {"auto": pg.PG_FORM_AUTO, "fused": pg.PG_FORM_FUSED, "tensor": pg.PG_FORM_TENSOR}[args.form]
    cfg = ti.ti_config(pg, pg.PG_MIXED, form)
    ctx.ti_setup(cfg, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref)
    K, W, M = args.steps, args.warmup, args.md_per_step
    beads = ti.nrings * ti.P
    form_used, launches_per_step = ctx.ti_form(M)

    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2
    for _ in range(W):
        ctx.ti_advance(M)
    sampler = ClockSampler(local)
    sampler.start()
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    times = []
    wall0 = time.perf_counter()
    for _ in range(K):
        flush.add_(1.0)  # evict L2 between timed steps
        torch.cuda.synchronize()
        times.append(ctx.ti_advance_timed(M) / 1e3)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    if ws > 1:
        dist.barrier()
    clocks = sampler.stop()
    dev_s = sum(times)
    if ws > 1:
        t = torch.tensor([dev_s], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_s = float(t.item())
    value = ws * beads * M * K / dev_s
    kernel_ms = 1e3 * dev_s / K
    s, n, _, st = ctx.ti_results()
    nan_rings = int(np.sum(st != 0))
    mixed_red = ctx.ti_lambda_reduce()  # the benchmarked batch, for the splitting check
    mixed_steps = ctx.ti_step()

    peaks, peak_kind = _peaks()
    print("[bench] timed advance: %.3f ms per step of %d MD steps, %.3e %s" % (kernel_ms, M, value, UNIT),
          file=sys.stderr, flush=True)
    roof = None
    extras = {}
    if rank == 0:
        try:
            fp32 = ctx.fp32_peak()
            # the dominant kernel, timed with CUDA events on the library stream
            roof = roofline(ctx, pg, c, ti, beads, M, kernel_ms, peaks, peak_kind, fp32)
            roof["fp32_peak_tflops_measured"] = fp32
        except Exception as e:
            extras["roofline_error"] = repr(e)
    try:
        if not args.no_split_check and rank == 0:
            extras["split_check"] = split_check(ctx, pg, c, ti, mixed_steps, mixed_red)
    except Exception as e:
        extras["split_check_error"] = repr(e)
    try:
        if not args.no_extras and rank == 0:
            _extras(ctx, pg, cfg, ti, M, K, value, ws, beads, extras)
    except Exception as e:  # report, keep the main measurement
        extras["extras_error"] = repr(e)
    if not args.no_extras and rank == 0:
        fp32 = roof["fp32_peak_tflops_measured"] if roof else None
        for key, leg in (("p256_c2", lambda: p256_leg(pg, local, peaks, peak_kind, fp32)),
                         ("instanton_c3", lambda: instanton_leg(pg, local)),
                         ("uneven_p_c4", lambda: uneven_p_leg(pg, peaks, fp32))):
            try:
                extras[key] = leg()
            except Exception as e:
                extras[key + "_error"] = repr(e)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": W,
            "ms_per_step": kernel_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": _config(M, args.form, args.workload),
            "roofline": roof, "clocks": clocks, "gpu_launches": K * launches_per_step, "wall_s": wall,
            "form": {pg.PG_FORM_FUSED: "fused-simt", pg.PG_FORM_TENSOR: "tcgen05", pg.PG_FORM_PLAIN: "plain"}[form_used],
            "nan_rings": nan_rings}
    line.update(extras)
    if rank == 0 and ws == 1 and not args.no_cpu:  # the CPU baseline: rank 0 at N = 1 only
        v, cores, sample = cpu_reference_rate(c, ti, target_s=12.0)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}
        v1, _, sample1 = cpu_reference_rate(c, ti, target_s=3.0, nthreads=1)
        line["cpu_baseline"]["single_core"] = {"value": v1, "sample": sample1}
    if "e2e" not in line:
        line["e2e"] = None
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if ws > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
