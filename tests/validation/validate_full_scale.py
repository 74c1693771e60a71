"""Full-scale validation runs (GPU + CPU oracle); writes a JSON summary.

Not collected by pytest (long).  Run on a GB300:
    python tests/validation/validate_full_scale.py [--out results.json] [--parts c0,c1,c2,c3,c4]

  c0: mcmod_1d, P=32, 11 lambda points, 20000 steps: the GPU plain (reference
      step order) and fused FP64 forms against the CPU restatement.
  c1: mcmod_2dtest, P=128, 1024 x 16 rings, 50000 steps: mixed precision
      (tcgen05) against FP64 (fused), same seeds: splitting error.
  c2: 9-atom surface, P=256, 256 x 12 rings: FP32 SIMT against FP64 (short run).
  c3: instanton, N=512, 32 beta: GPU L-BFGS + log-det; at two beta values the
      CPU oracle (scipy L-BFGS-B on the C action, dsbevd on the C band).
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
for p in (os.path.join(ROOT, "pimd-tunneling_gb300", "python"), os.path.join(ROOT, "pimd-tunneling_gb300"),
          os.path.join(ROOT, "oracle")):
    sys.path.insert(0, p)

import build as B  # noqa: E402


def part_c0(out):
    import drivers
    import oracle as O
    import pgconfigs
    import pimdgpu as pg
    c = pgconfigs.load("c0")
    res = {}
    for name, form in (("gpu_plain_fp64", pg.PG_FORM_PLAIN), ("gpu_fused_fp64", pg.PG_FORM_FUSED)):
        res[name] = drivers.run_ti(c, precision=pg.PG_FP64, form=form)
    # CPU restatement of the reference step on the same rings and seeds
    ti = pgconfigs.TiInputs(c, gauleg=O.gauleg)
    pes = O.Pes(c["pes_id"], c["ndim"], c["natom"], c["params"], V0=c["V0"])
    mass = np.array(c["mass"])
    prm = O.TiParams(ti.P, c["beta"], c["dt"], tau=c["tau"], gamma=c["gamma"], thermostat=2, nm_resident=False,
                     imin=c["imin"], init_sigma=c["init_sigma"])
    nd, P = ti.nd, ti.P
    x = np.zeros(ti.nrings * nd * P)
    p = np.zeros(ti.nrings * nd * P)
    for r in range(ti.nrings):
        li = ti.ring_lambda[r]
        xx, pp = O.ring_init(pes, mass, prm, ti.xref[li], int(ti.ring_seed[r]), int(ti.ring_stream[r]),
                             a=ti.a, b=ti.b[li])
        x[r * nd * P:(r + 1) * nd * P] = xx
        p[r * nd * P:(r + 1) * nd * P] = pp
    t0 = time.perf_counter()
    rr = O.ti_run_batch(pes, mass, prm, ti.ring_lambda, ti.ring_seed, ti.ring_stream, ti.a, ti.b, ti.dbdl, ti.xref,
                        c["nmc"], os.cpu_count(), x, p)
    dt = time.perf_counter() - t0
    integ = np.array([rr[i].dhdr_sum / rr[i].nsamples / ti.betan ** 2 for i in range(ti.nrings)])
    dA, sA, q = O.ti_assemble(ti.w, integ, 1, ti.betan)
    res["cpu_oracle_reference_order"] = dict(dA=dA, qratio=q, ln_qratio=-dA * ti.betan, wall_s=dt,
                                             integrand_mean=list(integ))
    out["c0"] = res


def part_c1(out):
    import drivers
    import pgconfigs
    import pimdgpu as pg
    c = pgconfigs.load("c1")
    mixed = drivers.run_ti(c, precision=pg.PG_MIXED, form=pg.PG_FORM_AUTO, chunk=5000)
    fp64 = drivers.run_ti(c, precision=pg.PG_FP64, form=pg.PG_FORM_FUSED, chunk=2500)
    rel = abs(mixed["delta"] - fp64["delta"]) / abs(fp64["delta"]) if fp64["delta"] == fp64["delta"] else None
    out["c1"] = dict(mixed=mixed, fp64=fp64, splitting_rel_err_mixed_vs_fp64=rel,
                     ln_qratio_diff=mixed["ln_qratio"] - fp64["ln_qratio"],
                     ln_qratio_stderr=fp64["ln_qratio_stderr"])


def part_c2(out, nmc=2000):
    import drivers
    import pgconfigs
    import pimdgpu as pg
    c = pgconfigs.load("c2")
    mixed = drivers.run_ti(c, precision=pg.PG_MIXED, form=pg.PG_FORM_AUTO, nmc=nmc, chunk=500)
    simt = drivers.run_ti(c, precision=pg.PG_MIXED, form=pg.PG_FORM_FUSED, nmc=nmc, chunk=500)
    fp64 = drivers.run_ti(c, precision=pg.PG_FP64, form=pg.PG_FORM_FUSED, nmc=nmc, chunk=250)
    out["c2"] = dict(mixed=mixed, mixed_simt=simt, fp64=fp64, ln_qratio_diff=mixed["ln_qratio"] - fp64["ln_qratio"],
                     ln_qratio_diff_simt=simt["ln_qratio"] - fp64["ln_qratio"],
                     ln_qratio_stderr=fp64["ln_qratio_stderr"])


def part_c4(out, nmc=None):
    """18-atom surface, 4096 rings with P in {64, 128, 256, 512}: one context
    per P, advanced together; mixed precision on the tensor-core form (AUTO) and
    on the SIMT form."""
    import drivers
    import pgconfigs
    import pimdgpu as pg
    c = pgconfigs.load("c4")
    mixed = drivers.run_ti_mixed(c, precision=pg.PG_MIXED, nmc=nmc, chunk=500)
    simt = drivers.run_ti_mixed(c, precision=pg.PG_MIXED, form=pg.PG_FORM_FUSED, nmc=nmc, chunk=500)
    # FP64 on a shorter run (GB300's FP64 rate), against mixed precision on the same steps
    short = min(int(nmc if nmc is not None else c["nmc"]), 1000)
    fp64 = drivers.run_ti_mixed(c, precision=pg.PG_FP64, nmc=short, chunk=250)
    mixed_short = drivers.run_ti_mixed(c, precision=pg.PG_MIXED, nmc=short, chunk=500)
    diff = [m["ln_qratio"] - f["ln_qratio"] for m, f in zip(mixed_short["per_P"], fp64["per_P"])]
    out["c4"] = dict(mixed=mixed, mixed_simt=simt, fp64_short=fp64, mixed_short=mixed_short,
                     ln_qratio_diff_mixed_minus_fp64_short=diff)


def part_c3(out, factr=1e2, pgtol=1e-8):
    import drivers
    import oracle as O
    import pgconfigs
    import pimdgpu as pg
    c = pgconfigs.load("c3")
    r = drivers.run_rpi(c, m=10, factr=factr, pgtol=pgtol)
    res = dict(gpu=[{k: v for k, v in d.items()} for d in r["results"]], optimize_s=r["optimize_s"],
               logdet_s=r["logdet_s"], N=r["N"], factr=factr, pgtol=pgtol)
    pes = O.Pes(c["pes_id"], c["ndim"], c["natom"], c["params"], V0=c["V0"])
    mass = np.array(c["mass"])
    w1, w2 = np.array(c["well1"]), np.array(c["well2"])
    N = r["N"]
    checks = []
    with pg.Context(0) as ctx:
        ctx.set_system(c["ndim"], c["natom"], c["mass"], c["pes_id"], c["params"], c["V0"])
        for k in (0, len(c["betas"]) - 1):
            betan = c["betas"][k] / N
            x0 = drivers.linear_guess(w1, w2, N)
            t0 = time.perf_counter()
            xo, fo, rr = O.instanton_lbfgs(pes, mass, N, betan, x0, w1, w2, m=10, factr=factr, pgtol=pgtol)
            t_opt = time.perf_counter() - t0
            t0 = time.perf_counter()
            band = O.UMhessian(pes, mass, N, betan, xo)
            ld, nneg, w0 = O.logdet_band(band, True)
            bandh = O.UMhessian(pes, mass, N, betan, np.repeat(w1, N), singlewell=True)
            ld0, _, _ = O.logdet_band(bandh, False)
            t_det = time.perf_counter() - t0
            # GPU log-det on the CPU optimiser's geometry: the log-det error alone
            ldg, emg, _ = ctx.instanton_logdet(N, xo, [betan], singlewell=False, skip_lowest=True)
            g = res["gpu"][k]
            checks.append(dict(beta_index=k, UM_gpu=g["UM"], UM_cpu=fo, UM_rel_err=abs(g["UM"] - fo) / abs(fo),
                               S_gpu=g["S"], lndetJ_gpu=g["lndetJ"], lndetJ_cpu=ld,
                               lndetJ_gpu_on_cpu_geometry=float(ldg[0]),
                               lndetJ_rel_err_same_geometry=abs(float(ldg[0]) - ld) / abs(ld),
                               eta2_min_cpu=w0, eta2_min_gpu_same_geometry=float(emg[0]),
                               lndetJ0_gpu=g["lndetJ0"], lndetJ0_cpu=ld0,
                               lndetJ0_rel_err=abs(g["lndetJ0"] - ld0) / abs(ld0), cpu_optimize_s=t_opt,
                               cpu_logdet_s=t_det, cpu_iterations=int(rr.nit), gpu_iterations=g["iterations"]))
    res["cpu_checks"] = checks
    out["c3"] = res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default="validation.json")
    ap.add_argument("--parts", default="c0,c1,c2,c3")
    args = ap.parse_args()
    B.build()
    out = {}
    for part in args.parts.split(","):
        t0 = time.perf_counter()
        globals()["part_" + part](out)
        out.setdefault("timing_s", {})[part] = time.perf_counter() - t0
        with open(args.out, "w") as f:
            json.dump(out, f, indent=1, default=float)
        print(part, "done in %.1f s" % out["timing_s"][part], flush=True)


if __name__ == "__main__":
    main()
