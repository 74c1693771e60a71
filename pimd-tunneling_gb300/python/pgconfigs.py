"""Load the benchmark configurations (configs/c*.json) and build TI inputs.

A TI batch follows pimd_par.f90: fixed start a = well 1, end points b(xi) on the
(straight-line) path at the Gauss-Legendre nodes xi_i, db/dxi, and nrep
replicas per node; ring r = i*nrep + j (pimd_par.f90:245-255).  Replica j uses
RNG key seed j and stream id i.
"""
import json
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
CONFIG_DIR = os.path.join(os.path.dirname(_HERE), "configs")


def load(name):
    with open(os.path.join(CONFIG_DIR, name + ".json")) as f:
        return json.load(f)


class TiInputs:
    """Arrays for pg_ti_setup for one configuration."""

    def __init__(self, cfg, nrep=None, nintegral=None, P=None, init="well", gauleg=None):
        self.cfg = cfg
        self.ndim, self.natom = cfg["ndim"], cfg["natom"]
        nd = self.ndim * self.natom
        self.nd = nd
        self.P = int(P if P is not None else cfg["P"])
        self.nrep = int(nrep if nrep is not None else cfg.get("nrep", 1))
        self.nint = int(nintegral if nintegral is not None else cfg["nintegral"])
        if gauleg is None:
            x, w = np.polynomial.legendre.leggauss(self.nint)
            self.xi, self.w = 0.5 * (x + 1.0), 0.5 * w
        else:
            self.xi, self.w = gauleg(0.0, 1.0, self.nint)
        w1 = np.asarray(cfg["well1"], dtype=float)
        w2 = np.asarray(cfg["well2"], dtype=float)
        self.a = w1.copy()
        self.b = np.array([w1 + t * (w2 - w1) for t in self.xi])
        self.dbdl = np.array([w2 - w1 for _ in self.xi])
        P = self.P
        if init == "well":
            # all beads at well 1 (plus init_sigma noise, drawn on the device)
            self.xref = np.array([np.repeat(w1, P) for _ in self.xi])
        else:
            # beads on the path, xi_eff = (k-1) xi/(P-1) (verletmodule.f90:40-48)
            xr = []
            for t in self.xi:
                k = np.arange(P)
                xe = k * t / (P - 1)
                xr.append(np.concatenate([w1[d] + xe * (w2[d] - w1[d]) for d in range(nd)]))
            self.xref = np.array(xr)
        nr = self.nint * self.nrep
        self.ring_lambda = np.repeat(np.arange(self.nint, dtype=np.int32), self.nrep)
        seeds = list(cfg.get("seeds", []))
        if len(seeds) < self.nrep:  # one key per replica: the base seed + j, as the namelist driver does
            seeds = [(seeds[0] if seeds else 0) + j for j in range(self.nrep)]
        self.ring_seed = np.array([seeds[j % len(seeds)] for _ in range(self.nint) for j in range(self.nrep)],
                                  dtype=np.uint64)
        self.ring_stream = self.ring_lambda.astype(np.uint32)
        self.nrings = nr
        P_ = self.P
        self.betan = cfg["beta"] / (P_ + 1)

    def ti_config(self, pimdgpu, precision, form=None, nmc=None):
        c = self.cfg
        t = pimdgpu.TiConfig()
        t.nbeads = self.P
        t.beta = c["beta"]
        t.dt = c["dt"]
        t.tau = c.get("tau", 1.0)
        t.gamma = c["gamma"]
        t.thermostat = c.get("thermostat", 2)
        t.precision = precision
        t.form = pimdgpu.PG_FORM_AUTO if form is None else form
        t.cayley = int(bool(c.get("cayley", False)))
        t.imin = c.get("imin", 0)
        t.noutput = c.get("noutput", 100000)
        t.dhdr_limit = c.get("dhdr_limit", -1.0)
        t.init_sigma = c.get("init_sigma", 0.0)
        return t
