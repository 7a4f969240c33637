"""ORACLE -- test infrastructure only: numpy restatement of the
hierarchical max-flow solver's full-flow iteration, maxflow/asetsHMF2D.m
and asetsHMF3D.m (MaxFullFlow: InitializeFullFlow, UpdateSinkFlows,
UpdateLabels, UpdateSpatialFlows, CalculateCostsFullFlow), in the precision
of Ct (float32 or float64) and in Matlab's evaluation order, to check the
GPU solver (asetsmatlabmaxflow_gb300/csrc/hmf.cu).  The anisotropic lx/ly
branch and MaxPseudoFlow are not restated.
"""
from __future__ import annotations

import numpy as np


class Node:
    def __init__(self, children, alpha, Ct=None):
        self.C = list(children)
        self.P = None
        for c in self.C:
            c.P = self
        if not self.C:
            self.Ct = np.asarray(Ct)
            self.D = self.Ct.shape
        else:
            self.D = self.C[0].D
            self.Ct = np.zeros(0, self.C[0].Ct.dtype)
        self.alpha = alpha
        self.dt = self.Ct.dtype

    # --- asetsHMF*D.m InitializeFullFlow
    def init(self):
        for c in self.C:
            c.init()
        D, dt = self.D, self.dt
        self.g = np.zeros(D, dt)
        self.pt = np.zeros(D, dt)
        self.u = np.zeros(D, dt)
        self.div = np.zeros(D, dt)
        self.p = [np.zeros(D[:k] + (D[k] - 1,) + D[k + 1:], dt) for k in range(len(D))]

    def max_full_flow(self, its, steps, cc):
        self.init()
        for _ in range(its):
            self.sink(cc)
            self.labels(cc)
            self.spatial(steps, cc)
        self.costs()

    # --- UpdateSinkFlows (children first)
    def sink(self, cc):
        for c in self.C:
            c.sink(cc)
        t = self.dt.type
        ccT = t(cc)
        if not self.C:
            x = (self.P.pt - self.div) + self.u / ccT
            self.pt = np.where((self.Ct <= x) | np.isnan(self.Ct), self.Ct, x).astype(self.dt)
            return
        if self.P is None:
            pt = np.full(self.D, t(1 / cc), self.dt)      # 1/cc .* ones(h.D)
        else:
            pt = (self.P.pt - self.div) + self.u / ccT
        for c in self.C:
            pt = ((pt + c.pt) + c.div) - c.u / ccT
        n = len(self.C) if self.P is None else 1 + len(self.C)
        self.pt = (pt / t(n)).astype(self.dt)

    # --- UpdateLabels
    def labels(self, cc):
        if self.P is not None:
            self.u = self.u + self.dt.type(cc) * ((self.P.pt - self.div) - self.pt)
        for c in self.C:
            c.labels(cc)

    # --- UpdateSpatialFlows (isotropic branch)
    def spatial(self, steps, cc):
        if self.P is not None:
            t = self.dt.type
            D, nd = self.D, len(self.D)
            g = t(steps) * (((self.div + self.pt) - self.P.pt) - self.u / t(cc))
            for k in range(nd):
                hi = np.take(g, range(1, D[k]), axis=k)
                lo = np.take(g, range(0, D[k] - 1), axis=k)
                if nd == 2:
                    self.p[k] = self.p[k] + (hi - lo)   # asetsHMF2D.m: px + (g(2:) - g(1:))
                else:
                    self.p[k] = (self.p[k] + hi) - lo   # asetsHMF3D.m: px + g(2:) - g(1:)
            m = np.zeros(D, self.dt)
            for k in range(nd):
                sq = self.p[k] * self.p[k]
                lo_sl = [slice(None)] * nd
                hi_sl = [slice(None)] * nd
                lo_sl[k] = slice(0, D[k] - 1)           # cells with a face above
                hi_sl[k] = slice(1, D[k])               # cells with a face below
                m[tuple(lo_sl)] = m[tuple(lo_sl)] + sq
                m[tuple(hi_sl)] = m[tuple(hi_sl)] + sq
            m = np.sqrt(m)
            al = self.alpha if np.ndim(self.alpha) == 0 else np.asarray(self.alpha, self.dt)
            with np.errstate(divide="ignore", invalid="ignore"):
                alm = np.broadcast_to(np.asarray(al, self.dt), D)
                gm = np.where(m <= alm, t(1), alm / m).astype(self.dt)
            for k in range(nd):
                hi = np.take(gm, range(1, D[k]), axis=k)
                lo = np.take(gm, range(0, D[k] - 1), axis=k)
                self.p[k] = (t(0.5) * self.p[k]) * (hi + lo)
            self.g = gm
            dv = np.zeros(D, self.dt)
            for k in range(nd):
                lo_sl = [slice(None)] * nd
                hi_sl = [slice(None)] * nd
                lo_sl[k] = slice(0, D[k] - 1)
                hi_sl[k] = slice(1, D[k])
                if k == 0:
                    dv[tuple(lo_sl)] = self.p[0]
                    dv[tuple(hi_sl)] = dv[tuple(hi_sl)] - self.p[0]
                else:
                    dv[tuple(lo_sl)] = dv[tuple(lo_sl)] + self.p[k]
                    dv[tuple(hi_sl)] = dv[tuple(hi_sl)] - self.p[k]
            self.div = dv
        for c in self.C:
            c.spatial(steps, cc)

    # --- CalculateCostsFullFlow
    def costs(self):
        self.dataCost = float(np.sum(self.u.astype(np.float64) * self.Ct)) if not self.C else 0.0
        self.reguCost = float(np.sum(self.u.astype(np.float64) * self.div)) if self.P is not None else 0.0
        for c in self.C:
            c.costs()
            self.dataCost += c.dataCost
            self.reguCost += c.reguCost


def preorder(root):
    out = [root]
    for c in root.C:
        out += preorder(c)
    return out
