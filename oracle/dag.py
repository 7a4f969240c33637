"""ORACLE -- test infrastructure only: numpy restatement of the DAG
max-flow solver's full-flow iteration, maxflow/asetsDAGMF2D.m and
asetsDAGMF3D.m (MaxFullFlow: the top-down node list, InitializeFullFlow,
UpdateSpatialFlows, PushDownFlows, PushCapacityUp, UpdateLabels), in the
precision of Ct and in Matlab's evaluation order, to check the GPU solver
(asetsmatlabmaxflow_gb300/csrc/hmf.cu).  The geodesic branch (direction
fields lx, ly, lz; asetsDAGMF2D.m:275-318, asetsDAGMF3D.m:281-331) shares
the restatement of oracle/hmf.py, whose conventions it follows.
"""
from __future__ import annotations

import numpy as np

from . import hmf as H


class Node:
    lx = ly = lz = None
    dirs = H.Node.dirs
    _normalize_dirs = H.Node._normalize_dirs

    def __init__(self, children, alpha, Ct=None):
        self.C = list(children)
        self.P = []
        for c in self.C:
            c.P.append(self)
        if not self.C:
            self.Ct = np.asarray(Ct)
            self.D = self.Ct.shape
        else:
            self.D = self.C[0].D
            self.Ct = np.zeros(0, self.C[0].Ct.dtype)
        self.alpha = alpha
        self.dt = self.Ct.dtype
        self.wC = None
        self.pn = None

    def par(self):
        """P{1}.pt or pn as the node's incoming flow."""
        return self.pn if len(self.P) > 1 else self.P[0].pt

    # --- InitializeFullFlow (asetsDAGMF2D.m / 3D)
    def init(self):
        if self.wC is None:
            self.wC = [1.0 / len(c.P) for c in self.C]
        for c in self.C:
            c.init()
        D, dt = self.D, self.dt
        self.g = np.zeros(D, dt)
        if len(self.C) > 1:
            pt = np.zeros(D, dt)
            for _ in self.C:
                x = self.C[0].pt
                pt = np.where((pt >= x) | np.isnan(pt), pt, x).astype(dt)
            self.pt = pt
        elif len(self.C) == 0:
            self.pt = self.Ct.copy()
        else:
            raise ValueError("an inner node needs two or more children")
        if len(self.P) > 1:
            self.pn = self.pt.copy() if len(D) == 2 else np.zeros(D, dt)
        self.div = np.zeros(D, dt)
        self.u = np.zeros(D, dt)
        self.p = [np.zeros(D[:k] + (D[k] - 1,) + D[k + 1:], dt) for k in range(len(D))]
        self._normalize_dirs()

    def max_full_flow(self, its, steps, cc):
        self.init()
        S, td = [self], []
        while S:
            q = S.pop()
            td.append(q)
            for r in q.C:
                if all(any(s is t for t in td) for s in r.P):
                    S.append(r)
        bu = td[::-1]
        for _ in range(its):
            for n in td:
                n.spatial(steps, cc)
                if n.pn is not None:
                    n.pn = np.zeros(n.D, n.dt)
            for n in td:
                n.push_down(cc)
            for n in bu:
                n.push_up(cc)
            for n in td:
                n.labels(cc)
        return td

    def labels(self, cc):
        if self.P:
            self.u = self.u + self.dt.type(cc) * ((self.par() - self.div) - self.pt)

    def push_down(self, cc):
        t = self.dt.type
        for i, c in enumerate(self.C):
            if len(c.P) > 1:
                c.pn = c.pn + t(self.wC[i]) * self.pt
        if self.P and self.C:
            self.g = (self.par() - self.div) + self.u / t(cc)
        elif not self.P:
            self.g = np.full(self.D, t(1 / cc), self.dt)

    def push_up(self, cc):
        t = self.dt.type
        if not self.C:
            x = (self.par() - self.div) + self.u / t(cc)
            self.pt = np.where((self.Ct <= x) | np.isnan(self.Ct), self.Ct, x).astype(self.dt)
            return
        g = self.g
        for i, c in enumerate(self.C):
            w = t(self.wC[i])
            if len(c.P) > 1:
                g = g + w * ((((c.div + c.pt) + w * self.pt) - c.pn) - c.u / t(cc))
            else:
                g = ((g + c.div) + c.pt) - c.u / t(cc)
        self.g = g
        s = 0.0
        for w in self.wC:
            s += w ** 2
        self.pt = (g / t(s if not self.P else 1 + s)).astype(self.dt)

    def spatial(self, steps, cc):
        if not self.P:
            return
        t = self.dt.type
        D, nd = self.D, len(self.D)
        g = t(steps) * (((self.div + self.pt) - self.par()) - self.u / t(cc))
        for k in range(nd):
            hi = np.take(g, range(1, D[k]), axis=k)
            lo = np.take(g, range(0, D[k] - 1), axis=k)
            self.p[k] = (self.p[k] + hi) - lo
        ls = self.dirs()
        e = None
        if ls is not None:
            self.p, e, _ = H.exemption(self.p, ls, D, self.dt)
        self.p, self.g, self.div = H.project(self.p, self.alpha, D, self.dt, e)
