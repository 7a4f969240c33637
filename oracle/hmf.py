"""ORACLE -- test infrastructure only: numpy restatement of the
hierarchical max-flow solver's full-flow iteration, maxflow/asetsHMF2D.m
and asetsHMF3D.m (MaxFullFlow: InitializeFullFlow, UpdateSinkFlows,
UpdateLabels, UpdateSpatialFlows, CalculateCostsFullFlow), in the precision
of Ct (float32 or float64) and in Matlab's evaluation order, to check the
GPU solver (asetsmatlabmaxflow_gb300/csrc/hmf.cu).  Also restated: the
geodesic branch of the spatial-flow update (direction fields lx, ly, lz;
asetsHMF2D.m:228-261, asetsHMF3D.m:215-262) and MaxPseudoFlow
(asetsHMF2D.m:91-105, :340-470; asetsHMF3D.m:89-102, :339-470).

Conventions where Matlab leaves room: x.^0.5 is sqrt(x); max(x, 0) is x for
x > 0 and +0 otherwise (NaN gives 0, as Matlab's max ignores NaN); the
direction fields are taken in the class of Ct, and the 0.001 length
threshold is compared in that class.
"""
from __future__ import annotations

import numpy as np


def _lo_hi(D, k):
    nd = len(D)
    lo = tuple(slice(0, D[j] - 1) if j == k else slice(None) for j in range(nd))
    hi = tuple(slice(1, D[j]) if j == k else slice(None) for j in range(nd))
    return lo, hi


def normalize_dirs(ls, dt):
    """InitializeFullFlow / InitializePseudoFlow (asetsHMF2D.m:118-126):
    unit direction vectors, 0 where the length is at most 0.001."""
    t = dt.type
    s = ls[0] * ls[0]
    for l in ls[1:]:
        s = s + l * l
    den = np.sqrt(s)
    keep = den > t(0.001)
    with np.errstate(divide="ignore", invalid="ignore"):
        return [np.where(keep, l / den, t(0)).astype(dt) for l in ls]


def _pos(mask, v, l, dt):
    """max((mask).*v.*l, 0)."""
    x = (mask.astype(dt) * v) * l
    return np.where(x > 0, x, dt.type(0)).astype(dt)


def exemption(p, ls, D, dt):
    """The geodesic branch (asetsHMF2D.m:228-247): per cell the exemption
    amount a -- the flow leaving the cell along its direction, summed over
    its faces (first axis backward and forward, then each further axis
    forward and backward) -- and per face the exempt part e of the flow.
    Returns the flows less e, e, and a."""
    nd = len(D)
    a = np.zeros(D, dt)
    for k in range(nd):
        lo, hi = _lo_hi(D, k)
        pk, lk = p[k], ls[k]
        if k == 0:
            a[hi] = a[hi] + _pos(pk < 0, pk, lk[hi], dt)
            a[lo] = a[lo] + _pos(pk > 0, pk, lk[lo], dt)
        else:
            a[lo] = a[lo] + _pos(pk > 0, pk, lk[lo], dt)
            a[hi] = a[hi] + _pos(pk < 0, pk, lk[hi], dt)
    q, e = [], []
    for k in range(nd):
        lo, hi = _lo_hi(D, k)
        pk, lk = p[k], ls[k]
        ek = (((pk > 0) & (lk[lo] > 0)).astype(dt) * lk[lo]) * a[lo]
        ek = ek + (((pk < 0) & (lk[hi] < 0)).astype(dt) * lk[hi]) * a[hi]
        e.append(ek.astype(dt))
        q.append((pk - ek).astype(dt))
    return q, e, a


def project(p, alpha, D, dt, e=None):
    """Flow magnitude per cell, the factor min(1, alpha/|p|), and the rescale
    p = e + 0.5 p (g(k+1) + g(k)) (e = 0 without direction fields).
    Returns the flows, the factor and the divergence."""
    t = dt.type
    nd = len(D)
    m = np.zeros(D, dt)
    for k in range(nd):
        sq = p[k] * p[k]
        lo, hi = _lo_hi(D, k)
        m[lo] = m[lo] + sq
        m[hi] = m[hi] + sq
    m = np.sqrt(m)
    alm = np.broadcast_to(np.asarray(alpha, dt), D)
    with np.errstate(divide="ignore", invalid="ignore"):
        gm = np.where(m <= alm, t(1), alm / m).astype(dt)
    out = []
    for k in range(nd):
        lo, hi = _lo_hi(D, k)
        r = (t(0.5) * p[k]) * (gm[hi] + gm[lo])
        out.append((r if e is None else e[k] + r).astype(dt))
    dv = np.zeros(D, dt)
    for k in range(nd):
        lo, hi = _lo_hi(D, k)
        if k == 0:
            dv[lo] = out[0]
            dv[hi] = dv[hi] - out[0]
        else:
            dv[lo] = dv[lo] + out[k]
            dv[hi] = dv[hi] - out[k]
    return out, gm, dv


class Node:
    lx = ly = lz = None

    def dirs(self):
        """The direction fields, or None (numel(h.lx) == 0)."""
        if self.lx is None or np.size(self.lx) == 0:
            return None
        ls = [self.lx, self.ly, self.lz][:len(self.D)]
        if any(l is None or np.size(l) == 0 for l in ls):
            raise ValueError("lx given without ly (and lz in 3D)")
        return [np.asarray(l, self.dt).reshape(self.D) for l in ls]

    def _normalize_dirs(self):
        ls = self.dirs()
        if ls is not None:
            ls = normalize_dirs(ls, self.dt)
            self.lx, self.ly = ls[0], ls[1]
            if len(ls) == 3:
                self.lz = ls[2]

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
        self.u = np.zeros(self.D, self.dt)

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
        self._normalize_dirs()

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

    # --- UpdateSpatialFlows
    def spatial(self, steps, cc):
        if self.P is not None:
            t = self.dt.type
            g = t(steps) * (((self.div + self.pt) - self.P.pt) - self.u / t(cc))
            self._flows(g, paren=len(self.D) == 2)
        for c in self.C:
            c.spatial(steps, cc)

    def _flows(self, g, paren):
        """Gradient step on g, the geodesic exemption if the node has
        direction fields, projection and divergence."""
        D, nd = self.D, len(self.D)
        for k in range(nd):
            hi = np.take(g, range(1, D[k]), axis=k)
            lo = np.take(g, range(0, D[k] - 1), axis=k)
            if paren:
                self.p[k] = self.p[k] + (hi - lo)   # asetsHMF2D.m:222: px + (g(2:) - g(1:))
            else:
                self.p[k] = (self.p[k] + hi) - lo   # px + g(2:) - g(1:)
        ls = self.dirs()
        e = None
        if ls is not None:
            self.p, e, _ = exemption(self.p, ls, D, self.dt)
        al = self.alpha if np.ndim(self.alpha) == 0 else np.asarray(self.alpha, self.dt)
        self.p, self.g, self.div = project(self.p, al, D, self.dt, e)

    # --- MaxPseudoFlow
    def max_pseudo_flow(self, its, steps, cc):
        nodes = preorder(self)
        leaves = [n for n in nodes if not n.C]
        self.init_pseudo()
        t = self.dt.type
        for _ in range(its):
            for n in nodes:                      # ResetPseudoFlowCapacity
                n.g = (n.div + n.Ct) if not n.C else np.zeros(n.D, n.dt)
            for n in nodes:                      # PushDownPseudoFlows
                for c in n.C:
                    c.g = c.g + n.g
            self.g = np.zeros(self.D, self.dt)
            for n in leaves:                     # UpdatePseudoFlowLabels
                n.u = n.u * np.exp(-n.g / t(cc))
                n.g = n.u
                self.g = self.g + n.u
            with np.errstate(divide="ignore", invalid="ignore"):
                for n in leaves:                 # NormalizePseudoFlowLabels
                    u = n.u / self.g
                    u[u > 1] = 1
                    u[u < 0] = 0
                    n.u = u
            self.push_up()                       # PushUpCapacityReqs
            for n in nodes[1:]:                  # UpdateSpatialPseudoFlows
                n._flows(t(steps) * n.g, paren=False)
        self.deinit_pseudo()

    def init_pseudo(self):
        for c in self.C:
            c.init_pseudo()
        D, dt = self.D, self.dt
        self.g = np.zeros(D, dt)
        self.div = np.zeros(D, dt)
        self.p = [np.zeros(D[:k] + (D[k] - 1,) + D[k + 1:], dt) for k in range(len(D))]
        if self.C:
            self.u = np.zeros(0, dt)
        else:
            self.u = np.asarray(self.u, dt).reshape(D)
        self._normalize_dirs()

    def push_up(self):
        if self.C:
            self.g = np.zeros(self.D, self.dt)
        for c in self.C:
            c.push_up()
        if self.P is not None and self.P.P is not None:
            self.P.g = self.P.g + self.g

    def deinit_pseudo(self):
        for i, c in enumerate(self.C):
            c.deinit_pseudo()
            self.u = c.u.copy() if i == 0 else self.u + c.u

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
