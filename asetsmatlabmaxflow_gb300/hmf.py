"""Hierarchical max-flow on the GPU with the reference's class interface
(maxflow/asetsHMF2D.m, asetsHMF3D.m): build the label tree from nodes,

    leaves = [asetsHMF2D([], alpha, Ct_i) for ...]
    s = asetsHMF2D(leaves, 0)
    s.MaxFullFlow(numIts, steps, cc)

then read u, pt, div, g, px, py (pz), dataCost, reguCost from the nodes.
Arrays use Matlab index order (numpy arrays shaped D, any memory order)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import native as N


class _HMF:
    DIM = 2

    def __init__(self, children, alpha, Ct=None):
        self.C = list(children)
        self.P = None
        self.Name = ""
        for c in self.C:
            c.P = self
        if not self.C:
            self.Ct = np.asarray(Ct)
            if self.Ct.dtype not in (np.float32, np.float64):
                self.Ct = self.Ct.astype(np.float64)
            self.D = tuple(self.Ct.shape) + (1,) * (self.DIM - self.Ct.ndim)
        else:
            self.D = self.C[0].D
            self.Ct = np.zeros(0, self.C[0].Ct.dtype)
        self.alpha = alpha
        self.u = np.zeros(self.D, self.Ct.dtype)

    def _nodes(self):
        out = [self]
        for c in self.C:
            out += c._nodes()
        return out

    def MaxFullFlow(self, numIts: int, steps: float, cc: float, *, ctx=None) -> None:
        """numIts full-flow iterations from zero flows (InitializeFullFlow),
        then CalculateCostsFullFlow; results are stored on every node."""
        nodes = self._nodes()
        m = len(nodes)
        index = {id(n): i for i, n in enumerate(nodes)}
        parent = np.array([-1] + [index[id(n.P)] for n in nodes[1:]], np.int32)
        dt = np.dtype(next(n.Ct.dtype for n in nodes if not n.C))
        D = self.D
        nvox = int(np.prod(D))
        keep = []

        def col(a):
            a = np.ascontiguousarray(np.asarray(a, dt).reshape(D, order="A").ravel(order="F"))
            keep.append(a)
            return a.ctypes.data

        ct = (ctypes.c_void_p * m)(*[col(n.Ct) if not n.C else None for n in nodes])
        al_arr = (ctypes.c_void_p * m)(*[col(n.alpha) if np.ndim(n.alpha) > 0 else None
                                          for n in nodes])
        al_s = np.array([float(n.alpha) if np.ndim(n.alpha) == 0 else 0.0 for n in nodes])
        shapes = {"u": D, "pt": D, "div": D, "g": D}
        fshape = [D[:k] + (D[k] - 1,) + D[k + 1:] for k in range(self.DIM)]
        outs = {k: [np.empty(int(np.prod(s)), dt) for _ in nodes] for k, s in shapes.items()}
        pouts = [[np.empty(int(np.prod(fs)), dt) for _ in nodes] for fs in fshape]

        def ptrs(lst):
            return (ctypes.c_void_p * m)(*[a.ctypes.data for a in lst])

        p3 = ptrs(pouts[2]) if self.DIM == 3 else None
        dc = np.zeros(m)
        rc = np.zeros(m)
        N.check(N.lib().asets_hmf_full_flow(
            (ctx or N.Context.default()).handle, dt.itemsize, self.DIM, D[0], D[1],
            D[2] if self.DIM == 3 else 1, m, parent.ctypes.data, ct, al_arr, al_s.ctypes.data,
            int(numIts), float(steps), float(cc), ptrs(outs["u"]), ptrs(outs["pt"]),
            ptrs(outs["div"]), ptrs(outs["g"]), ptrs(pouts[0]), ptrs(pouts[1]), p3,
            dc.ctypes.data, rc.ctypes.data))
        names = ["px", "py", "pz"]
        for i, n in enumerate(nodes):
            for k, s in shapes.items():
                setattr(n, k, outs[k][i].reshape(s, order="F"))
            for k in range(self.DIM):
                setattr(n, names[k], pouts[k][i].reshape(fshape[k], order="F"))
            n.dataCost, n.reguCost = float(dc[i]), float(rc[i])


class asetsHMF2D(_HMF):
    DIM = 2


class asetsHMF3D(_HMF):
    DIM = 3


class _DAG:
    """DAG max-flow (maxflow/asetsDAGMF2D.m, asetsDAGMF3D.m): like the HMF
    classes, but a node may be the child of several nodes (P is a list)."""
    DIM = 2

    def __init__(self, children, alpha, Ct=None):
        self.C = list(children)
        self.P = []
        self.Name = ""
        for c in self.C:
            c.P.append(self)
        if not self.C:
            self.Ct = np.asarray(Ct)
            if self.Ct.dtype not in (np.float32, np.float64):
                self.Ct = self.Ct.astype(np.float64)
            self.D = tuple(self.Ct.shape) + (1,) * (self.DIM - self.Ct.ndim)
        else:
            self.D = self.C[0].D
            self.Ct = np.zeros(0, self.C[0].Ct.dtype)
        self.alpha = alpha
        self.u = np.zeros(self.D, self.Ct.dtype)
        self.pn = None

    def _nodes(self):
        out, seen, stack = [], set(), [self]
        while stack:
            n = stack.pop(0)
            if id(n) in seen:
                continue
            seen.add(id(n))
            out.append(n)
            stack.extend(n.C)
        return out

    def MaxFullFlow(self, numIts: int, steps: float, cc: float, *, ctx=None) -> None:
        nodes = self._nodes()
        m = len(nodes)
        index = {id(n): i for i, n in enumerate(nodes)}
        nchild = np.array([len(n.C) for n in nodes], np.int32)
        kids = np.array([index[id(c)] for n in nodes for c in n.C] or [0], np.int32)
        dt = np.dtype(next(n.Ct.dtype for n in nodes if not n.C))
        D = self.D
        keep = []

        def col(a):
            a = np.ascontiguousarray(np.asarray(a, dt).reshape(D, order="A").ravel(order="F"))
            keep.append(a)
            return a.ctypes.data

        ct = (ctypes.c_void_p * m)(*[col(n.Ct) if not n.C else None for n in nodes])
        al_arr = (ctypes.c_void_p * m)(*[col(n.alpha) if np.ndim(n.alpha) > 0 else None
                                          for n in nodes])
        al_s = np.array([float(n.alpha) if np.ndim(n.alpha) == 0 else 0.0 for n in nodes])
        names = ["u", "pt", "pn", "div", "g"]
        outs = {k: [np.empty(int(np.prod(D)), dt) for _ in nodes] for k in names}
        fshape = [D[:k] + (D[k] - 1,) + D[k + 1:] for k in range(self.DIM)]
        pouts = [[np.empty(int(np.prod(fs)), dt) for _ in nodes] for fs in fshape]

        def ptrs(lst):
            return (ctypes.c_void_p * m)(*[a.ctypes.data for a in lst])

        N.check(N.lib().asets_dag_full_flow(
            (ctx or N.Context.default()).handle, dt.itemsize, self.DIM, D[0], D[1],
            D[2] if self.DIM == 3 else 1, m, nchild.ctypes.data, kids.ctypes.data, ct, al_arr,
            al_s.ctypes.data, int(numIts), float(steps), float(cc),
            *[ptrs(outs[k]) for k in names], ptrs(pouts[0]), ptrs(pouts[1]),
            ptrs(pouts[2]) if self.DIM == 3 else None))
        for i, n in enumerate(nodes):
            for k in names:
                setattr(n, k, outs[k][i].reshape(D, order="F"))
            if len(n.P) < 2:
                n.pn = None
            for k, nm in enumerate(["px", "py", "pz"][:self.DIM]):
                setattr(n, nm, pouts[k][i].reshape(fshape[k], order="F"))


class asetsDAGMF2D(_DAG):
    DIM = 2


class asetsDAGMF3D(_DAG):
    DIM = 3
