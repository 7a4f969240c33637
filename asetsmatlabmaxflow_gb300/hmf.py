"""Hierarchical max-flow on the GPU with the reference's class interface
(maxflow/asetsHMF2D.m, asetsHMF3D.m): build the label tree from nodes,

    leaves = [asetsHMF2D([], alpha, Ct_i) for ...]
    s = asetsHMF2D(leaves, 0)
    s.MaxFullFlow(numIts, steps, cc)

then read u, pt, div, g, px, py (pz), dataCost, reguCost from the nodes.
MaxPseudoFlow(numIts, steps, cc) runs the class's pseudo-flow algorithm from
the leaves' current labels u.  A node's direction fields lx, ly (, lz) --
the geodesic shape constraint -- are optional; they are normalised when a
run starts and kept normalised on the node, as the class does.
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
        self.lx = self.ly = self.lz = np.zeros(0)

    def _nodes(self):
        out = [self]
        for c in self.C:
            out += c._nodes()
        return out

    def MaxFullFlow(self, numIts: int, steps: float, cc: float, *, ctx=None) -> None:
        """numIts full-flow iterations from zero flows (InitializeFullFlow),
        then CalculateCostsFullFlow; results are stored on every node."""
        self._run(0, numIts, steps, cc, ctx)

    def MaxPseudoFlow(self, numIts: int, steps: float, cc: float, *, ctx=None) -> None:
        """numIts pseudo-flow iterations from zero flows and the leaves'
        labels u; leaves get the new labels, inner nodes the sum of their
        children's (DeInitializePseudoFlow); pt and the costs are left as
        they were."""
        self._run(1, numIts, steps, cc, ctx)

    def _run(self, algo, numIts, steps, cc, ctx):
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
        if algo == 1:
            for i, n in enumerate(nodes):
                if not n.C:
                    outs["u"][i][:] = np.asarray(n.u, dt).reshape(D, order="A").ravel(order="F")
            del outs["pt"]
        lp = _dir_arrays(nodes, self.DIM, D, dt)
        dc = np.zeros(m)
        rc = np.zeros(m)
        N.check(N.lib().asets_hmf_run(
            (ctx or N.Context.default()).handle, algo, dt.itemsize, self.DIM, D[0], D[1],
            D[2] if self.DIM == 3 else 1, m, parent.ctypes.data, ct, al_arr, al_s.ctypes.data,
            *lp["ptrs"], int(numIts), float(steps), float(cc), ptrs(outs["u"]),
            ptrs(outs["pt"]) if "pt" in outs else None,
            ptrs(outs["div"]), ptrs(outs["g"]), ptrs(pouts[0]), ptrs(pouts[1]), p3,
            dc.ctypes.data, rc.ctypes.data))
        _store_dirs(nodes, lp, D)
        names = ["px", "py", "pz"]
        for i, n in enumerate(nodes):
            for k, a in outs.items():
                setattr(n, k, a[i].reshape(shapes[k], order="F"))
            for k in range(self.DIM):
                setattr(n, names[k], pouts[k][i].reshape(fshape[k], order="F"))
            if algo == 0:
                n.dataCost, n.reguCost = float(dc[i]), float(rc[i])


def _dir_arrays(nodes, dim, D, dt):
    """Column-major copies of the nodes' direction fields (the class's
    numel(h.lx) > 0 test) and the pointer tables for the C call."""
    names = ["lx", "ly", "lz"][:dim]
    cols = []
    for n in nodes:
        lx = getattr(n, "lx", None)
        if lx is None or np.size(lx) == 0:
            cols.append(None)
            continue
        row = []
        for nm in names:
            a = getattr(n, nm, None)
            if a is None or np.size(a) == 0:
                raise ValueError(f"a node with lx needs {', '.join(names[1:])} as well")
            row.append(np.ascontiguousarray(np.asarray(a, dt).reshape(D, order="A").ravel(order="F")))
        cols.append(row)
    m = len(nodes)
    ptrs = [None, None, None]
    if any(c is not None for c in cols):
        for k in range(dim):
            ptrs[k] = (ctypes.c_void_p * m)(*[c[k].ctypes.data if c is not None else None
                                               for c in cols])
    return {"cols": cols, "ptrs": ptrs, "names": names}


def _store_dirs(nodes, lp, D):
    """The normalised fields back on the nodes, as the class keeps them."""
    for n, row in zip(nodes, lp["cols"]):
        if row is not None:
            for nm, a in zip(lp["names"], row):
                setattr(n, nm, a.reshape(D, order="F"))


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
        self.lx = self.ly = self.lz = np.zeros(0)

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

        lp = _dir_arrays(nodes, self.DIM, D, dt)
        N.check(N.lib().asets_dag_run(
            (ctx or N.Context.default()).handle, dt.itemsize, self.DIM, D[0], D[1],
            D[2] if self.DIM == 3 else 1, m, nchild.ctypes.data, kids.ctypes.data, ct, al_arr,
            al_s.ctypes.data, *lp["ptrs"], int(numIts), float(steps), float(cc),
            *[ptrs(outs[k]) for k in names], ptrs(pouts[0]), ptrs(pouts[1]),
            ptrs(pouts[2]) if self.DIM == 3 else None))
        _store_dirs(nodes, lp, D)
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
