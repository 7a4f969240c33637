"""ORACLE -- test infrastructure only: float64 numpy restatement of the
star-shape Potts 2D solver maxflow/asetsPotts2D_starShape.m (Matlab, double
precision), operation by operation in the order Matlab evaluates them, to
check the GPU solver (asetsmatlabmaxflow_gb300/csrc/starshape.cu).

Arrays are (rows, cols[, nlab]) float64; ss_init_points is (nlab, 2) of
1-based (column, row) pairs as ss_initPoints(k,1), ss_initPoints(k,2).
"""
from __future__ import annotations

import numpy as np


def distance_field(rows, cols, p):
    """bwdist of one set pixel: the Euclidean distance to it, in single
    precision as bwdist returns it (asetsPotts2D_starShape.m:87-89)."""
    y, x = np.mgrid[0:rows, 0:cols]
    d2 = (y - (p[1] - 1)).astype(np.float64) ** 2 + (x - (p[0] - 1)).astype(np.float64) ** 2
    return np.sqrt(d2).astype(np.float32)


def direction_fields(rows, cols, pts):
    """ve1 (rows x cols+1), ve2 (rows+1 x cols), div_ve (:84-97)."""
    L = len(pts)
    ve1 = np.zeros((rows, cols + 1, L))
    ve2 = np.zeros((rows + 1, cols, L))
    div_ve = np.zeros((rows, cols, L))
    for k in range(L):
        vd = distance_field(rows, cols, pts[k])
        ve1[:, 1:cols, k] = (vd[:, 1:cols] - vd[:, 0:cols - 1]).astype(np.float64)
        ve2[1:rows, :, k] = (vd[1:rows, :] - vd[0:rows - 1, :]).astype(np.float64)
        div_ve[:, :, k] = ((ve1[:, 1:cols + 1, k] - ve1[:, 0:cols, k]) + ve2[1:rows + 1, :, k]) \
            - ve2[0:rows, :, k]
    return ve1, ve2, div_ve


def solve(Ct, alpha, pars, pts):
    """Returns (u, erriter, i) with i the 1-based iteration of the break (or
    iterNum), as the .m function's outputs."""
    rows, cols, nlab, iterNum = (int(v) for v in pars[:4])
    beta, cc, steps, stepv = (float(v) for v in pars[4:8])
    Ct = np.array(Ct, dtype=np.float64)
    alpha = np.asarray(alpha, dtype=np.float64)
    vol = rows * cols * nlab
    for k in range(nlab):  # hard constraints at the init points (:34-38)
        Ct[pts[k][1] - 1, pts[k][0] - 1, :] = 10e11
        Ct[pts[k][1] - 1, pts[k][0] - 1, k] = 0
    u = np.zeros((rows, cols, nlab))
    pt = np.zeros((rows, cols, nlab))
    ps = Ct.min(axis=2)
    divp = np.zeros((rows, cols, nlab))
    pp1 = np.zeros((rows, cols + 1, nlab))
    pp2 = np.zeros((rows + 1, cols, nlab))
    v = np.zeros((rows, cols, nlab))
    vx1 = np.zeros((rows, cols + 1, nlab))
    vx2 = np.zeros((rows + 1, cols, nlab))
    gdv = np.zeros((rows, cols, nlab))
    ve1, ve2, div_ve = direction_fields(rows, cols, pts)
    erriter = np.zeros(iterNum)
    i = 0
    for i in range(1, iterNum + 1):
        pd = np.zeros((rows, cols))
        for k in range(nlab):
            ud = (divp[:, :, k] + gdv[:, :, k]) - ((ps - pt[:, :, k]) + u[:, :, k] / cc)
            pp1[:, 1:cols, k] = steps * (ud[:, 1:cols] - ud[:, 0:cols - 1]) + pp1[:, 1:cols, k]
            pp2[1:rows, :, k] = steps * (ud[1:rows, :] - ud[0:rows - 1, :]) + pp2[1:rows, :, k]
            gk = np.sqrt((((pp1[:, 0:cols, k] ** 2 + pp1[:, 1:cols + 1, k] ** 2)
                           + pp2[0:rows, :, k] ** 2) + pp2[1:rows + 1, :, k] ** 2) * 0.5)
            le = gk <= alpha[:, :, k]
            with np.errstate(invalid="ignore", divide="ignore"):
                gk = le.astype(np.float64) + (~le).astype(np.float64) * (gk / alpha[:, :, k])
                gk = 1.0 / gk
            pp1[:, 1:cols, k] = (0.5 * (gk[:, 1:cols] + gk[:, 0:cols - 1])) * pp1[:, 1:cols, k]
            pp2[1:rows, :, k] = (0.5 * (gk[1:rows, :] + gk[0:rows - 1, :])) * pp2[1:rows, :, k]
            divp[:, :, k] = ((pp1[:, 1:cols + 1, k] - pp1[:, 0:cols, k]) + pp2[1:rows + 1, :, k]) \
                - pp2[0:rows, :, k]
            ud = ((-(divp[:, :, k] + gdv[:, :, k])) + ps) + u[:, :, k] / cc
            pt[:, :, k] = np.minimum(ud, Ct[:, :, k])
            pd = pd + (((divp[:, :, k] + gdv[:, :, k]) + pt[:, :, k]) - u[:, :, k] / cc)
        ps = pd / nlab + 1 / (cc * nlab)
        for k in range(nlab):
            ud = ((gdv[:, :, k] + divp[:, :, k]) + pt[:, :, k]) - (ps + u[:, :, k] / cc)
            vx1[:, 1:cols, k] = ud[:, 1:cols] - ud[:, 0:cols - 1]
            vx2[1:rows, :, k] = ud[1:rows, :] - ud[0:rows - 1, :]
            gk = (((vx1[:, 0:cols, k] * ve1[:, 0:cols, k] + vx1[:, 1:cols + 1, k] * ve1[:, 1:cols + 1, k])
                   + vx2[0:rows, :, k] * ve2[0:rows, :, k]) + vx2[1:rows + 1, :, k] * ve2[1:rows + 1, :, k]) * 0.5
            v[:, :, k] = v[:, :, k] + stepv * gk
            v[:, :, k] = np.minimum(v[:, :, k], 0)
            vx1[:, 1:cols, k] = v[:, 1:cols, k] - v[:, 0:cols - 1, k]
            vx2[1:rows, :, k] = v[1:rows, :, k] - v[0:rows - 1, :, k]
            gdv[:, :, k] = (((vx1[:, 0:cols, k] * ve1[:, 0:cols, k] + vx1[:, 1:cols + 1, k] * ve1[:, 1:cols + 1, k])
                             + vx2[0:rows, :, k] * ve2[0:rows, :, k])
                            + vx2[1:rows + 1, :, k] * ve2[1:rows + 1, :, k]) * 0.5 + v[:, :, k] * div_ve[:, :, k]
        erru_sum = 0.0
        for k in range(nlab):
            erru = cc * (((divp[:, :, k] + gdv[:, :, k]) + pt[:, :, k]) - ps)
            u[:, :, k] = u[:, :, k] - erru
            erru_sum = erru_sum + np.sum(np.abs(erru))
        erriter[i - 1] = erru_sum / vol
        if erriter[i - 1] < beta:
            break
    return u, erriter, i
