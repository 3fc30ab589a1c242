"""Test infrastructure only: a CPU restatement of fastqslpy/MagTool.py
(the reference's NumPy field-line plotter) used as the checker of the GPU
polyline tracer.  Nothing in the product imports it.

The reference module computes in float64: its corner weights are float
positions minus int64 indices (MagTool.py:12,15), which NumPy promotes to
float64, so every product and sum after the float32 corner gather is
float64; the points are stored into float32 arrays (:31, :40).  This
restatement uses Python floats (IEEE float64) in the same order:

* trilerp (:3-18): per axis, a value below 0 becomes 1e-8 and one above n
  becomes n - 1e-8 (in place on the caller's array); the corner block is
  B[i0:i0+2, j0:j0+2, k0:k0+2], shorter at the last node and broadcast
  against the (2, 2, 2) weights w[i]*w[j]*w[k] (left to right); np.sum of the
  C-contiguous product array sums the 8 terms as ((p0+p1)+(p2+p3)) +
  ((p4+p5)+(p6+p7)) in [x][y][z] order;
* Bnorm (:20-22): B / sqrt((bx^2 + by^2) + bz^2);
* RK4_bline (:24-34): stop when a coordinate is below 0 or above the FIRST
  axis length; f1 is sampled at the current point itself (so its clamp
  persists), f2..f4 at P + dr*f/2, P + dr*f/2, P + dr*f3; the point is
  stored, then P += (dr*(((f1 + 2 f2) + 2 f3) + f4)) / 6;
* TraceBline (:36-45): NaN-filled float32 arrays of maxstep points; forward
  over range(maxstep//2, maxstep) with dr = +0.25 and backward over
  range(maxstep//2, 0, -1) with dr = -0.25 (its own dr argument is not
  used), both from the same seed array.
"""
import math

import numpy as np


def _clamp(v, n):
    if v < 0:
        return 1e-8
    if v > n:
        return n - 1e-8
    return v


def trilerp(B, vec):
    """B = (Bx, By, Bz), arrays indexed [x, y, z]; vec: 3 floats (clamped
    copy).  Returns 3 floats."""
    shape = B[0].shape
    c = [_clamp(float(vec[d]), shape[d]) for d in range(3)]
    i0 = [min(int(c[d]), shape[d] - 1) for d in range(3)]
    i1 = [min(i0[d] + 1, shape[d] - 1) for d in range(3)]
    w = [(1.0 - (c[d] - i0[d]), c[d] - i0[d]) for d in range(3)]
    out = []
    for comp in B:
        p = []
        for i in range(2):
            for j in range(2):
                for k in range(2):
                    wt = w[0][i] * w[1][j] * w[2][k]
                    p.append(float(comp[i1[0] if i else i0[0], i1[1] if j else i0[1], i1[2] if k else i0[2]]) * wt)
        out.append(((p[0] + p[1]) + (p[2] + p[3])) + ((p[4] + p[5]) + (p[6] + p[7])))
    return out


def bnorm(B, vec):
    b = trilerp(B, vec)
    s = math.sqrt((b[0] * b[0] + b[1] * b[1]) + b[2] * b[2])
    return [x / s for x in b]


def rk4_bline(B, P, xl, yl, zl, steprange, dr):
    """Fills xl, yl, zl (float32 arrays) at the indices of `steprange`."""
    shape = B[0].shape
    bound = shape[0]
    P = [float(v) for v in P]
    for idx in steprange:
        if min(P) < 0 or max(P) > bound or any(math.isnan(v) for v in P):
            break
        P = [_clamp(P[d], shape[d]) for d in range(3)]
        f1 = bnorm(B, P)
        f2 = bnorm(B, [P[d] + dr * f1[d] / 2.0 for d in range(3)])
        f3 = bnorm(B, [P[d] + dr * f2[d] / 2.0 for d in range(3)])
        f4 = bnorm(B, [P[d] + dr * f3[d] for d in range(3)])
        xl[idx], yl[idx], zl[idx] = (np.float32(v) for v in P)
        P = [P[d] + dr * (f1[d] + 2.0 * f2[d] + 2.0 * f3[d] + f4[d]) / 6.0 for d in range(3)]


def trace_bline(B, seed, maxstep=2e4):
    maxstep = int(maxstep)
    mid = int(maxstep / 2)
    xl, yl, zl = (np.full(maxstep, np.nan, np.float32) for _ in range(3))
    rk4_bline(B, seed, xl, yl, zl, range(mid, maxstep), 0.25)
    rk4_bline(B, seed, xl, yl, zl, range(mid, 0, -1), -0.25)
    return xl, yl, zl
