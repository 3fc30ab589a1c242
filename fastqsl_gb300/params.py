"""Integrator settings (``qsl_trace_params`` of include/fastqsl_gb300.h).

The reference hard-wires its settings as ``#define``s in each kernel file;
the presets below reproduce them:

* RK4   — ``fastqslpy/cu/TraceBline.cu:10-12``: length limit 2*(nx+ny+nz),
  100000 steps, exit-segment twist term (``:362-365``).
* RKF45 — ``fastqslpy/cu/TraceBlineAdaptive.cu:10-13,354-370``: tol 1e-3 with
  the ``|b0.n|^1.5`` law, accepted step clamped to [0.1, 100], shrink 0.618 on
  rejection, length limit 3*(nx+ny+nz), 500000 steps.
* Scott — ``fastqslpy/cu/TraceBlineScott.cu:10-14``: length limit
  2*(nx+ny+nz), 10000 steps shared by both directions, tol 1e-3*tol_coef.
* ``max_rejects`` (no counterpart in the reference, 0 in its presets): the
  number of rejected trial steps in a row that ends a direction.

* Stretched-grid RKF45 — ``fastqslpy/cu/TraceBlineAdaptiveStretch.cu:10-12,
  336-371``: the RKF45 settings with length limit 2 x the summed coordinate
  extents, no step limit (capped here at 2^31 - 1), exit-segment twist term
  (``:401-404``).
"""
import ctypes

RK4 = 0
RKF45 = 1
TOL_REFERENCE = 0
TOL_ABSOLUTE = 1
ARITH_EXACT = 0
ARITH_FAST = 1
# qsl_trace on the fp16 brick store only: fp16 x weights (opt-in, see
# QSL_ARITH_FAST_W16 in include/fastqsl_gb300.h)
ARITH_FAST_W16 = 2

# qsl_line_status: how one direction of a line ended
LINE_FACE = 0
LINE_EDGE = 1
LINE_NAN = 2
LINE_MAX_STEPS = 3
LINE_MAX_LENGTH = 4
LINE_REJECT_LIMIT = 5

# Rejected trial steps in a row that end a direction in the absolute-
# tolerance preset: 64 rejections shrink the step by 0.618^64 ~ 4e-14, far
# below what a float position can resolve, so a controller that has not
# accepted by then never will (the reference presets keep 0, no limit).
MAX_REJECTS = 64


class TraceParams(ctypes.Structure):
    _fields_ = [
        ("integrator", ctypes.c_int32),
        ("tol_law", ctypes.c_int32),
        ("tol", ctypes.c_double),
        ("h_min", ctypes.c_double),
        ("h_max", ctypes.c_double),
        ("reject_factor", ctypes.c_double),
        ("len_ratio", ctypes.c_double),
        ("max_steps", ctypes.c_int64),
        ("boundary_twist", ctypes.c_int32),
        ("arith", ctypes.c_int32),
        ("max_rejects", ctypes.c_int32),
    ]

    def copy(self, **kw):
        p = TraceParams()
        ctypes.pointer(p)[0] = self
        for k, v in kw.items():
            setattr(p, k, v)
        return p

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}

    def __repr__(self):
        return "TraceParams(%s)" % ", ".join(f"{k}={v!r}" for k, v in self.as_dict().items())


def reference_rk4(arith=ARITH_EXACT) -> TraceParams:
    return TraceParams(RK4, TOL_REFERENCE, 1e-3, 0.1, 100.0, 0.618, 2.0, 100000, 1, arith)


def reference_rkf45(arith=ARITH_EXACT) -> TraceParams:
    return TraceParams(RKF45, TOL_REFERENCE, 1e-3, 0.1, 100.0, 0.618, 3.0, 500000, 0, arith)


def reference_scott(arith=ARITH_EXACT) -> TraceParams:
    """The Scott tracer's settings; its tolerance is 1e-3*tol_coef (the
    reference leaves the variable uninitialised, TraceBlineScott.cu:352,378)."""
    return TraceParams(RKF45, TOL_ABSOLUTE, 1e-3, 0.1, 100.0, 0.618, 2.0, 10000, 0, arith)


def reference_stretch(arith=ARITH_EXACT) -> TraceParams:
    return TraceParams(RKF45, TOL_REFERENCE, 1e-3, 0.1, 100.0, 0.618, 2.0, 2**31 - 1, 1, arith)


def absolute_rkf45(tol=1e-4, h_min=1e-3, h_max=1.0, arith=ARITH_FAST, max_rejects=MAX_REJECTS) -> TraceParams:
    """RKF45 with an absolute local tolerance and explicit step bounds (the
    benchmark settings: tol 1e-4, h in [1e-3, 1]); a direction ends where
    `max_rejects` trial steps in a row were rejected (status REJECT_LIMIT)."""
    return TraceParams(RKF45, TOL_ABSOLUTE, tol, h_min, h_max, 0.618, 3.0, 500000, 0, arith, max_rejects)


def fixed_rk4(max_steps=100000, len_ratio=2.0, arith=ARITH_EXACT) -> TraceParams:
    return TraceParams(RK4, TOL_REFERENCE, 1e-3, 0.1, 100.0, 0.618, len_ratio, max_steps, 1, arith)
