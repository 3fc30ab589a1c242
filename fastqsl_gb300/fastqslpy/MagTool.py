"""Drop-in for fastqslpy/MagTool.py: field-line polylines on the GPU.

Same functions and positional signatures as the reference (``trilerp``
MagTool.py:3-18, ``Bnorm`` :20-22, ``RK4_bline`` :24-34, ``TraceBline``
:36-45), computed by the float64 kernels of libfastqsl_gb300.so
(qsl_sample_points, qsl_trace_path) in the reference's operation order, so
the returned points are the reference's bit for bit; plus ``TraceBlines``,
many seeds in one launch.  Fields may be NumPy arrays, PyTorch tensors or
CuPy arrays of shape (nx, ny, nz) in any memory order; they are read as
float32 (the notebooks' arrays).  ``nk`` is accepted and ignored: results
come back as NumPy arrays, as with the reference's default ``nk=np``.

Kept from the reference: TraceBline runs its fixed steps of 0.25 forward
and -0.25 backward whatever ``dr`` it is given; lines stop when a
coordinate is below 0 or above the FIRST axis length (y and z above their
own lengths are clamped to the top plane and the line runs on along it);
index 0 of the output is never written; trilerp/Bnorm clamp the caller's
point in place.  Where the reference raises (a zero field sample, a float32
point exactly on the far face), a line here stops and an index is clamped
to the last node.
"""
import numpy as np
import torch

from .. import _lib
from ..api import as_xfast, stream_handle

__all__ = ["trilerp", "Bnorm", "RK4_bline", "TraceBline", "TraceBlines"]


def _field(Bx, By, Bz):
    B = [as_xfast(b) for b in (Bx, By, Bz)]
    if not (B[0].shape == B[1].shape == B[2].shape):
        raise ValueError("Bx, By, Bz shapes differ")
    return B


def _clamp_inplace(vec, shape):
    """trilerp's in-place clamp of the caller's point (MagTool.py:4-10), in
    the point's own precision; the sample is then taken at the clamped
    values, as there."""
    if isinstance(vec, np.ndarray) and vec.dtype.kind == "f" and vec.shape == (3,):
        for d in range(3):
            if vec[d] < 0:
                vec[d] = 1e-8
            if vec[d] > shape[d]:
                vec[d] = shape[d] - 1e-8


def _seed_clamp(P, shape):
    """RK4_bline clamps its start point in place at its first sample, which
    is taken only when the point passes the loop's bounds check (every
    coordinate in [0, nx])."""
    if isinstance(P, np.ndarray) and P.shape == (3,) and P.dtype.kind == "f":
        if not (np.any(P < 0) or np.any(P > shape[0]) or np.any(np.isnan(P))):
            _clamp_inplace(P, shape)


def _sample(Bx, By, Bz, vec, normalize):
    B = _field(Bx, By, Bz)
    nx, ny, nz = (int(v) for v in B[0].shape)
    _clamp_inplace(vec, (nx, ny, nz))
    v = np.asarray(vec, dtype=np.float64).reshape(-1, 3)
    pts = torch.from_numpy(np.ascontiguousarray(v)).to(B[0].device)
    out = torch.empty_like(pts)
    _lib.check(_lib.load().qsl_sample_points(B[0].data_ptr(), B[1].data_ptr(), B[2].data_ptr(), nx, ny, nz,
                                             pts.data_ptr(), len(v), int(normalize), out.data_ptr(),
                                             stream_handle()), "qsl_sample_points")
    res = out.cpu().numpy()
    return res[0] if np.ndim(vec) == 1 else res


def trilerp(Bx, By, Bz, vec, nk=np):
    """B at the point `vec` by trilinear interpolation (float64, shape (3,));
    `vec` of shape (n, 3) gives (n, 3)."""
    return _sample(Bx, By, Bz, vec, False)


def Bnorm(Bx, By, Bz, vec, nk=np):
    """The unit field vector at `vec`."""
    return _sample(Bx, By, Bz, vec, True)


def _trace(B, seeds, out, start, stop, step, dr):
    nx, ny, nz = (int(v) for v in B[0].shape)
    n, length = int(out.shape[1]), int(out.shape[2])
    _lib.check(_lib.load().qsl_trace_path(B[0].data_ptr(), B[1].data_ptr(), B[2].data_ptr(), nx, ny, nz,
                                          seeds.data_ptr(), n, int(start), int(stop), int(step), float(dr),
                                          out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(), length,
                                          stream_handle()), "qsl_trace_path")


def RK4_bline(Bx, By, Bz, PP0, xl, yl, zl, steprange, dr=0.25, nk=np):
    """Fixed-step RK4 from PP0, writing the points into xl, yl, zl (NumPy
    arrays, in place) at the indices of `steprange` (a range)."""
    if not isinstance(steprange, range):
        steprange = range(*steprange) if isinstance(steprange, tuple) else steprange
        if not isinstance(steprange, range):
            raise TypeError("steprange must be a range")
    B = _field(Bx, By, Bz)
    dev = B[0].device
    out = torch.from_numpy(np.stack([np.asarray(a, np.float32) for a in (xl, yl, zl)])[:, None, :].copy()).to(dev)
    _seed_clamp(PP0, tuple(B[0].shape))
    seeds = torch.tensor(np.asarray(PP0, np.float64).reshape(1, 3), device=dev)
    _trace(B, seeds, out, steprange.start, steprange.stop, steprange.step, dr)
    res = out[:, 0, :].cpu().numpy()
    for a, r in zip((xl, yl, zl), res):
        a[...] = r


def TraceBlines(Bx, By, Bz, seeds, maxstep=2e4, dr=0.25):
    """TraceBline for many seeds (n, 3) in one pair of launches; returns
    (xlines, ylines, zlines) float32 arrays of shape (n, maxstep), NaN where
    a line has no point.  Unlike TraceBline, the step is `dr` (forward +dr,
    backward -dr)."""
    B = _field(Bx, By, Bz)
    dev = B[0].device
    maxstep = int(maxstep)
    mid = int(maxstep / 2)
    s = torch.tensor(np.asarray(seeds, np.float64).reshape(-1, 3), device=dev)
    out = torch.full((3, s.shape[0], maxstep), float("nan"), dtype=torch.float32, device=dev)
    _trace(B, s, out, mid, maxstep, 1, abs(dr))
    _trace(B, s, out, mid, 0, -1, -abs(dr))
    r = out.cpu().numpy()
    return r[0], r[1], r[2]


def TraceBline(Bx, By, Bz, Pxyz0, dr=0.25, maxstep=2e4, nk=np):
    """The field line through Pxyz0: (xline, yline, zline) float32 arrays of
    maxstep points, the seed at index maxstep // 2, forward points after it
    and backward points before it, NaN elsewhere.  Steps are 0.25 cell
    whatever `dr` is."""
    _seed_clamp(Pxyz0, tuple(int(v) for v in Bx.shape))
    x, y, z = TraceBlines(Bx, By, Bz, np.asarray(Pxyz0).reshape(1, 3), maxstep=maxstep, dr=0.25)
    return x[0], y[0], z[0]
