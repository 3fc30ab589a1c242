"""Drop-in for fastqslpy/FastQSL.py: Q assembly on the GPU.

Same functions and positional signatures as the reference
(``CookPseudoLine`` FastQSL.py:4-57, ``ResReshape`` :59-63, ``QCalcPlane``
:65-117, ``curl_of_B_grid`` :120-131, ``copy_boundary`` :133-141,
``diff_3point`` :143-163), plus the pseudo-line Q and merge steps that the
reference keeps in notebook cells (``QCalcCut``, ``QMerge``: demo/
Q_RKF45CuPy.ipynb cells 10-11).  The Q computations run in the CUDA kernels
of libfastqsl_gb300.so with the reference's FP32 rounding; inputs may be
PyTorch CUDA tensors or CuPy arrays, results are PyTorch CUDA tensors.
"""
import ctypes

import numpy as np
import torch

from .. import _lib
from ..api import ptr, stream_handle


def _t(a):
    """A contiguous CUDA tensor view of a device array (no copy when possible)."""
    if isinstance(a, torch.Tensor):
        t = a
    else:
        t = torch.as_tensor(a, device="cuda")
    if not t.is_cuda:
        raise ValueError("expected a device array")
    return t.contiguous()


def _dir3(d):
    if d is None:
        return (0.0, 0.0, 1.0)
    if isinstance(d, torch.Tensor):
        return tuple(float(v) for v in d.detach().cpu().tolist())
    if hasattr(d, "get"):  # CuPy
        return tuple(float(v) for v in d.get().tolist())
    return tuple(float(v) for v in np.asarray(d).tolist())


def ResReshape(shape, *args):
    """Reshapes each array to `shape` (FastQSL.py:59-63)."""
    return [a.reshape(shape) for a in args]


def QCalcPlane(x_end_arr, y_end_arr, z_end_arr, flag_end_arr,
               x_start_arr, y_start_arr, z_start_arr, flag_start_arr,
               Bx_in_arr, By_in_arr, Bz_in_arr,
               Bx_out_arr, By_out_arr, Bz_out_arr,
               Bx_0_arr, By_0_arr, Bz_0_arr,
               B_flag_arr, stride_step, CrossBC_dir=None):
    """Q on the interior of a 2-D seed grid from the traced footpoints
    (FastQSL.py:65-117).  Returns (n0-2, n1-2) float32: Q >= 1, NaN where a
    neighbouring seed's start or end flag differs."""
    xe = _t(x_end_arr)
    n0, n1 = int(xe.shape[0]), int(xe.shape[1])
    Q = torch.empty((n0 - 2, n1 - 2), dtype=torch.float32, device=xe.device)
    jac = (1. / (2. * stride_step)) ** 4.
    cd = (ctypes.c_float * 3)(*_dir3(CrossBC_dir))
    arrs = [xe] + [_t(a) for a in (y_end_arr, z_end_arr, flag_end_arr, x_start_arr, y_start_arr, z_start_arr,
                                   flag_start_arr, Bz_in_arr, Bz_out_arr, Bx_0_arr, By_0_arr, Bz_0_arr)]
    lib = _lib.load()
    _lib.check(lib.qsl_qcalc_plane(*[ptr(a) for a in arrs], n0, n1, 1, float(np.float32(jac)), cd, ptr(Q), None,
                                   stream_handle()), "QCalcPlane")
    return Q


def _uint64(v, device):
    dt = getattr(torch, "uint64", torch.int64)
    return torch.tensor([v], dtype=dt, device=device)


def CookPseudoLine(x_end_arr, y_end_arr, z_end_arr, flag_end_arr,
                   x_start_arr, y_start_arr, z_start_arr, flag_start_arr,
                   Bx_in_arr, By_in_arr, Bz_in_arr,
                   Bx_out_arr, By_out_arr, Bz_out_arr,
                   Bz_0_arr, B_flag_arr, stride_this):
    """Pseudo-line seeds for the near-in-plane pixels (B_flag == 1) and
    zeroed output buffers for their trace (FastQSL.py:4-57).  Returns the
    reference's 25-tuple."""
    bf = _t(B_flag_arr)
    dev = bf.device
    n = int(bf.numel())
    lib = _lib.load()
    cut = [torch.empty(4 * n, dtype=torch.float32, device=dev) for _ in range(3)]
    bz0s = torch.empty(n, dtype=torch.float32, device=dev)
    bz0e = torch.empty(n, dtype=torch.float32, device=dev)
    count = torch.zeros(2, dtype=torch.int64, device=dev)
    wb = int(lib.qsl_cook_workspace_bytes(n))
    work = torch.empty((wb + 7) // 8, dtype=torch.int64, device=dev)
    _lib.check(lib.qsl_cook_pseudo_line(ptr(bf), ptr(_t(x_start_arr)), ptr(_t(y_start_arr)), ptr(_t(z_start_arr)),
                                        ptr(_t(flag_start_arr)), ptr(_t(Bz_in_arr)), ptr(_t(Bz_out_arr)), n, 1, n, 0,
                                        float(np.float32(stride_this)), ptr(cut[0]), ptr(cut[1]), ptr(cut[2]),
                                        ptr(bz0s), ptr(bz0e), None, ptr(count), ptr(work), wb, stream_handle()),
               "CookPseudoLine")
    k = int(count[0].item())
    m = 4 * k
    cut_inp_x, cut_inp_y, cut_inp_z = (c[:m].clone() for c in cut)
    z = [torch.zeros(m, dtype=torch.float32, device=dev) for _ in range(15)]
    (cut_start_x, cut_start_y, cut_start_z, cut_end_x, cut_end_y, cut_end_z,
     Bx_start_cut, By_start_cut, Bz_start_cut, Bx_end_cut, By_end_cut, Bz_end_cut,
     Bx_inp_cut, By_inp_cut, Bz_inp_cut) = z
    line_len_cut = torch.zeros(m, dtype=torch.float64, device=dev)
    N_cut = _uint64(m, dev)
    B_flag_cut, flag_cut_start, flag_cut_end = (torch.zeros(m, dtype=torch.int32, device=dev) for _ in range(3))
    return (cut_inp_x, cut_inp_y, cut_inp_z,
            cut_start_x, cut_start_y, cut_start_z, flag_cut_start,
            cut_end_x, cut_end_y, cut_end_z, flag_cut_end,
            Bx_inp_cut, By_inp_cut, Bz_inp_cut, B_flag_cut,
            Bx_start_cut, By_start_cut, Bz_start_cut,
            Bx_end_cut, By_end_cut, Bz_end_cut, N_cut, line_len_cut,
            bz0s[:k].clone(), bz0e[:k].clone())


def QCalcCut(cut_start_x, cut_start_y, cut_start_z, flag_cut_start,
             cut_end_x, cut_end_y, cut_end_z, flag_cut_end,
             Bz0_start, Bz0_end, stride_this):
    """Q of each pseudo-line pixel from its 4 traced pseudo-lines
    (demo/Q_RKF45CuPy.ipynb cell 10).  Returns float32 (len(Bz0_start),)."""
    s = _t(Bz0_start)
    k = int(s.numel())
    out = torch.empty(k, dtype=torch.float32, device=s.device)
    st = np.float32(stride_this)
    jac = float((1 / st / 2) ** 4)
    arrs = [_t(a) for a in (cut_start_x, cut_start_y, cut_start_z, flag_cut_start,
                            cut_end_x, cut_end_y, cut_end_z, flag_cut_end, Bz0_start, Bz0_end)]
    _lib.check(_lib.load().qsl_qcut(*[ptr(a) for a in arrs], k, None, k, jac, ptr(out), None, stream_handle()),
               "QCalcCut")
    return out


def QMerge(Q, Qcut, B_flag_arr):
    """Q_all with the interior from QCalcPlane and the flagged pixels from
    QCalcCut; returns (Q_all, Q_final = Q_all[1:-1, 1:-1])
    (demo/Q_RKF45CuPy.ipynb cell 11)."""
    bf = _t(B_flag_arr)
    Q_all = torch.zeros(bf.shape, dtype=torch.float32, device=bf.device)
    Q_all[1:-1, 1:-1] = _t(Q)
    Q_all[bf == 1] = _t(Qcut)
    return Q_all, Q_all[1:-1, 1:-1]


# ---- curl of B on a (possibly non-uniform) grid (FastQSL.py:119-163) ----

def diff_3point(Cube, arr_x, axis):
    """Three-point derivative of a 3-D array along `axis` on the grid
    coordinates arr_x, at the interior points (FastQSL.py:143-163)."""
    C = _t(Cube) if not isinstance(Cube, torch.Tensor) else Cube
    x = torch.as_tensor(arr_x, device=C.device, dtype=C.dtype)
    dx = x[1:] - x[:-1]
    shape = [1, 1, 1]
    shape[axis] = -1
    dxl = dx[:-1].reshape(shape)
    dxr = dx[1:].reshape(shape)
    sl = [slice(1, -1)] * 3

    def take(off):
        s = list(sl)
        s[axis] = slice(1 + off, C.shape[axis] - 1 + off)
        return C[tuple(s)]

    ctr = take(0)
    return ((take(1) - ctr) / dxr * dxl / (dxr + dxl) + (ctr - take(-1)) / dxl * dxr / (dxr + dxl))


def copy_boundary(arr):
    arr[:, :, 0] = arr[:, :, 1]
    arr[:, 0, :] = arr[:, 1, :]
    arr[0, :, :] = arr[1, :, :]
    arr[:, :, -1] = arr[:, :, -2]
    arr[:, -1, :] = arr[:, -2, :]
    arr[-1, :, :] = arr[-2, :, :]
    return arr


def curl_of_B_grid(Bx, By, Bz, arr_x, arr_y, arr_z):
    """curl B by three-point differences with the boundary copy
    (FastQSL.py:120-141) on the GPU (qsl_curl_grid): float32 arithmetic in
    the reference's order, float64 results of shape (nx, ny, nz), x fastest in
    memory, ready (after .float()) to be the current density of the twist
    integral."""
    from .. import _lib
    from ..api import as_xfast, ptr, stream_handle
    arrs = [as_xfast(b) for b in (Bx, By, Bz)]
    nx, ny, nz = (int(v) for v in arrs[0].shape)
    dev = arrs[0].device
    ax = [torch.as_tensor(c).to(device=dev, dtype=torch.float32).contiguous() for c in (arr_x, arr_y, arr_z)]
    out = [torch.empty((nz, ny, nx), dtype=torch.float64, device=dev).permute(2, 1, 0) for _ in range(3)]
    _lib.check(_lib.load().qsl_curl_grid(*[ptr(a) for a in arrs], nx, ny, nz, *[ptr(a) for a in ax],
                                         *[ptr(o) for o in out], stream_handle()), "qsl_curl_grid")
    return tuple(out)
