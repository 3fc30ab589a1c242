"""CPU ORACLE (test infrastructure): NumPy restatement of the reference's Q
assembly.

* ``qcalc_plane``      — fastqslpy/FastQSL.py:65-117 (QCalcPlane)
* ``cook_pseudo_line`` — fastqslpy/FastQSL.py:4-57 (CookPseudoLine), seed part
* ``qcut``             — demo/Q_RKF45CuPy.ipynb cell 10 (pseudo-line Q)
* ``merge``            — demo/Q_RKF45CuPy.ipynb cell 11 (Q_all, Q_final)
* ``qcalc_plane_f64``  — the same formulas in float64 (the FP64 oracle's Q)

Arithmetic follows the reference: float32 arrays throughout (NumPy/CuPy
semantics with Python-float scalars kept weak), Q clamped to >= 1, NaN where a
neighbour's start or end flag differs from the centre's.
"""
import numpy as np


def face_coords(x, y, z, flag):
    """Maps a footpoint to 2-D coordinates on its exit face: z-face -> (x, y),
    y-face -> (z, x), x-face -> (y, z) (FastQSL.py:76-84).  Flags outside
    1..6 give (0, 0)."""
    d = (flag - 1) // 2
    X = np.zeros(flag.shape, np.float32)
    Y = np.zeros(flag.shape, np.float32)
    m = d == 2
    X[m], Y[m] = x[m], y[m]
    m = d == 1
    X[m], Y[m] = z[m], x[m]
    m = d == 0
    X[m], Y[m] = y[m], z[m]
    return X, Y


def _jacobian_terms(X1, Y1, X2, Y2):
    """Central differences of both footpoint maps along the two grid axes of
    the seed plane and the four Jacobian-product terms a, b, c, d
    (FastQSL.py:99-107)."""
    def d0(A):
        return A[2:, 1:-1] - A[:-2, 1:-1]

    def d1(A):
        return A[1:-1, 2:] - A[1:-1, :-2]

    dx2xc, dx2yc = d0(X2), d1(X2)
    dy2xc, dy2yc = d0(Y2), d1(Y2)
    dx1xc, dx1yc = d0(X1), d1(X1)
    dy1xc, dy1yc = d0(Y1), d1(Y1)
    a = dx2xc * dy1yc - dx2yc * dy1xc
    b = dx2yc * dx1xc - dx2xc * dx1yc
    c = dy2xc * dy1yc - dy2yc * dy1xc
    d = dy2yc * dx1xc - dy2xc * dx1yc
    return a, b, c, d


def _flag_jump(fs, fe):
    """Sum over the 4 neighbours of |flag difference|, start and end maps
    (FastQSL.py:86-96); > 0 marks a pixel whose neighbourhood straddles a
    change of exit face."""
    def jump(F):
        c = F[1:-1, 1:-1]
        return (np.abs(F[2:, 1:-1] - c) + np.abs(F[:-2, 1:-1] - c)
                + np.abs(F[1:-1, 2:] - c) + np.abs(F[1:-1, :-2] - c))
    out = np.zeros(fs.shape, np.float32)
    out[1:-1, 1:-1] = jump(fs) + jump(fe)
    return out


def qcalc_plane(x_end, y_end, z_end, flag_end, x_start, y_start, z_start, flag_start,
                Bx_in, By_in, Bz_in, Bx_out, By_out, Bz_out, Bx_0, By_0, Bz_0, B_flag,
                stride_step, cross_dir=(0.0, 0.0, 1.0)):
    """Q on the interior pixels of a 2-D seed grid.  Arrays are 2-D (n0, n1);
    returns (n0-2, n1-2) float32.  The flux ratio uses the z components of B
    at the two footpoints whatever their exit faces, as the reference does."""
    X1, Y1 = face_coords(x_start, y_start, z_start, flag_start)
    X2, Y2 = face_coords(x_end, y_end, z_end, flag_end)
    nan_arr = _flag_jump(flag_start, flag_end)
    a, b, c, d = _jacobian_terms(X1, Y1, X2, Y2)
    cd = np.asarray(cross_dir, dtype=np.float32)
    B_norm = Bx_0 * cd[0] + By_0 * cd[1] + Bz_0 * cd[2]
    bnr = np.abs(Bz_in[1:-1, 1:-1]) / (np.abs(B_norm[1:-1, 1:-1]) ** 2) * np.abs(Bz_out[1:-1, 1:-1]) * (
        (1. / (2. * stride_step)) ** 4.)
    with np.errstate(all="ignore"):
        Q = (a ** 2 + b ** 2 + c ** 2 + d ** 2) * bnr
    Q[Q < 1.0] = 1.0
    Q[nan_arr[1:-1, 1:-1] > 0] = np.nan
    return Q


def qcalc_plane_f64(x_end, y_end, z_end, flag_end, x_start, y_start, z_start, flag_start,
                    Bz_in, Bz_out, B_norm, stride_step):
    """FP64 version of qcalc_plane (footpoint differences, Jacobian norm and
    flux ratio in float64)."""
    f = lambda a: np.asarray(a, np.float64)  # noqa: E731
    X1, Y1 = face_coords(f(x_start), f(y_start), f(z_start), flag_start)
    X2, Y2 = face_coords(f(x_end), f(y_end), f(z_end), flag_end)
    X1, Y1, X2, Y2 = (np.where((fl - 1) // 2 >= 0, A, 0.0) for A, fl in
                      ((X1, flag_start), (Y1, flag_start), (X2, flag_end), (Y2, flag_end)))
    nan_arr = _flag_jump(flag_start, flag_end)
    a, b, c, d = _jacobian_terms(f(X1), f(Y1), f(X2), f(Y2))
    bnr = np.abs(f(Bz_in)[1:-1, 1:-1]) / (np.abs(f(B_norm)[1:-1, 1:-1]) ** 2) * np.abs(f(Bz_out)[1:-1, 1:-1]) * (
        (1. / (2. * stride_step)) ** 4.)
    with np.errstate(all="ignore"):
        Q = (a ** 2 + b ** 2 + c ** 2 + d ** 2) * bnr
    Q[Q < 1.0] = 1.0
    Q[nan_arr[1:-1, 1:-1] > 0] = np.nan
    return Q


def cook_pseudo_line(x_start, y_start, z_start, flag_start, Bz_in, Bz_out, B_flag, stride):
    """Pseudo-line seeds for the pixels with B_flag == 1 (FastQSL.py:10-49):
    four seeds per pixel around its START footpoint, offset by +-stride along
    the two axes of the start face, ordered (+u, +v, -u, -v) with (u, v) =
    (x, y) on a z-face, (x, z) on a y-face, (y, z) on an x-face.  Returns the
    three seed arrays and Bz at the start and end footpoints of the flagged
    pixels (flattened in row-major order)."""
    m = B_flag == 1
    xs, ys, zs = x_start[m], y_start[m], z_start[m]
    fs = flag_start[m]
    k = xs.shape[0]
    cx = np.repeat(xs, 4).astype(np.float32)
    cy = np.repeat(ys, 4).astype(np.float32)
    cz = np.repeat(zs, 4).astype(np.float32)
    dim = (fs - 1) // 2
    s = np.float32(stride)
    seed = {"x": cx, "y": cy, "z": cz}
    src = {"x": xs, "y": ys, "z": zs}
    for face, (u, v) in ((2, ("x", "y")), (1, ("x", "z")), (0, ("y", "z"))):
        sel = np.nonzero(dim == face)[0]
        seed[u][sel * 4 + 0] = src[u][sel] + s
        seed[u][sel * 4 + 2] = src[u][sel] - s
        seed[v][sel * 4 + 1] = src[v][sel] + s
        seed[v][sel * 4 + 3] = src[v][sel] - s
    assert cx.shape[0] == 4 * k
    return cx, cy, cz, Bz_in[m], Bz_out[m]


def qcut(start_x, start_y, start_z, flag_start, end_x, end_y, end_z, flag_end, Bz0_start, Bz0_end, stride):
    """Q of each flagged pixel from its 4 pseudo-lines (Q_RKF45CuPy.ipynb cell
    10): Jacobian terms from the differences of pseudo-lines (0, 2) and
    (1, 3), flux ratio |Bz_end| / |Bz_start| of the original line, clamp >= 1."""
    X1, Y1 = face_coords(start_x, start_y, start_z, flag_start)
    X2, Y2 = face_coords(end_x, end_y, end_z, flag_end)
    dx2xc = X2[0::4] - X2[2::4]
    dx2yc = X2[1::4] - X2[3::4]
    dy2xc = Y2[0::4] - Y2[2::4]
    dy2yc = Y2[1::4] - Y2[3::4]
    dx1xc = X1[0::4] - X1[2::4]
    dx1yc = X1[1::4] - X1[3::4]
    dy1xc = Y1[0::4] - Y1[2::4]
    dy1yc = Y1[1::4] - Y1[3::4]
    a = dx2xc * dy1yc - dx2yc * dy1xc
    b = dx2yc * dx1xc - dx2xc * dx1yc
    c = dy2xc * dy1yc - dy2yc * dy1xc
    d = dy2yc * dx1xc - dy2xc * dx1yc
    s = np.float32(stride)
    with np.errstate(all="ignore"):
        bnr = np.abs(Bz0_end) / (np.abs(Bz0_start)) * ((1 / s / 2) ** 4)
        Q = (a ** 2 + b ** 2 + c ** 2 + d ** 2) * bnr
    Q[Q < 1.0] = 1.0
    return Q


def merge(Q, Qcut, B_flag):
    """Q_all with the interior from qcalc_plane and every flagged pixel
    replaced by its pseudo-line Q; returns (Q_all, Q_all[1:-1, 1:-1])
    (Q_RKF45CuPy.ipynb cell 11)."""
    Q_all = np.zeros(B_flag.shape, np.float32)
    Q_all[1:-1, 1:-1] = Q
    Q_all[B_flag == 1] = Qcut
    return Q_all, Q_all[1:-1, 1:-1]


def qcut_f64(start_x, start_y, start_z, flag_start, end_x, end_y, end_z, flag_end, Bz0_start, Bz0_end, stride):
    """qcut in float64."""
    f = lambda a: np.asarray(a, np.float64)  # noqa: E731
    X1, Y1 = face_coords(f(start_x), f(start_y), f(start_z), flag_start)
    X2, Y2 = face_coords(f(end_x), f(end_y), f(end_z), flag_end)
    X1, Y1, X2, Y2 = (f(A) for A in (X1, Y1, X2, Y2))
    a = (X2[0::4] - X2[2::4]) * (Y1[1::4] - Y1[3::4]) - (X2[1::4] - X2[3::4]) * (Y1[0::4] - Y1[2::4])
    b = (X2[1::4] - X2[3::4]) * (X1[0::4] - X1[2::4]) - (X2[0::4] - X2[2::4]) * (X1[1::4] - X1[3::4])
    c = (Y2[0::4] - Y2[2::4]) * (Y1[1::4] - Y1[3::4]) - (Y2[1::4] - Y2[3::4]) * (Y1[0::4] - Y1[2::4])
    d = (Y2[1::4] - Y2[3::4]) * (X1[0::4] - X1[2::4]) - (Y2[0::4] - Y2[2::4]) * (X1[1::4] - X1[3::4])
    with np.errstate(all="ignore"):
        Q = (a * a + b * b + c * c + d * d) * (np.abs(f(Bz0_end)) / np.abs(f(Bz0_start))) * (
            (1.0 / (2.0 * float(stride))) ** 4)
    Q[Q < 1.0] = 1.0
    return Q


def qmap_pipeline(trace_fn, xs, ys, zs, nplanes, n0, n1, stride, cross_dir=(0.0, 0.0, 1.0), f64=True):
    """The whole Q-map workflow on stacked (n0, n1) planes, with pseudo-lines
    for the interior B_flag pixels only (the border ones are discarded by the
    reference's final crop).  trace_fn(xs, ys, zs) -> trace dict.  Returns Q of
    shape (nplanes, n0-2, n1-2) (float64 when f64)."""
    o = trace_fn(xs, ys, zs)
    shp = (nplanes, n0, n1)
    r = {k: np.asarray(v).reshape(shp) for k, v in o.items() if isinstance(v, np.ndarray) and v.size == xs.size}
    Qs = []
    cut_seeds = []
    meta = []
    for p in range(nplanes):
        g = {k: v[p] for k, v in r.items()}
        if f64:
            bn = (np.float64(g["B_this_x"]) * cross_dir[0] + np.float64(g["B_this_y"]) * cross_dir[1]
                  + np.float64(g["B_this_z"]) * cross_dir[2])
            Q = qcalc_plane_f64(g["end_x"], g["end_y"], g["end_z"], g["flag_end"], g["start_x"], g["start_y"],
                                g["start_z"], g["flag_start"], g["B_start_z"], g["B_end_z"], bn, stride)
        else:
            Q = qcalc_plane(g["end_x"], g["end_y"], g["end_z"], g["flag_end"], g["start_x"], g["start_y"],
                            g["start_z"], g["flag_start"], g["B_start_x"], g["B_start_y"], g["B_start_z"],
                            g["B_end_x"], g["B_end_y"], g["B_end_z"], g["B_this_x"], g["B_this_y"], g["B_this_z"],
                            g["B_flag"], stride, cross_dir)
        bf = g["B_flag"].copy()
        inner = np.zeros_like(bf)
        inner[1:-1, 1:-1] = 1
        bf = bf * inner
        cx, cy, cz, bzs, bze = cook_pseudo_line(g["start_x"], g["start_y"], g["start_z"], g["flag_start"],
                                                g["B_start_z"], g["B_end_z"], bf, np.float32(stride))
        cut_seeds.append((cx, cy, cz))
        meta.append((bf, bzs, bze))
        Qs.append(Q)
    allx = np.concatenate([c[0] for c in cut_seeds]) if cut_seeds else np.zeros(0, np.float32)
    ally = np.concatenate([c[1] for c in cut_seeds]) if cut_seeds else np.zeros(0, np.float32)
    allz = np.concatenate([c[2] for c in cut_seeds]) if cut_seeds else np.zeros(0, np.float32)
    if allx.size:
        s = trace_fn(allx, ally, allz)
    off = 0
    out = []
    for p in range(nplanes):
        bf, bzs, bze = meta[p]
        k = bzs.size
        Q = Qs[p]
        if k:
            sl = slice(4 * off, 4 * (off + k))
            fn = qcut_f64 if f64 else qcut
            Qc = fn(s["start_x"][sl], s["start_y"][sl], s["start_z"][sl], s["flag_start"][sl], s["end_x"][sl],
                    s["end_y"][sl], s["end_z"][sl], s["flag_end"][sl], bzs, bze, np.float32(stride))
            Qall = np.zeros(bf.shape, Q.dtype)
            Qall[1:-1, 1:-1] = Q
            Qall[bf == 1] = Qc
            Q = Qall[1:-1, 1:-1]
        off += k
        out.append(Q)
    return np.stack(out)


def hybrid_merge(Q, B_flag, q_perp):
    """Hybrid finite-difference + Scott Q of one plane (the crop of
    demo/Q_RKF45MixCuPyDiffScott.ipynb cell 9 to the interior pixels): Q of
    the interior pixels with B_flag set or Q NaN becomes q_perp of their seed.
    Q: (n0-2, n1-2); B_flag, q_perp: (n0, n1)."""
    bad = (B_flag[1:-1, 1:-1] != 0) | np.isnan(Q)
    out = np.array(Q, dtype=np.float64, copy=True)
    out[bad] = np.asarray(q_perp, np.float64)[1:-1, 1:-1][bad]
    return out


def qmap_hybrid(trace_fn, scott_fn, xs, ys, zs, nplanes, n0, n1, stride, cross_dir=(0.0, 0.0, 1.0)):
    """The hybrid Q-map workflow on stacked (n0, n1) planes: FP64 finite
    difference Q, then the Scott tracer (scott_fn(xs, ys, zs) -> dict with
    'q_perp') on the seeds of the interior pixels it cannot serve.  Returns
    (Q, n_selected)."""
    o = trace_fn(xs, ys, zs)
    shp = (nplanes, n0, n1)
    r = {k: np.asarray(v).reshape(shp) for k, v in o.items() if isinstance(v, np.ndarray) and v.size == xs.size}
    Qs, sel = [], []
    for p in range(nplanes):
        g = {k: v[p] for k, v in r.items()}
        bn = (np.float64(g["B_this_x"]) * cross_dir[0] + np.float64(g["B_this_y"]) * cross_dir[1]
              + np.float64(g["B_this_z"]) * cross_dir[2])
        Q = qcalc_plane_f64(g["end_x"], g["end_y"], g["end_z"], g["flag_end"], g["start_x"], g["start_y"],
                            g["start_z"], g["flag_start"], g["B_start_z"], g["B_end_z"], bn, stride)
        bad = np.zeros((n0, n1), bool)
        bad[1:-1, 1:-1] = (g["B_flag"][1:-1, 1:-1] != 0) | np.isnan(Q)
        Qs.append(Q)
        sel.append(np.flatnonzero(bad.ravel()) + p * n0 * n1)
    idx = np.concatenate(sel) if sel else np.zeros(0, np.int64)
    q_perp = np.full(nplanes * n0 * n1, np.nan, np.float32)
    if idx.size:
        q_perp[idx] = scott_fn(np.asarray(xs)[idx], np.asarray(ys)[idx], np.asarray(zs)[idx])["q_perp"]
    q_perp = q_perp.reshape(shp)
    return np.stack([hybrid_merge(Qs[p], r["B_flag"][p], q_perp[p]) for p in range(nplanes)]), int(idx.size)


def _diff3(C, a, axis):
    """Three-point non-uniform derivative at the interior nodes along `axis`
    (fastqslpy/FastQSL.py:143-163), in the arrays' float32 arithmetic."""
    a = np.asarray(a, np.float32)
    d = a[1:] - a[:-1]
    shape = [1, 1, 1]
    shape[axis] = -1
    dl, dr = d[:-1].reshape(shape), d[1:].reshape(shape)
    n = C.shape[axis]

    def take(lo, hi):
        s = [slice(1, -1)] * 3
        s[axis] = slice(lo, hi)
        return C[tuple(s)]
    c0, cp, cm = take(1, n - 1), take(2, n), take(0, n - 2)
    return (cp - c0) / dr * dl / (dr + dl) + (c0 - cm) / dl * dr / (dr + dl)


def curl_grid(Bx, By, Bz, xa, ya, za):
    """curl B with the reference's boundary copy (FastQSL.py:120-141);
    float64 arrays of the field's shape."""
    Bx, By, Bz = (np.asarray(b, np.float32) for b in (Bx, By, Bz))
    out = [np.zeros(Bx.shape) for _ in range(3)]
    out[0][1:-1, 1:-1, 1:-1] = _diff3(Bz, ya, 1) - _diff3(By, za, 2)
    out[1][1:-1, 1:-1, 1:-1] = _diff3(Bx, za, 2) - _diff3(Bz, xa, 0)
    out[2][1:-1, 1:-1, 1:-1] = _diff3(By, xa, 0) - _diff3(Bx, ya, 1)
    for a in out:
        a[:, :, 0] = a[:, :, 1]
        a[:, 0, :] = a[:, 1, :]
        a[0, :, :] = a[1, :, :]
        a[:, :, -1] = a[:, :, -2]
        a[:, -1, :] = a[:, -2, :]
        a[-1, :, :] = a[-2, :, :]
    return tuple(out)
