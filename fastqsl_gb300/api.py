"""Native Python API over the C ABI: resident field stores, tracing and the
on-device Q-map pipeline.

Buffers are PyTorch CUDA tensors (or any object exposing
``__cuda_array_interface__``); every computation runs in the CUDA kernels of
libfastqsl_gb300.so on the given (default: current) stream.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .params import TraceParams, absolute_rkf45

LAYOUTS = {"soa": 0, "f4": 1, "h4b": 2, "h8c": 3}
SCHEDULES = {"queue": 0, "static": 1}

TRACE_F32 = ["start_x", "start_y", "start_z", "end_x", "end_y", "end_z",
             "B_this_x", "B_this_y", "B_this_z", "B_start_x", "B_start_y", "B_start_z",
             "B_end_x", "B_end_y", "B_end_z"]
TRACE_I32 = ["flag_start", "flag_end", "B_flag"]
_TRACE_OUT = TRACE_F32 + TRACE_I32 + ["LineLen"]


def ptr(a):
    """Device address of a CUDA tensor / __cuda_array_interface__ array (an
    int is taken as an address already)."""
    if a is None or type(a) is int:
        return a
    if isinstance(a, torch.Tensor):
        if not a.is_cuda:
            raise ValueError("expected a CUDA tensor")
        return a.data_ptr()
    cai = getattr(a, "__cuda_array_interface__", None)
    if cai is not None:
        return int(cai["data"][0])
    raise TypeError(f"not a device array: {type(a)}")


def stream_handle(stream=None):
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, torch.cuda.Stream):
        return stream.cuda_stream
    return int(stream)


def as_xfast(a, device="cuda"):
    """A float32 CUDA tensor of shape (nx, ny, nz) with x fastest in memory
    (strides (1, nx, nx*ny)), copying only when needed."""
    t = a if isinstance(a, torch.Tensor) else torch.as_tensor(a)
    if t.dim() != 3:
        raise ValueError("field arrays must be 3-D (nx, ny, nz)")
    t = t.to(device=device, dtype=torch.float32)
    nx, ny, _ = t.shape
    if t.stride() != (1, nx, nx * ny):
        t = t.permute(2, 1, 0).contiguous().permute(2, 1, 0)
    return t


class FieldStore:
    """A field resident on the device in one of the GB300 layouts.

    layout: 'h4b' (fp16 8^3 bricks + per-brick scale, stored as x-pair
    records of 16 B, ~20 B per node: the fastest store and the default),
    'h8c' (fp16 cell records: each cell's 8 corners in 64 B), 'f4'
    (interleaved float4, float32 values) or 'soa' (the caller's float32
    arrays in place)."""

    def __init__(self, Bx, By, Bz, layout="h4b", stream=None):
        lib = _lib.load()
        if layout not in LAYOUTS:
            raise ValueError(f"layout must be one of {list(LAYOUTS)}")
        self.layout = layout
        arrs = [as_xfast(b) for b in (Bx, By, Bz)]
        if len({tuple(a.shape) for a in arrs}) != 1:
            raise ValueError("Bx, By, Bz must have the same shape")
        self.shape = tuple(int(s) for s in arrs[0].shape)
        self._keep = arrs if layout == "soa" else None
        h = ctypes.c_void_p()
        _lib.check(lib.qsl_field_create(ptr(arrs[0]), ptr(arrs[1]), ptr(arrs[2]), *self.shape, LAYOUTS[layout],
                                        stream_handle(stream), ctypes.byref(h)), "qsl_field_create")
        self._h = h
        self.nbytes = int(lib.qsl_field_bytes(h))
        if layout != "soa" and isinstance(stream, torch.cuda.Stream):
            # the conversion read the source arrays on `stream`; the caching
            # allocator may hand their memory to another stream once freed
            for a in arrs:
                a.record_stream(stream)

    def update(self, Bx, By, Bz, stream=None):
        """Refills the store from new arrays of the same shape (x fastest,
        float32, on the device) without reallocating."""
        arrs = [as_xfast(b) for b in (Bx, By, Bz)]
        if tuple(arrs[0].shape) != self.shape:
            raise ValueError("shape differs from the store's")
        if self.layout == "soa":
            self._keep = arrs
        _lib.check(_lib.load().qsl_field_update(self.handle, ptr(arrs[0]), ptr(arrs[1]), ptr(arrs[2]),
                                                stream_handle(stream)), "qsl_field_update")

    @staticmethod
    def store_bytes(shape, layout):
        return int(_lib.load().qsl_field_store_bytes(*shape, LAYOUTS[layout]))

    @property
    def handle(self):
        if self._h is None:
            raise ValueError("field store is closed")
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None:
            _lib.load().qsl_field_destroy(self._h)
            self._h = None
            self._keep = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class FieldUploader:
    """Double-buffered upload of host fields into a FieldStore: upload() puts
    the H2D copy of a field (pinned host arrays) on its own copy stream into
    one of `slots` device staging buffers, pack() makes the store's stream
    wait for that copy and refills the store from it.  Uploading field k+1
    before running field k's trace overlaps the copy with the trace; a slot
    is reused only after everything queued on the store's stream up to the
    following pack() (the pack, and the trace that read the field) is done.
    """

    def __init__(self, shape, device="cuda", slots=2):
        nx, ny, nz = (int(v) for v in shape)
        self.shape = (nx, ny, nz)
        self.device = torch.device(device)
        self.bufs = [[torch.empty((nz, ny, nx), dtype=torch.float32, device=self.device) for _ in range(3)]
                     for _ in range(max(2, int(slots)))]
        self.ready = [torch.cuda.Event() for _ in self.bufs]
        self.free = [None] * len(self.bufs)
        self.copy_stream = torch.cuda.Stream(device=self.device)
        self._next, self._last = 0, None

    def upload(self, Bx, By, Bz):
        """Queues the copy of one field (torch CPU tensors shaped (nz, ny, nx),
        contiguous, pinned for an asynchronous copy; or x-fastest arrays
        shaped (nx, ny, nz)); returns the slot to pass to pack()."""
        host = []
        for b in (Bx, By, Bz):
            t = b if isinstance(b, torch.Tensor) else torch.from_numpy(np.asarray(b))
            if tuple(t.shape) == self.shape and t.dim() == 3 and t.stride(0) == 1:
                t = t.permute(2, 1, 0)
            if tuple(t.shape) != self.shape[::-1] or not t.is_contiguous() or t.dtype != torch.float32:
                raise ValueError("each component must be float32, x fastest, of the uploader's shape")
            host.append(t)
        s = self._next
        self._next = (s + 1) % len(self.bufs)
        if self.free[s] is not None:
            self.copy_stream.wait_event(self.free[s])
        with torch.cuda.stream(self.copy_stream):
            for d, h in zip(self.bufs[s], host):
                d.copy_(h, non_blocking=True)
            self.ready[s].record(self.copy_stream)
        return s

    def pack(self, store: "FieldStore", slot, stream=None):
        """Refills `store` from an uploaded slot on `stream` (default: the
        current stream) once its copy has landed."""
        st = stream if isinstance(stream, torch.cuda.Stream) else torch.cuda.current_stream(self.device)
        if self._last is not None:
            ev = torch.cuda.Event()
            ev.record(st)
            self.free[self._last] = ev
        st.wait_event(self.ready[slot])
        with torch.cuda.stream(st):
            store.update(*[d.permute(2, 1, 0) for d in self.bufs[slot]], stream=st)
        self._last = slot


_ESIZE = {torch.float32: 4, torch.float64: 8, torch.int32: 4, torch.int64: 8, torch.uint8: 1}


def _layout(parts):
    """Byte offsets of parts = [(name, numel, dtype)] packed on 256-byte
    boundaries, and the total."""
    offs, total = {}, 0
    for name, n, dt in parts:
        offs[name] = total
        total += (int(n) * _ESIZE[dt] + 255) // 256 * 256
    return offs, max(total, 256)


def carve(parts, device="cuda"):
    """One device allocation split into tensors: parts = [(name, numel,
    dtype)], each starting on a 256-byte boundary, uninitialised.  Returns
    ({name: tensor}, backing uint8 tensor)."""
    offs, total = _layout(parts)
    buf = torch.empty(total, dtype=torch.uint8, device=device)
    out = {name: buf[offs[name]:offs[name] + int(n) * _ESIZE[dt]].view(dt) for name, n, dt in parts}
    return out, buf


def trace_output_parts(n, twist=False, status=False, prefix=""):
    """carve() parts of the per-seed outputs of a trace."""
    parts = [(prefix + k, n, torch.float32) for k in TRACE_F32] + [(prefix + k, n, torch.int32) for k in TRACE_I32]
    parts.append((prefix + "LineLen", n, torch.float64))
    if twist:
        parts.append((prefix + "twist", n, torch.float64))
    if status:
        parts += [(prefix + "status_start", n, torch.int32), (prefix + "status_end", n, torch.int32)]
    return parts


def alloc_trace_outputs(n, device="cuda", twist=False, status=False, zero=True):
    """The per-seed output arrays of a trace, views of one allocation
    (zeroed by one memset unless zero=False: a trace writes every output of
    each of its n lines).  status=True adds int32 'status_start' /
    'status_end' (qsl_line_status of each direction: params.LINE_FACE ...
    LINE_REJECT_LIMIT)."""
    out, buf = carve(trace_output_parts(n, twist, status), device)
    if zero:
        buf.zero_()
    out.setdefault("twist", None)
    return out


def _io(xs, ys, zs, out):
    io = _lib.TraceIO()
    io.inp_x, io.inp_y, io.inp_z = ptr(xs), ptr(ys), ptr(zs)
    for k in TRACE_F32 + TRACE_I32 + ["LineLen"]:
        setattr(io, k, ptr(out[k]))
    io.twist = ptr(out.get("twist"))
    io.status_start = ptr(out.get("status_start"))
    io.status_end = ptr(out.get("status_end"))
    return io


def trace(field: FieldStore, xs, ys, zs, params: TraceParams | None = None, s_len=0.125, tol_coef=1.0,
          cross_dir=(0.0, 0.0, 1.0), curB=None, schedule="queue", out=None, n=None, n_dev=None, samples=None,
          queue=None, order=None, chunk=0, occupancy=0, stream=None, status=False):
    """Traces every seed (xs, ys, zs: float32 CUDA vectors) both ways.
    Returns the output dict (allocated unless `out` is given).  `n_dev`: a
    device counter holding the seed count (outputs must then hold the largest
    count).  `samples`: optional int64 CUDA tensor accumulating the number of
    trilinear samples taken.  `order`: optional int32 permutation; line k
    traces seed order[k] (see tile_order).  `chunk`: lines per warp refill.
    `curB`: the current density for the twist integral, as three x-fastest
    float32 device arrays or as a FieldStore of the field's layout and shape
    (qsl_trace_cur: each current sample costs a field sample).  `status`:
    also return each direction's qsl_line_status ('status_start',
    'status_end'; with `out` given, it is written when `out` holds them)."""
    lib = _lib.load()
    if params is None:
        params = absolute_rkf45()
    n = int(xs.shape[0]) if n is None else int(n)
    if out is None:
        out = alloc_trace_outputs(n, xs.device, twist=curB is not None, status=status)
    cd = (ctypes.c_float * 3)(*[float(c) for c in cross_dir])
    if curB is not None and out.get("twist") is None:
        out["twist"] = torch.zeros(out["LineLen"].shape[0], dtype=torch.float64, device=xs.device)
    io = _io(xs, ys, zs, out)
    sc = _lib.Sched(SCHEDULES[schedule], int(chunk), ptr(order), ptr(queue), ptr(samples), int(occupancy))
    if isinstance(curB, FieldStore):
        _lib.check(lib.qsl_trace_cur(field.handle, curB.handle, ctypes.byref(params), ctypes.byref(io), n,
                                     ptr(n_dev), float(s_len), float(tol_coef), cd, ctypes.byref(sc),
                                     stream_handle(stream)), "qsl_trace_cur")
        return out
    cur = [ptr(c) for c in curB] if curB is not None else [None, None, None]
    _lib.check(lib.qsl_trace(field.handle, ctypes.byref(params), ctypes.byref(io), n, ptr(n_dev),
                             float(s_len), float(tol_coef), cd, *cur, ctypes.byref(sc), stream_handle(stream)),
               "qsl_trace")
    return out


def trace_stretch(Bx, By, Bz, coords, xs, ys, zs, params: TraceParams | None = None, s_len=0.01, tol_coef=1.0,
                  uni=False, cross_dir=(0.0, 0.0, 1.0), curB=None, schedule="static", out=None, samples=None,
                  order=None, occupancy=0, stream=None):
    """Traces every seed both ways on a stretched grid: Bx, By, Bz of shape
    (nx, ny, nz) (x fastest; moved to the device if needed and read in place),
    coords = (x_arr, y_arr, z_arr) increasing node coordinates, seeds in the
    same physical coordinates (float32 CUDA vectors).  uni: index cells by the
    uniform-spacing formula instead of the search.  occupancy: resident-block
    variant of the fast kernels (4, 5 or 6 blocks per SM; 0 or 7-10 take the
    default, 5).
    Fast arithmetic traces a copy of the nodes as x-pair records and finds
    cells through per-axis search tables, both built for the launch; the
    results equal the drop-in's bit for bit.  Defaults to the reference
    stretched kernel's settings (TraceBlineAdaptiveStretch.cu)."""
    from .params import reference_stretch
    # the native entry takes the coordinates on the host (the per-axis
    # constants of the cell location are formed there); device arrays are
    # copied back first
    ax = []
    for c in coords:
        a = c.detach().cpu().numpy() if isinstance(c, torch.Tensor) else np.asarray(c)
        # checked on the float32 values the kernels use: two distinct doubles
        # can round to one float
        a = np.ascontiguousarray(np.asarray(a, dtype=np.float64).astype(np.float32))
        if a.ndim != 1 or a.size < 2 or not np.all(np.diff(a) > 0):
            raise ValueError("each coordinate array must be 1-D, with at least 2 strictly increasing entries "
                             "(as float32)")
        ax.append(a)
    lib = _lib.load()
    if params is None:
        params = reference_stretch()
    arrs = [as_xfast(b) for b in (Bx, By, Bz)]
    nx, ny, nz = (int(v) for v in arrs[0].shape)
    if [a.size for a in ax] != [nx, ny, nz]:
        raise ValueError("coordinate arrays must have nx, ny, nz entries")
    n = int(xs.shape[0])
    if out is None:
        out = alloc_trace_outputs(n, xs.device, twist=curB is not None)
    cd = (ctypes.c_float * 3)(*[float(c) for c in cross_dir])
    curs = [as_xfast(c) for c in curB] if curB is not None else None
    cur = [ptr(c) for c in curs] if curs is not None else [None, None, None]
    if curB is not None and out.get("twist") is None:
        out["twist"] = torch.zeros(n, dtype=torch.float64, device=xs.device)
    io = _io(xs, ys, zs, out)
    sc = _lib.Sched(SCHEDULES[schedule], 0, ptr(order), None, ptr(samples), int(occupancy))
    _lib.check(lib.qsl_trace_stretch(*[ptr(a) for a in arrs], nx, ny, nz,
                                     *[a.ctypes.data_as(ctypes.c_void_p) for a in ax], int(bool(uni)),
                                     ctypes.byref(params), ctypes.byref(io), n, float(s_len), float(tol_coef), cd,
                                     *cur, ctypes.byref(sc), stream_handle(stream)), "qsl_trace_stretch")
    return out


def tile_order(nplanes, n0, n1, ty=16, tx=16, device="cuda", plane_group=None, stream=None):
    """A permutation of the seeds of `nplanes` stacked (n0, n1) planes that
    visits them tile by tile (ty x tx seeds, row-major inside a tile), as
    int32 on the device.  Neighbouring seeds start neighbouring field lines,
    so a warp given consecutive lines of this order gathers from a compact
    patch of the field.  Tiles go column by column: each (y, x) tile is
    visited in `plane_group` consecutive planes before the next tile (default:
    all planes; 1 = plane by plane), so the blocks resident at a time trace
    the lines through a few thin columns of the stack rather than through
    whole planes, and share more of L1 and L2 (the benchmark cube's main
    trace: 57.9 ms against 62.2 ms plane by plane).  One launch
    (qsl_tile_order) on `stream` (default: the current stream)."""
    g = int(nplanes if plane_group is None else max(1, plane_group))
    out = torch.empty(int(nplanes) * int(n0) * int(n1), dtype=torch.int32, device=device)
    _lib.check(_lib.load().qsl_tile_order(int(nplanes), int(n0), int(n1), int(ty), int(tx), g, out.data_ptr(),
                                          stream_handle(stream)), "qsl_tile_order")
    return out


_D3 = ctypes.c_double * 3


def plane_seeds(center, normal, u, v, spacing, n0, n1, nplanes=1, device="cuda", stream=None):
    """Seeds of `nplanes` stacked (n0, n1) planes centred on `center`, rows
    along v, columns along u, planes stepping along `normal`, `spacing`
    apart (qsl_plane_seeds: one launch): seed (k, i, j) at ((center + k s
    normal) + (i - (n0-1)/2) s v) + (j - (n1-1)/2) s u in double, rounded
    to float32.  Returns xs, ys, zs (views of one allocation)."""
    total = int(n0) * int(n1) * int(nplanes)
    buf = torch.empty((3, total), dtype=torch.float32, device=device)
    base = buf.data_ptr()
    _lib.check(_lib.load().qsl_plane_seeds(_D3(*center), _D3(*normal), _D3(*u), _D3(*v), float(spacing), int(n0),
                                           int(n1), int(nplanes), base, base + 4 * total, base + 8 * total,
                                           stream_handle(stream)), "qsl_plane_seeds")
    return buf.unbind(0)


SCOTT_F32 = ["start_x", "start_y", "start_z", "end_x", "end_y", "end_z", "B_this_x", "B_this_y", "B_this_z",
             "q_0", "q_perp"]
GRAD_MODES = {"fd": 0, "analytic": 1}


def alloc_scott_outputs(n, device="cuda", twist=False):
    out = {k: torch.zeros(n, dtype=torch.float32, device=device) for k in SCOTT_F32}
    out["flag_start"] = torch.zeros(n, dtype=torch.int32, device=device)
    out["flag_end"] = torch.zeros(n, dtype=torch.int32, device=device)
    out["LineLen"] = torch.zeros(n, dtype=torch.float64, device=device)
    out["twist"] = torch.zeros(n, dtype=torch.float64, device=device) if twist else None
    return out


def trace_scott(field: FieldStore, xs, ys, zs, params: TraceParams | None = None, s_len=0.25, tol_coef=1.0,
                curB=None, grad="analytic", out=None, n=None, n_dev=None, samples=None, order=None, stream=None):
    """Scott deviation-vector tracer: footpoints, flags, q_0 and q_perp per
    seed (reference: fastqslpy/cu/TraceBlineScott.cu:334-595).  grad:
    'fd' (the reference's central differences) or 'analytic' (exact
    trilinear derivative, fast arithmetic only)."""
    from .params import reference_scott, ARITH_FAST
    lib = _lib.load()
    if params is None:
        params = reference_scott(arith=ARITH_FAST)
    n = int(xs.shape[0]) if n is None else int(n)
    if out is None:
        out = alloc_scott_outputs(n, xs.device, twist=curB is not None)
    if curB is not None and out.get("twist") is None:
        out["twist"] = torch.zeros(out["LineLen"].shape[0], dtype=torch.float64, device=xs.device)
    io = _lib.ScottIO()
    io.inp_x, io.inp_y, io.inp_z = ptr(xs), ptr(ys), ptr(zs)
    for k in SCOTT_F32 + ["flag_start", "flag_end", "LineLen"]:
        setattr(io, k, ptr(out[k]))
    io.twist = ptr(out.get("twist"))
    cur = [ptr(c) for c in curB] if curB is not None else [None, None, None]
    sc = _lib.Sched(SCHEDULES["static"], 0, ptr(order), None, ptr(samples), 0)
    _lib.check(lib.qsl_trace_scott(field.handle, ctypes.byref(params), ctypes.byref(io), n, ptr(n_dev),
                                   float(s_len), float(tol_coef), *cur, GRAD_MODES[grad], ctypes.byref(sc),
                                   stream_handle(stream)), "qsl_trace_scott")
    return out


class QMapPlan:
    """Device buffers and launch sequence of the Q pipeline for `nplanes`
    stacked (n0, n1) seed planes (rows along y, columns along x):

    trace all seeds -> Q on interior pixels (FP64 Jacobian norm and flux
    ratio) -> compact the B_flag pixels -> trace their 4 pseudo-lines -> Q of
    those pixels -> merge.  The main trace visits the seeds in `tile` order
    with lanes in lockstep (`schedule`='static'): a warp's lanes start on
    neighbouring seeds and advance together, so their gathers stay on a
    compact patch of the field.  No host synchronisation inside; the pseudo-line
    trace reads its seed count from the device, so a whole run can be
    captured in a CUDA graph.  Outputs Q of shape (nplanes, n0-2, n1-2)
    (float64).  Reference workflow: demo/Q_RKF45CuPy3D.ipynb cell 7 and
    demo/Q_RKF45CuPy.ipynb cells 7-11."""

    # measured best per field layout on GB300 (trace of the 512x512x256 cube):
    # register budget for 7 resident blocks/SM for the brick store (FP32
    # interpolation), 8 for the cell-record and float4 stores, the compiler's
    # choice for SoA
    DEFAULT_OCCUPANCY = {"h8c": 8, "h4b": 7, "f4": 8, "soa": 0}

    def __init__(self, n0, n1, nplanes=1, device="cuda", pseudo=True, tile=(8, 8), chunk=256, schedule="static",
                 occupancy=None, hybrid=False):
        """hybrid: instead of the pseudo-line pass, the interior pixels with
        B_flag set or a NaN finite-difference Q take the Scott tracer's
        q_perp (demo/Q_RKF45MixCuPyDiffScott.ipynb cell 9)."""
        self.n0, self.n1, self.nplanes = int(n0), int(n1), int(nplanes)
        self.hybrid = bool(hybrid)
        if self.hybrid:
            pseudo = False
        if self.n0 < 3 or self.n1 < 3:
            raise ValueError("planes must be at least 3 x 3 seeds")
        self.n = self.n0 * self.n1 * self.nplanes
        self.device = device
        self.pseudo = pseudo
        self.schedule = schedule
        self.chunk = int(chunk)
        self.occupancy = occupancy  # None: per-layout default at run time
        self.order = tile_order(self.nplanes, self.n0, self.n1, tile[0], tile[1], device) if tile else None
        self.main = alloc_trace_outputs(self.n, device)
        self.Q = torch.empty((self.nplanes, self.n0 - 2, self.n1 - 2), dtype=torch.float64, device=device)
        self._side = None  # side stream of the Q assembly (created at the first run)
        self.queue = torch.zeros(2, dtype=torch.int64, device=device)
        self.samples_buf = torch.zeros(2, dtype=torch.int64, device=device)  # main, pseudo-line trace
        if pseudo:
            m = self.nplanes * (self.n0 - 2) * (self.n1 - 2)  # at most every interior pixel
            self.max_pix = m
            self.cut = [torch.empty(4 * m, dtype=torch.float32, device=device) for _ in range(3)]
            self.bz0s = torch.empty(m, dtype=torch.float32, device=device)
            self.bz0e = torch.empty(m, dtype=torch.float32, device=device)
            self.pix = torch.empty(m, dtype=torch.int64, device=device)
            self.count = torch.zeros(2, dtype=torch.int64, device=device)
            wb = int(_lib.load().qsl_cook_workspace_bytes(self.n))
            self.work = torch.empty((wb + 7) // 8, dtype=torch.int64, device=device)
            self.work_bytes = wb
            self.sub = alloc_trace_outputs(4 * m, device)
            self.qcut = torch.empty(m, dtype=torch.float64, device=device)
        if self.hybrid:
            m = self.nplanes * (self.n0 - 2) * (self.n1 - 2)
            self.max_pix = m
            self.hseeds = torch.empty(m, dtype=torch.int32, device=device)
            self.hcount = torch.zeros(1, dtype=torch.int64, device=device)
            self.scott = alloc_scott_outputs(self.n, device)

    def occupancy_for(self, field):
        if self.occupancy is not None:
            return int(self.occupancy)
        return self.DEFAULT_OCCUPANCY.get(field.layout, 0)

    @property
    def samples_main(self):
        return self.samples_buf[0]

    @property
    def samples(self):
        return self.samples_buf.sum()

    @property
    def twist_map(self):
        """Twist number of every seed line of the last run with a current
        density, shape (nplanes, n0, n1) (None before such a run)."""
        t = self.main.get("twist")
        return None if t is None else t.view(self.nplanes, self.n0, self.n1)

    def run(self, field, xs, ys, zs, params=None, s_len=0.125, tol_coef=1.0, stride=1.0, cross_dir=(0.0, 0.0, 1.0),
            pseudo_tol_factor=1.0, count_samples=False, kernel_events=None, stream=None, scott_params=None,
            scott_grad="analytic", curB=None):
        """Runs the pipeline; `kernel_events` (start, end) CUDA events are
        recorded around the main trace launch when given.  scott_params /
        scott_grad: the Scott pass of a hybrid plan (default: the Scott
        tracer's reference settings in fast arithmetic with the main trace's
        tolerance and step bounds).  curB: the current density (three arrays
        or a FieldStore of the field's layout); the main trace then also
        integrates each seed's twist number (`twist_map`)."""
        lib = _lib.load()
        st = stream_handle(stream)
        if params is None:
            params = absolute_rkf45()
        if count_samples:
            self.samples_buf.zero_()
        m = self.main
        if curB is not None and m.get("twist") is None:
            m["twist"] = torch.zeros(self.n, dtype=torch.float64, device=m["LineLen"].device)
        ev_stream = stream if isinstance(stream, torch.cuda.Stream) else torch.cuda.current_stream()
        if kernel_events is not None:
            kernel_events[0].record(ev_stream)
        trace(field, xs, ys, zs, params, s_len, tol_coef, cross_dir, curB=curB, out=m, n=self.n,
              samples=self.samples_buf[0:1] if count_samples else None, queue=self.queue, order=self.order,
              chunk=self.chunk, schedule=self.schedule, occupancy=self.occupancy_for(field), stream=stream)
        if kernel_events is not None:
            kernel_events[1].record(ev_stream)
        jac = (1.0 / (2.0 * float(stride))) ** 4.0
        cd = (ctypes.c_float * 3)(*[float(c) for c in cross_dir])
        def qcalc(qst):
            _lib.check(lib.qsl_qcalc_plane(ptr(m["end_x"]), ptr(m["end_y"]), ptr(m["end_z"]), ptr(m["flag_end"]),
                                           ptr(m["start_x"]), ptr(m["start_y"]), ptr(m["start_z"]),
                                           ptr(m["flag_start"]), ptr(m["B_start_z"]), ptr(m["B_end_z"]),
                                           ptr(m["B_this_x"]), ptr(m["B_this_y"]), ptr(m["B_this_z"]), self.n0,
                                           self.n1, self.nplanes, jac, cd, None, ptr(self.Q), qst), "qsl_qcalc_plane")

        # with pseudo-lines the Q assembly of all pixels runs on a side stream
        # beside the pseudo-line trace (both depend only on the main trace and
        # the compaction), launched after it so that the trace's blocks are
        # dispatched first and the assembly fills the SMs its few long lines
        # leave idle; the merge waits for it
        overlap = self.pseudo and not self.hybrid and (stream is None or isinstance(stream, torch.cuda.Stream))
        if not overlap:
            qcalc(st)
        if self.hybrid:
            return self._hybrid(field, xs, ys, zs, params, s_len, tol_coef, scott_params, scott_grad, stream, st)
        if not self.pseudo:
            return self.Q
        _lib.check(lib.qsl_cook_pseudo_line(ptr(m["B_flag"]), ptr(m["start_x"]), ptr(m["start_y"]),
                                            ptr(m["start_z"]), ptr(m["flag_start"]), ptr(m["B_start_z"]),
                                            ptr(m["B_end_z"]), self.n, self.n0, self.n1, 1, float(stride),
                                            ptr(self.cut[0]), ptr(self.cut[1]), ptr(self.cut[2]), ptr(self.bz0s),
                                            ptr(self.bz0e), ptr(self.pix), ptr(self.count), ptr(self.work),
                                            self.work_bytes, st), "qsl_cook_pseudo_line")
        cnt_seeds = self.count[1:2]
        if overlap:
            fork = torch.cuda.Event()
            fork.record(ev_stream)
        trace(field, self.cut[0], self.cut[1], self.cut[2], params, s_len, tol_coef * pseudo_tol_factor, cross_dir,
              out=self.sub, n=4 * self.max_pix, n_dev=cnt_seeds, schedule="static",
              occupancy=self.occupancy_for(field),
              samples=self.samples_buf[1:2] if count_samples else None, queue=self.queue[1:2],
              stream=stream)
        if overlap:
            if self._side is None:
                self._side = torch.cuda.Stream(device=self.Q.device)
            self._side.wait_event(fork)
            qcalc(self._side.cuda_stream)
            qdone = torch.cuda.Event()
            qdone.record(self._side)
        s = self.sub
        _lib.check(lib.qsl_qcut(ptr(s["start_x"]), ptr(s["start_y"]), ptr(s["start_z"]), ptr(s["flag_start"]),
                                ptr(s["end_x"]), ptr(s["end_y"]), ptr(s["end_z"]), ptr(s["flag_end"]),
                                ptr(self.bz0s), ptr(self.bz0e), 0, ptr(self.count[0:1]), self.max_pix, jac, None,
                                ptr(self.qcut), st), "qsl_qcut")
        if overlap:
            ev_stream.wait_event(qdone)
        _lib.check(lib.qsl_qmerge(ptr(self.pix), None, ptr(self.qcut), 0, ptr(self.count[0:1]), self.max_pix,
                                  self.n0, self.n1, None, ptr(self.Q), st), "qsl_qmerge")
        return self.Q


def _hybrid_impl(self, field, xs, ys, zs, params, s_len, tol_coef, scott_params, scott_grad, stream, st):
    """Select -> Scott on the selected seeds (count and order on the device)
    -> merge q_perp into Q."""
    from .params import reference_scott
    lib = _lib.load()
    m = self.main
    if scott_params is None:
        scott_params = reference_scott(arith=params.arith).copy(tol=params.tol, h_min=params.h_min,
                                                                h_max=params.h_max)
    _lib.check(lib.qsl_hybrid_select(ptr(m["B_flag"]), ptr(self.Q), self.n0, self.n1, self.nplanes,
                                     ptr(self.hseeds), ptr(self.hcount), st), "qsl_hybrid_select")
    trace_scott(field, xs, ys, zs, scott_params, s_len, tol_coef, grad=scott_grad, out=self.scott, n=self.max_pix,
                n_dev=self.hcount, order=self.hseeds, stream=stream)
    _lib.check(lib.qsl_hybrid_merge(ptr(m["B_flag"]), ptr(self.scott["q_perp"]), self.n0, self.n1, self.nplanes,
                                    ptr(self.Q), st), "qsl_hybrid_merge")
    return self.Q


QMapPlan._hybrid = _hybrid_impl


class PlaneQBatch:
    """Q maps of many plane jobs as one native batch (qsl_qmap_batch_*): the
    seed grids, tile orders, job tables, batched traces and the batched Q
    assembly are laid out in one workspace allocation and queued by the C++
    library: two launches per job (seed grid, tile order), then the batch's
    traces and six Q-assembly launches for all jobs, and no per-array host
    bookkeeping.  The Q maps equal QBatch's on the same jobs bit for bit (the
    same trace kernels; the Q-assembly kernels' arithmetic per pixel).  Reference workflow per job: demo/Q_RKF45CuPy.ipynb
    cells 7-11.

    jobs: list of dicts with keys field (FieldStore), params, center, normal,
    u, v (unit plane axes: columns along u, rows along v), spacing, n0, n1,
    nplanes and optionally s_len (0.25), tol_coef (1.0).  tile: the seed tile
    of the trace order (None: seed order).  blocks_per_sm > 0: the batched
    traces keep at most that many resident blocks per SM.  The object owns
    the workspace and the pinned staging buffer its queued work reads: keep
    it alive until that work has completed (an event after run_post)."""

    def __init__(self, jobs, device="cuda", tile=(8, 8), stream=None, blocks_per_sm=0):
        lib = _lib.load()
        self.max_blocks = 0
        if blocks_per_sm:
            sms = ctypes.c_int(0)
            _lib.check(lib.qsl_device_sm_count(ctypes.byref(sms)), "qsl_device_sm_count")
            self.max_blocks = int(blocks_per_sm) * sms.value
        self.njobs = len(jobs)
        arr = (_lib.QmapJob * max(1, self.njobs))()
        ty, tx = (int(tile[0]), int(tile[1])) if tile else (0, 0)
        for k, j in enumerate(jobs):
            a = arr[k]
            a.field = j["field"].handle
            a.params = j["params"]
            a.center[:] = [float(c) for c in j["center"]]
            a.normal[:] = [float(c) for c in j["normal"]]
            a.u[:] = [float(c) for c in j["u"]]
            a.v[:] = [float(c) for c in j["v"]]
            a.spacing = float(j["spacing"])
            a.n0, a.n1, a.nplanes = int(j["n0"]), int(j["n1"]), int(j.get("nplanes", 1))
            a.tile_y, a.tile_x = ty, tx
            a.s_len = float(j.get("s_len", 0.25))
            a.tol_coef = float(j.get("tol_coef", 1.0))
        db, hb = ctypes.c_int64(0), ctypes.c_int64(0)
        _lib.check(lib.qsl_qmap_batch_size(arr, self.njobs, ctypes.byref(db), ctypes.byref(hb)), "qsl_qmap_batch_size")
        self.workspace = torch.empty(max(256, db.value), dtype=torch.uint8, device=device)
        self._host = torch.empty(max(256, hb.value), dtype=torch.uint8, pin_memory=True)
        h = ctypes.c_void_p()
        _lib.check(lib.qsl_qmap_batch_create(arr, self.njobs, self.workspace.data_ptr(), db.value,
                                             self._host.data_ptr(), hb.value, stream_handle(stream), ctypes.byref(h)),
                   "qsl_qmap_batch_create")
        self.handle = h
        base = self.workspace.data_ptr()
        self.Q = []
        for k, j in enumerate(jobs):
            off = int(lib.qsl_qmap_batch_q(h, k)) - base
            n0, n1, npl = int(j["n0"]), int(j["n1"]), int(j.get("nplanes", 1))
            qn = npl * (n0 - 2) * (n1 - 2)
            self.Q.append(self.workspace[off:off + 8 * qn].view(torch.float64).view(npl, n0 - 2, n1 - 2))
        # register budget of the batched kernels (resident blocks per SM; 0 = 8)
        self.occupancy = 0

    @property
    def main_lines(self):
        return int(_lib.load().qsl_qmap_batch_lines(self.handle))

    def run_main(self, stream=None, lo=0, hi=-1):
        """The batched main trace, or the window [lo, hi) of its lines."""
        _lib.check(_lib.load().qsl_qmap_batch_run_main(self.handle, int(lo), int(hi), self.max_blocks, self.occupancy,
                                                       stream_handle(stream)), "qsl_qmap_batch_run_main")

    def run_post(self, stream=None):
        """Everything after the main trace: Q, pseudo-lines, merge; returns
        the jobs' Q maps (views of the workspace)."""
        _lib.check(_lib.load().qsl_qmap_batch_run_post(self.handle, self.max_blocks, self.occupancy,
                                                       stream_handle(stream)), "qsl_qmap_batch_run_post")
        return self.Q

    def run(self, stream=None):
        self.run_main(stream)
        return self.run_post(stream)

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().qsl_qmap_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class QSeries:
    """Q maps of a series of fields given on the host (the snapshots of a
    simulation, a run of magnetograms' extrapolations) on one seed geometry,
    pipelined over two field stores and two plans:

    * upload: field k's H2D copy on the uploader's copy stream (pinned host
      arrays, FieldUploader) while earlier fields are on the GPU;
    * pack: field k into store k % 2 on a pack stream, once that store's
      previous trace (field k - 2) is done: it overlaps field k - 1's trace;
    * trace + Q: plan k % 2 on `stream` (default: the current stream), once
      field k is packed and that plan's previous Q (field k - 2) has been
      copied out;
    * D2H: field k's Q into the caller's pinned host tensor on a copy stream,
      overlapping field k + 1's trace.

    Nothing here synchronises the host; wait() makes `stream` wait for every
    queued copy.  Each field's Q equals QMapPlan.run's on that field alone
    (the same kernels on the same inputs)."""

    def __init__(self, shape, n0, n1, nplanes, layout="h4b", device="cuda", tile=(8, 8), occupancy=None):
        self.device = torch.device(device)
        self.up = FieldUploader(shape, device=self.device)
        zero = torch.zeros(tuple(shape)[::-1], dtype=torch.float32, device=self.device).permute(2, 1, 0)
        self.stores = [FieldStore(zero, zero, zero, layout=layout) for _ in range(2)]
        self.plans = [QMapPlan(n0, n1, nplanes, device=self.device, tile=tile, occupancy=occupancy)
                      for _ in range(2)]
        self.pack_stream = torch.cuda.Stream(device=self.device)
        self.d2h_stream = torch.cuda.Stream(device=self.device)
        self.traced = [None, None]   # per store / plan: the event after its last trace and Q
        self.copied = [None, None]   # per plan: the event after its last Q copy to the host
        self.k = 0

    def push(self, Bx, By, Bz, xs, ys, zs, params, q_out, stream=None, **run_kw):
        """Queues one field (pinned host arrays as FieldUploader.upload takes
        them) through the pipeline; its Q lands in `q_out`, a pinned CPU
        float64 tensor of the plan's Q shape, once wait() (or an event after
        it) has completed.  run_kw: QMapPlan.run's settings (s_len, stride,
        cross_dir, tol_coef, ...)."""
        st = stream if isinstance(stream, torch.cuda.Stream) else torch.cuda.current_stream(self.device)
        s = self.k % 2
        self.k += 1
        slot = self.up.upload(Bx, By, Bz)
        if self.traced[s] is not None:
            self.pack_stream.wait_event(self.traced[s])
        self.up.pack(self.stores[s], slot, self.pack_stream)
        packed = torch.cuda.Event()
        packed.record(self.pack_stream)
        st.wait_event(packed)
        if self.copied[s] is not None:
            st.wait_event(self.copied[s])
        q = self.plans[s].run(self.stores[s], xs, ys, zs, params, stream=st, **run_kw)
        ev = torch.cuda.Event()
        ev.record(st)
        self.traced[s] = ev
        self.d2h_stream.wait_event(ev)
        with torch.cuda.stream(self.d2h_stream):
            q_out.copy_(q, non_blocking=True)
        done = torch.cuda.Event()
        done.record(self.d2h_stream)
        self.copied[s] = done
        return q_out

    def wait(self, stream=None):
        """Makes `stream` (default: the current stream) wait for every field
        queued so far, its Q copied to the host included."""
        st = stream if isinstance(stream, torch.cuda.Stream) else torch.cuda.current_stream(self.device)
        for ev in self.copied:
            if ev is not None:
                st.wait_event(ev)

    def close(self):
        for fs in self.stores:
            fs.close()


def plane_seed_grid(x0, x1, nx, y0, y1, ny, zs, device="cuda"):
    """Stacked seed planes: for each z in `zs`, an (ny, nx) grid over
    [x0, x1] x [y0, y1] (linspace per axis, rows along y).  Returns flattened
    float32 CUDA vectors (x, y, z)."""
    xi = torch.linspace(x0, x1, nx, dtype=torch.float32, device=device)
    yi = torch.linspace(y0, y1, ny, dtype=torch.float32, device=device)
    zt = torch.as_tensor(zs, dtype=torch.float32, device=device).reshape(-1)
    npl = zt.shape[0]
    X = xi.view(1, 1, nx).expand(npl, ny, nx)
    Y = yi.view(1, ny, 1).expand(npl, ny, nx)
    Z = zt.view(npl, 1, 1).expand(npl, ny, nx)
    return X.reshape(-1).contiguous(), Y.reshape(-1).contiguous(), Z.reshape(-1).contiguous()


class BatchPlan:
    """Many trace jobs in one launch per field-store type.

    jobs: list of dicts with keys field (FieldStore), xs, ys, zs, params,
    s_len, tol_coef, cross_dir, out (trace output dict), optional order,
    n_dev (device seed count; then n = capacity) and n.  The job table is
    serialised once (qsl_batch_pack) into pinned host memory and copied
    asynchronously to the device on `stream`; launch() only launches kernels
    (qsl_batch_run), so it can be captured into a CUDA graph.  Nothing here
    synchronises the device."""

    def __init__(self, jobs, stream=None, device="cuda"):
        lib = _lib.load()
        arr = (_lib.BatchJob * max(1, len(jobs)))()
        self._keep = []
        for k, j in enumerate(jobs):
            b = arr[k]
            b.field = j["field"].handle
            b.params = j["params"]
            b.io = _io(j["xs"], j["ys"], j["zs"], j["out"])
            b.n = int(j["n"]) if "n" in j else int(j["xs"].shape[0])
            b.s_len = float(j.get("s_len", 0.25))
            b.tol_coef = float(j.get("tol_coef", 1.0))
            for c in range(3):
                b.cross_dir[c] = float(j.get("cross_dir", (0.0, 0.0, 1.0))[c])
            b.order = ptr(j.get("order"))
            b.n_dev = ptr(j.get("n_dev"))
            self._keep.append(j)
        info = _lib.BatchInfo()
        _lib.check(lib.qsl_batch_pack(arr, len(jobs), None, 0, ctypes.byref(info)), "qsl_batch_pack")
        nbytes = max(256, int(info.table_bytes))
        self._host = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        _lib.check(lib.qsl_batch_pack(arr, len(jobs), self._host.data_ptr(), nbytes, ctypes.byref(info)),
                   "qsl_batch_pack")
        self._dev = torch.empty(nbytes, dtype=torch.uint8, device=device)
        if stream is not None and isinstance(stream, torch.cuda.Stream):
            with torch.cuda.stream(stream):
                self._dev.copy_(self._host, non_blocking=True)
        else:
            self._dev.copy_(self._host, non_blocking=True)
        self.info = info
        self.lines = int(info.lines)

    def launch(self, samples=None, stream=None, max_blocks=0, lo=0, hi=-1, occupancy=0):
        """Lines [lo, hi) of the batch (hi < 0: all); max_blocks > 0: at most
        that many resident blocks (they loop over the lines), leaving the rest
        of the GPU's block slots free; occupancy: the kernels' register budget
        in resident blocks per SM (6-10, 0 = 8)."""
        _lib.check(_lib.load().qsl_batch_run_window(self._dev.data_ptr(), ctypes.byref(self.info), ptr(samples),
                                                    int(lo), int(hi), int(max_blocks), int(occupancy),
                                                    stream_handle(stream)),
                   "qsl_batch_run")

    @property
    def window_lines(self):
        """Length of the longest store type's line space (padded per job): the
        end of the last window of launch(lo, hi)."""
        return max(int(self.info.total[k]) for k in range(4))


class QBatch:
    """Q maps of many independent jobs (each: a resident field, a stack of
    (n0, n1) seed planes on arbitrary planes, its own integrator settings)
    solved together: one batched main-trace launch, per-job Q assembly and
    pseudo-line compaction, one batched pseudo-line launch, per-job pseudo Q
    and merge.  All buffers are allocated up front; run() issues only
    kernels, so it can be captured once into a CUDA graph (capture()) and
    replayed.  Reference workflow per job: demo/Q_RKF45CuPy.ipynb cells 7-11.

    specs: list of dicts with keys field, xs, ys, zs (flattened stacked
    planes), n0, n1, nplanes, params, s_len, tol_coef, stride, cross_dir."""

    def __init__(self, specs, device="cuda", tile=(8, 8), stream=None, blocks_per_sm=0):
        """blocks_per_sm > 0: the batched traces keep at most that many
        resident blocks per SM (see BatchPlan.launch)."""
        self.max_blocks = 0
        if blocks_per_sm:
            sms = ctypes.c_int(0)
            _lib.check(_lib.load().qsl_device_sm_count(ctypes.byref(sms)), "qsl_device_sm_count")
            self.max_blocks = int(blocks_per_sm) * sms.value
        self.specs = specs
        lib = _lib.load()
        self.jobs = []
        main_jobs, sub_jobs = [], []
        for sp in specs:
            n0, n1, npl = int(sp["n0"]), int(sp["n1"]), int(sp.get("nplanes", 1))
            n = n0 * n1 * npl
            m = npl * (n0 - 2) * (n1 - 2)
            J = dict(sp=sp, n0=n0, n1=n1, npl=npl, n=n, m=m)
            # every array of the job in one allocation, uninitialised: the
            # kernels write each element they later read (the pseudo-line
            # arrays up to the device count the compaction writes)
            wb = int(lib.qsl_cook_workspace_bytes(n))
            parts = (trace_output_parts(n, prefix="main.") + trace_output_parts(4 * m, prefix="sub.") +
                     [("Q", npl * (n0 - 2) * (n1 - 2), torch.float64), ("cut0", 4 * m, torch.float32),
                      ("cut1", 4 * m, torch.float32), ("cut2", 4 * m, torch.float32), ("bz0s", m, torch.float32),
                      ("bz0e", m, torch.float32), ("pix", m, torch.int64), ("count", 2, torch.int64),
                      ("work", (wb + 7) // 8, torch.int64), ("qcut", m, torch.float64)])
            if tile:
                parts.append(("order", n, torch.int32))
            # the arrays only kernels touch are carried as device addresses
            # (no tensor objects: the host cost of a small request's batch
            # is mostly per-array bookkeeping); Q is a tensor for the caller
            offs, total = _layout(parts)
            J["buf"] = torch.empty(total, dtype=torch.uint8, device=device)
            base = J["buf"].data_ptr()
            a = {name: base + o for name, o in offs.items()}
            J["main"] = {k: a["main." + k] for k in _TRACE_OUT}
            J["sub"] = {k: a["sub." + k] for k in _TRACE_OUT}
            J["main"]["twist"] = J["sub"]["twist"] = None
            qn = npl * (n0 - 2) * (n1 - 2)
            J["Q"] = J["buf"][offs["Q"]:offs["Q"] + 8 * qn].view(torch.float64).view(npl, n0 - 2, n1 - 2)
            J["cut"] = [a["cut0"], a["cut1"], a["cut2"]]
            J["bz0s"], J["bz0e"], J["pix"], J["qcut"] = a["bz0s"], a["bz0e"], a["pix"], a["qcut"]
            J["count"] = a["count"]  # written by the compaction before anything reads it
            J["work"], J["work_bytes"] = a["work"], wb
            J["order"] = None
            if tile:
                J["order"] = a["order"]
                _lib.check(lib.qsl_tile_order(npl, n0, n1, int(tile[0]), int(tile[1]), npl, J["order"],
                                              stream_handle(stream)), "qsl_tile_order")
            common = dict(field=sp["field"], params=sp["params"], s_len=sp.get("s_len", 0.25),
                          tol_coef=sp.get("tol_coef", 1.0), cross_dir=sp.get("cross_dir", (0.0, 0.0, 1.0)))
            main_jobs.append(dict(common, xs=sp["xs"], ys=sp["ys"], zs=sp["zs"], out=J["main"], order=J["order"]))
            sub_jobs.append(dict(common, xs=J["cut"][0], ys=J["cut"][1], zs=J["cut"][2], out=J["sub"],
                                 n=4 * m, n_dev=J["count"] + 8))
            self.jobs.append(J)
        self.main_batch = BatchPlan(main_jobs, stream=stream)
        self.sub_batch = BatchPlan(sub_jobs, stream=stream)
        self.graph = None
        # register budget of the batched kernels (resident blocks per SM;
        # autotune.tune_batch measures the choices; 0 = 8)
        self.occupancy = 0

    @property
    def main_lines(self):
        return self.main_batch.window_lines

    def run(self, stream=None):
        self.run_main(stream)
        return self.run_post(stream)

    def run_main(self, stream=None, lo=0, hi=-1):
        """The batched main trace, or the window [lo, hi) of its lines."""
        self.main_batch.launch(stream=stream, max_blocks=self.max_blocks, lo=lo, hi=hi, occupancy=self.occupancy)

    def run_post(self, stream=None):
        """Everything after the main trace: Q, pseudo-lines, merge."""
        lib = _lib.load()
        st = stream_handle(stream)
        for J in self.jobs:
            sp, m = J["sp"], J["main"]
            jac = (1.0 / (2.0 * float(sp.get("stride", 1.0)))) ** 4.0
            cd = (ctypes.c_float * 3)(*[float(c) for c in sp.get("cross_dir", (0.0, 0.0, 1.0))])
            _lib.check(lib.qsl_qcalc_plane(ptr(m["end_x"]), ptr(m["end_y"]), ptr(m["end_z"]), ptr(m["flag_end"]),
                                           ptr(m["start_x"]), ptr(m["start_y"]), ptr(m["start_z"]),
                                           ptr(m["flag_start"]), ptr(m["B_start_z"]), ptr(m["B_end_z"]),
                                           ptr(m["B_this_x"]), ptr(m["B_this_y"]), ptr(m["B_this_z"]), J["n0"],
                                           J["n1"], J["npl"], jac, cd, None, ptr(J["Q"]), st), "qcalc_plane")
            _lib.check(lib.qsl_cook_pseudo_line(ptr(m["B_flag"]), ptr(m["start_x"]), ptr(m["start_y"]),
                                                ptr(m["start_z"]), ptr(m["flag_start"]), ptr(m["B_start_z"]),
                                                ptr(m["B_end_z"]), J["n"], J["n0"], J["n1"], 1,
                                                float(sp.get("stride", 1.0)), ptr(J["cut"][0]), ptr(J["cut"][1]),
                                                ptr(J["cut"][2]), ptr(J["bz0s"]), ptr(J["bz0e"]), ptr(J["pix"]),
                                                ptr(J["count"]), ptr(J["work"]), J["work_bytes"], st), "cook")
        self.sub_batch.launch(stream=stream, max_blocks=self.max_blocks, occupancy=self.occupancy)
        for J in self.jobs:
            sp, s = J["sp"], J["sub"]
            jac = (1.0 / (2.0 * float(sp.get("stride", 1.0)))) ** 4.0
            _lib.check(lib.qsl_qcut(ptr(s["start_x"]), ptr(s["start_y"]), ptr(s["start_z"]), ptr(s["flag_start"]),
                                    ptr(s["end_x"]), ptr(s["end_y"]), ptr(s["end_z"]), ptr(s["flag_end"]),
                                    ptr(J["bz0s"]), ptr(J["bz0e"]), 0, J["count"], J["m"], jac, None,
                                    ptr(J["qcut"]), st), "qcut")
            _lib.check(lib.qsl_qmerge(ptr(J["pix"]), None, ptr(J["qcut"]), 0, J["count"], J["m"],
                                      J["n0"], J["n1"], None, ptr(J["Q"]), st), "qmerge")
        return [J["Q"] for J in self.jobs]

    def capture(self):
        """Captures run() into a CUDA graph (replay with replay())."""
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.run(stream=s)  # warm-up outside capture
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run()
        self.graph = g
        return g

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()
        return [J["Q"] for J in self.jobs]
