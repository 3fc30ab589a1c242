"""CPU ORACLE — test infrastructure, not part of the fastqsl_gb300 product.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg use this package, and only as the checker (or the timed CPU baseline);
the product path never imports it.

* ``port32`` — C restatement of the reference tracer in reference-parity FP32
  arithmetic (oracle/port/qsl_port.c, ``qo32_*``);
* ``port32cr`` — the same with a correctly rounded power function, the
  rounding of the GPU's exact kernels (``qo32cr_*``);
* ``port64`` — the same algorithm in FP64 (``qo64_*``), the FP64 oracle;
* ``ref``    — the reference's own kernels compiled for the host
  (oracle/_ref, only where the reference checkout exists);
* ``oracle.qassembly`` — NumPy restatement of the reference's Q assembly.
"""
import ctypes
import os

import numpy as np

from fastqsl_gb300.params import TraceParams

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libqsl_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)

_libs = {}
_PREFIX = {"port32": "qo32_", "port32cr": "qo32cr_", "port64": "qo64_"}


def _load(path):
    if path not in _libs:
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} is not built (run oracle/build.py)")
        _libs[path] = ctypes.CDLL(path)
    return _libs[path]


def port_lib():
    if not os.path.exists(PORT_SO):
        from . import build
        build.build_port()
    return _load(PORT_SO)


def ref_available(kind="rkf45"):
    return os.path.exists(os.path.join(REF_DIR, f"libqslref_{kind}.so"))


def ref_lib(kind):
    return _load(os.path.join(REF_DIR, f"libqslref_{kind}.so"))


def _p(a, t):
    return a.ctypes.data_as(t)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _field_ptrs(Bx, By, Bz):
    """Field arrays of shape (nx, ny, nz), x fastest -> flat float32 buffers
    in memory order and the int32 shape."""
    shape = np.array(Bx.shape, dtype=np.int32)
    flat = [np.asfortranarray(a, dtype=np.float32).ravel(order="F") for a in (Bx, By, Bz)]
    return flat, shape


TRACE_KEYS_F32 = ["start_x", "start_y", "start_z", "end_x", "end_y", "end_z",
                  "B_this_x", "B_this_y", "B_this_z", "B_start_x", "B_start_y", "B_start_z",
                  "B_end_x", "B_end_y", "B_end_z"]
TRACE_KEYS_I32 = ["flag_start", "flag_end", "B_flag"]


def trace_all(impl, Bx, By, Bz, xs, ys, zs, cross_dir=(0, 0, 1), s_len=0.125, tol_coef=1.0,
              params=None, curB=None, threads=None, coords=None, uni=False):
    """Traces every seed.  impl: 'port32', 'port32cr', 'port64' or
    'ref_rk4'/'ref_rkf45'/'ref_stretch' (the reference build ignores `params`:
    its settings are compiled in).  coords=(xa, ya, za): node coordinates of
    a stretched grid (TraceBlineAdaptiveStretch.cu), uni: its uniform-spacing
    index formula.  Returns a dict of numpy arrays keyed like the reference
    kernel's outputs, plus 'LineLen', 'twist' and (port) 'samples'."""
    flat, shape = _field_ptrs(Bx, By, Bz)
    stretch = coords is not None
    if impl == "ref_stretch" and not stretch:
        raise ValueError("ref_stretch needs coords")
    ax = [_f32(c) for c in coords] if stretch else []
    args_coords = [_p(a, _f32p) for a in ax] + [ctypes.c_int(int(bool(uni)))] if stretch else []
    xs, ys, zs = _f32(xs), _f32(ys), _f32(zs)
    n = xs.size
    out = {k: np.zeros(n, np.float32) for k in TRACE_KEYS_F32}
    out.update({k: np.zeros(n, np.int32) for k in TRACE_KEYS_I32})
    out["LineLen"] = np.zeros(n, np.float64)
    twist_on = curB is not None
    out["twist"] = np.zeros(n, np.float64)
    cur = [np.asfortranarray(a, dtype=np.float32).ravel(order="F") for a in curB] if twist_on else [None] * 3
    cd = np.array(cross_dir, dtype=np.float32)
    args_field = [_p(a, _f32p) for a in flat] + [_p(shape, _i32p)]
    args_cur = [(_p(a, _f32p) if a is not None else None) for a in cur]
    common = [
        _p(xs, _f32p), _p(ys, _f32p), _p(zs, _f32p), _p(cd, _f32p),
        _p(out["start_x"], _f32p), _p(out["start_y"], _f32p), _p(out["start_z"], _f32p), _p(out["flag_start"], _i32p),
        _p(out["end_x"], _f32p), _p(out["end_y"], _f32p), _p(out["end_z"], _f32p), _p(out["flag_end"], _i32p),
        _p(out["B_this_x"], _f32p), _p(out["B_this_y"], _f32p), _p(out["B_this_z"], _f32p), _p(out["B_flag"], _i32p),
        _p(out["B_start_x"], _f32p), _p(out["B_start_y"], _f32p), _p(out["B_start_z"], _f32p),
        _p(out["B_end_x"], _f32p), _p(out["B_end_y"], _f32p), _p(out["B_end_z"], _f32p),
    ]
    if impl.startswith("ref"):
        lib = ref_lib(impl.split("_", 1)[1])
        if threads:
            lib.qref_set_threads(int(threads))
        fn = lib.qref_trace_all_stretch if stretch else lib.qref_trace_all
        rc = fn(*args_field, *args_coords, *args_cur, _p(out["twist"], _f64p), ctypes.c_int(int(twist_on)),
                *common, ctypes.c_float(s_len), ctypes.c_ulonglong(n),
                _p(out["LineLen"], _f64p), ctypes.c_float(tol_coef))
    else:
        lib = port_lib()
        fn = getattr(lib, _PREFIX[impl] + ("trace_all_stretch" if stretch else "trace_all"))
        if params is None:
            raise ValueError("port oracle needs params")
        samples = ctypes.c_int64(0)
        _set_threads(threads)
        rc = fn(*args_field, *args_coords, *args_cur, _p(out["twist"], _f64p), ctypes.c_int(int(twist_on)),
                *common, ctypes.c_float(s_len), ctypes.c_int64(n), _p(out["LineLen"], _f64p),
                ctypes.c_float(tol_coef), ctypes.byref(params), ctypes.byref(samples))
        out["samples"] = int(samples.value)
    if rc != 0:
        raise RuntimeError(f"oracle trace_all failed: {rc}")
    return out


SCOTT_KEYS_F32 = ["start_x", "start_y", "start_z", "end_x", "end_y", "end_z",
                  "B_this_x", "B_this_y", "B_this_z", "q_0", "q_perp"]


def scott_all(impl, Bx, By, Bz, xs, ys, zs, s_len=0.25, tol_coef=1.0, params=None, curB=None, threads=None,
              cross_dir=(0, 0, 1)):
    """Scott deviation-vector tracer: the restatement (impl 'port32',
    'port32cr', 'port64'; see qsl_port.c header) or 'ref_scott', the
    reference's whole-line routine built from the copy with its tolerance
    initialised (oracle/build_ref.sh; its settings are compiled in, `params`
    is ignored, and it reports no line length)."""
    flat, shape = _field_ptrs(Bx, By, Bz)
    xs, ys, zs = _f32(xs), _f32(ys), _f32(zs)
    n = xs.size
    out = {k: np.zeros(n, np.float32) for k in SCOTT_KEYS_F32}
    out["flag_start"] = np.zeros(n, np.int32)
    out["flag_end"] = np.zeros(n, np.int32)
    out["LineLen"] = np.zeros(n, np.float64)
    out["twist"] = np.zeros(n, np.float64)
    twist_on = curB is not None
    cur = [np.asfortranarray(a, dtype=np.float32).ravel(order="F") for a in curB] if twist_on else [None] * 3
    if impl == "ref_scott":
        lib = ref_lib("scott")
        if threads:
            lib.qref_set_threads(int(threads))
        cd = np.array(cross_dir, dtype=np.float32)
        rc = lib.qref_scott_all(*[_p(a, _f32p) for a in flat], _p(shape, _i32p),
                                *[(_p(a, _f32p) if a is not None else None) for a in cur], _p(out["twist"], _f64p),
                                ctypes.c_int(int(twist_on)), _p(xs, _f32p), _p(ys, _f32p), _p(zs, _f32p),
                                _p(cd, _f32p),
                                _p(out["start_x"], _f32p), _p(out["start_y"], _f32p), _p(out["start_z"], _f32p),
                                _p(out["flag_start"], _i32p),
                                _p(out["end_x"], _f32p), _p(out["end_y"], _f32p), _p(out["end_z"], _f32p),
                                _p(out["flag_end"], _i32p),
                                _p(out["B_this_x"], _f32p), _p(out["B_this_y"], _f32p), _p(out["B_this_z"], _f32p),
                                _p(out["q_0"], _f32p), _p(out["q_perp"], _f32p),
                                ctypes.c_float(s_len), ctypes.c_ulonglong(n), ctypes.c_float(tol_coef))
        if rc != 0:
            raise RuntimeError(f"reference scott_all failed: {rc}")
        del out["LineLen"]
        return out
    lib = port_lib()
    fn = getattr(lib, _PREFIX[impl] + "scott_all")
    samples = ctypes.c_int64(0)
    _set_threads(threads)
    rc = fn(*[_p(a, _f32p) for a in flat], _p(shape, _i32p),
            *[(_p(a, _f32p) if a is not None else None) for a in cur], _p(out["twist"], _f64p),
            ctypes.c_int(int(twist_on)),
            _p(xs, _f32p), _p(ys, _f32p), _p(zs, _f32p),
            _p(out["start_x"], _f32p), _p(out["start_y"], _f32p), _p(out["start_z"], _f32p),
            _p(out["flag_start"], _i32p),
            _p(out["end_x"], _f32p), _p(out["end_y"], _f32p), _p(out["end_z"], _f32p), _p(out["flag_end"], _i32p),
            _p(out["B_this_x"], _f32p), _p(out["B_this_y"], _f32p), _p(out["B_this_z"], _f32p),
            _p(out["q_0"], _f32p), _p(out["q_perp"], _f32p),
            ctypes.c_float(s_len), ctypes.c_int64(n), _p(out["LineLen"], _f64p), ctypes.c_float(tol_coef),
            ctypes.byref(params), ctypes.byref(samples))
    if rc != 0:
        raise RuntimeError(f"oracle scott_all failed: {rc}")
    out["samples"] = int(samples.value)
    return out


def _set_threads(threads):
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(int(threads))
        try:
            ctypes.CDLL("libgomp.so.1").omp_set_num_threads(int(threads))
        except OSError:
            pass


class Probe:
    """Single-function calls into one implementation ('port32', 'port64',
    'ref_rk4', 'ref_rkf45', 'ref_scott')."""

    def __init__(self, impl, Bx, By, Bz):
        self.impl = impl
        flat, self.shape = _field_ptrs(Bx, By, Bz)
        self.flat = flat
        self.fp = [_p(a, _f32p) for a in flat]
        self.sp = _p(self.shape, _i32p)
        if impl.startswith("ref"):
            self.lib = ref_lib(impl.split("_", 1)[1])
            self.pre = "qref_"
        else:
            self.lib = port_lib()
            self.pre = _PREFIX[impl]
        for nm, rt in (("interp3d", ctypes.c_float), ("rkf45_scott", ctypes.c_float)):
            f = getattr(self.lib, self.pre + nm, None)
            if f is not None:
                f.restype = rt

    def _fn(self, name):
        return getattr(self.lib, self.pre + name)

    def interp(self, p, unit=True):
        o = np.zeros(3, np.float32)
        self._fn("interp3dxyzn")(*self.fp, self.sp, _p(_f32(p), _f32p), ctypes.c_int(int(unit)), _p(o, _f32p))
        return o

    def interp_scalar(self, comp, p):
        return float(self._fn("interp3d")(self.fp[comp], self.sp, _p(_f32(p), _f32p)))

    def checkflag(self, p):
        return int(self._fn("checkflag")(self.sp, _p(_f32(p), _f32p)))

    def rk4(self, p, h):
        o = np.zeros(3, np.float32)
        self._fn("rk4_step")(*self.fp, self.sp, _p(_f32(p), _f32p), ctypes.c_float(h), _p(o, _f32p))
        return o

    def rk4_boundary(self, p, h, d):
        o = np.zeros(3, np.float32)
        self._fn("rk4_boundary")(*self.fp, self.sp, _p(_f32(p), _f32p), ctypes.c_float(h), ctypes.c_int(d),
                                 _p(o, _f32p))
        return o

    def rkf45(self, p, h):
        o = np.zeros(4, np.float32)
        self._fn("rkf45_step")(*self.fp, self.sp, _p(_f32(p), _f32p), ctypes.c_float(h), _p(o, _f32p))
        return o

    def grad_unit_b(self, p):
        o = np.zeros(9, np.float32)
        self._fn("grad_unit_vec_B")(*self.fp, self.sp, _p(_f32(p), _f32p), _p(o, _f32p))
        return o

    def f_scott(self, v9):
        o = np.zeros(9, np.float32)
        self._fn("f_scott")(*self.fp, self.sp, _p(_f32(v9), _f32p), _p(o, _f32p))
        return o

    def rkf45_scott(self, v9, h):
        o = np.zeros(9, np.float32)
        err = self._fn("rkf45_scott")(*self.fp, self.sp, _p(_f32(v9), _f32p), ctypes.c_float(h), _p(o, _f32p))
        return o, float(err)


class StretchProbe:
    """Single-function calls of the stretched-grid tracer into one
    implementation ('port32', 'port64', 'ref_stretch')."""

    def __init__(self, impl, Bx, By, Bz, coords, uni=False):
        flat, self.shape = _field_ptrs(Bx, By, Bz)
        self.flat = flat
        self.ax = [_f32(c) for c in coords]
        self.fp = [_p(a, _f32p) for a in flat]
        self.sp = _p(self.shape, _i32p)
        self.cp = [_p(a, _f32p) for a in self.ax]
        self.uni = ctypes.c_int(int(bool(uni)))
        if impl.startswith("ref"):
            self.lib, self.pre = ref_lib("stretch"), "qref_"
        else:
            self.lib, self.pre = port_lib(), _PREFIX[impl]

    def _fn(self, name):
        return getattr(self.lib, self.pre + name)

    def index(self, p, axis, uni=None):
        a = self.ax[axis]
        u = bool(self.uni.value) if uni is None else uni
        return int(self._fn("index_uni" if u else "index_bisect")(ctypes.c_float(p), ctypes.c_int(a.size),
                                                                 _p(a, _f32p)))

    def interp(self, p, unit=True):
        o = np.zeros(3, np.float32)
        self._fn("interp_stretch")(*self.fp, self.sp, *self.cp, self.uni, _p(_f32(p), _f32p), ctypes.c_int(int(unit)),
                                   _p(o, _f32p))
        return o

    def checkflag(self, p):
        return int(self._fn("checkflag_stretch")(self.sp, *self.cp, self.uni, _p(_f32(p), _f32p)))
