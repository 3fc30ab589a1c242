"""ctypes binding of libfastqsl_gb300.so (the C ABI in include/fastqsl_gb300.h).

There is no CPU fallback: if the shared object is missing or no CUDA device
is visible, every entry point raises.
"""
import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfastqsl_gb300.so")

_lib = None
_lock = threading.Lock()

c_f32p = ctypes.c_void_p  # device pointers travel as integers
c_i64 = ctypes.c_int64
c_int = ctypes.c_int
c_float = ctypes.c_float
c_double = ctypes.c_double
c_vp = ctypes.c_void_p


class QslError(RuntimeError):
    pass


class TraceIO(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in (
        "inp_x", "inp_y", "inp_z", "start_x", "start_y", "start_z", "flag_start",
        "end_x", "end_y", "end_z", "flag_end", "B_this_x", "B_this_y", "B_this_z", "B_flag",
        "B_start_x", "B_start_y", "B_start_z", "B_end_x", "B_end_y", "B_end_z", "LineLen", "twist",
        "status_start", "status_end")]


class BatchJob(ctypes.Structure):
    pass  # fields set below (needs TraceParams and TraceIO)


class BatchInfo(ctypes.Structure):
    _fields_ = [("jobs_offset", ctypes.c_int64 * 4), ("begin_offset", ctypes.c_int64 * 4),
                ("total", ctypes.c_int64 * 4), ("njobs", ctypes.c_int32 * 4), ("twist", ctypes.c_int32 * 4),
                ("table_bytes", ctypes.c_int64), ("lines", ctypes.c_int64)]


class ScottIO(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in (
        "inp_x", "inp_y", "inp_z", "start_x", "start_y", "start_z", "flag_start",
        "end_x", "end_y", "end_z", "flag_end", "B_this_x", "B_this_y", "B_this_z", "q_0", "q_perp",
        "LineLen", "twist")]


class Sched(ctypes.Structure):
    _fields_ = [("schedule", ctypes.c_int32), ("chunk", ctypes.c_int32), ("order", ctypes.c_void_p),
                ("queue", ctypes.c_void_p), ("samples", ctypes.c_void_p), ("occupancy", ctypes.c_int32)]


def _finish_batch_job():
    from .params import TraceParams
    BatchJob._fields_ = [("field", ctypes.c_void_p), ("params", TraceParams), ("io", TraceIO),
                         ("n", ctypes.c_int64), ("s_len", ctypes.c_float), ("tol_coef", ctypes.c_float),
                         ("cross_dir", ctypes.c_float * 3), ("curB", ctypes.c_void_p * 3),
                         ("order", ctypes.c_void_p), ("n_dev", ctypes.c_void_p)]


_finish_batch_job()


class QmapJob(ctypes.Structure):
    pass  # fields set below (needs TraceParams)


def _finish_qmap_job():
    from .params import TraceParams
    d3 = ctypes.c_double * 3
    QmapJob._fields_ = [("field", ctypes.c_void_p), ("params", TraceParams), ("center", d3), ("normal", d3),
                        ("u", d3), ("v", d3), ("spacing", ctypes.c_double), ("n0", ctypes.c_int32),
                        ("n1", ctypes.c_int32), ("nplanes", ctypes.c_int32), ("tile_y", ctypes.c_int32),
                        ("tile_x", ctypes.c_int32), ("s_len", ctypes.c_float), ("tol_coef", ctypes.c_float)]


_finish_qmap_job()

# name -> (restype, argtypes); every pointer is c_void_p
_P = c_vp
_SIGS = {
    "qsl_version": (ctypes.c_char_p, []),
    "qsl_last_error": (ctypes.c_char_p, []),
    "qsl_device_sm_count": (c_int, [_P]),
    "qsl_params_reference_rk4": (None, [_P]),
    "qsl_params_reference_rkf45": (None, [_P]),
    "qsl_trace_all_bline": (c_int, [c_int, c_int] + [_P] * 35 + [c_i64, _P]),
    "qsl_trace_all_bline_rkf45": (c_int, [_P] * 35 + [_P]),
    "qsl_trace_all_bline_rk4": (c_int, [_P] * 34 + [_P]),
    "qsl_params_reference_scott": (None, [_P]),
    "qsl_batch_pack": (c_int, [_P, c_int, _P, c_i64, _P]),
    "qsl_batch_run": (c_int, [_P, _P, _P, _P]),
    "qsl_batch_run_window": (c_int, [_P, _P, _P, c_i64, c_i64, c_int, c_int, _P]),
    "qsl_batch_create": (c_int, [_P, c_int, _P, _P]),
    "qsl_batch_launch": (c_int, [_P, _P, _P]),
    "qsl_batch_lines": (c_i64, [_P]),
    "qsl_batch_destroy": (c_int, [_P]),
    "qsl_trace_all_bline_scott": (c_int, [_P] * 30 + [c_i64, _P]),
    "qsl_params_reference_stretch": (None, [_P]),
    "qsl_hybrid_select": (c_int, [_P, _P, c_int, c_int, c_i64, _P, _P, _P]),
    "qsl_curl_grid": (c_int, [_P, _P, _P, c_int, c_int, c_int] + [_P] * 7),
    "qsl_trace_path": (c_int, [_P, _P, _P, c_int, c_int, c_int, _P, c_i64, c_i64, c_i64, c_i64, c_double,
                               _P, _P, _P, c_i64, _P]),
    "qsl_sample_points": (c_int, [_P, _P, _P, c_int, c_int, c_int, _P, c_i64, c_int, _P, _P]),
    "qsl_hybrid_merge": (c_int, [_P, _P, c_int, c_int, c_i64, _P, _P]),
    "qsl_trace_all_bline_stretch": (c_int, [c_int] + [_P] * 39 + [c_i64, _P]),
    "qsl_trace_stretch": (c_int, [_P, _P, _P, c_int, c_int, c_int, _P, _P, _P, c_int, _P, _P, c_i64, c_float,
                                  c_float, _P, _P, _P, _P, _P, _P]),
    "qsl_trace_scott": (c_int, [_P, _P, _P, c_i64, _P, c_float, c_float, _P, _P, _P, c_int, _P, _P]),
    "qsl_field_store_bytes": (c_i64, [c_int, c_int, c_int, c_int]),
    "qsl_field_create": (c_int, [_P, _P, _P, c_int, c_int, c_int, c_int, _P, _P]),
    "qsl_field_destroy": (c_int, [_P]),
    "qsl_field_bytes": (c_i64, [_P]),
    "qsl_field_update": (c_int, [_P, _P, _P, _P, _P]),
    "qsl_trace": (c_int, [_P, _P, _P, c_i64, _P, c_float, c_float, _P, _P, _P, _P, _P, _P]),
    "qsl_trace_cur": (c_int, [_P, _P, _P, _P, c_i64, _P, c_float, c_float, _P, _P, _P]),
    "qsl_qcalc_plane": (c_int, [_P] * 13 + [c_int, c_int, c_i64, c_double, _P, _P, _P, _P]),
    "qsl_cook_workspace_bytes": (c_i64, [c_i64]),
    "qsl_cook_pseudo_line": (c_int, [_P] * 7 + [c_i64, c_int, c_int, c_int, c_float] + [_P] * 8 + [c_i64, _P]),
    "qsl_cook_noalloc_max_pixels": (c_i64, []),
    "qsl_cook_pseudo_line_noalloc": (c_int, [_P] * 7 + [c_i64, c_int, c_int, c_int, c_float] + [_P] * 7 + [_P]),
    "qsl_qcut": (c_int, [_P] * 10 + [c_i64, _P, c_i64, c_double, _P, _P, _P]),
    "qsl_qmerge": (c_int, [_P, _P, _P, c_i64, _P, c_i64, c_int, c_int, _P, _P, _P]),
    "qsl_l1_probe": (c_int, [_P, c_i64, c_int, c_int, c_int, _P, _P]),
    "qsl_plane_seeds": (c_int, [_P, _P, _P, _P, c_double, c_int, c_int, c_int, _P, _P, _P, _P]),
    "qsl_tile_order": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, _P, _P]),
    "qsl_qmap_batch_size": (c_int, [_P, c_int, _P, _P]),
    "qsl_qmap_batch_create": (c_int, [_P, c_int, _P, c_i64, _P, c_i64, _P, _P]),
    "qsl_qmap_batch_lines": (c_i64, [_P]),
    "qsl_qmap_batch_run_main": (c_int, [_P, c_i64, c_i64, c_int, c_int, _P]),
    "qsl_qmap_batch_run_post": (c_int, [_P, c_int, c_int, _P]),
    "qsl_qmap_batch_q": (_P, [_P, c_int]),
    "qsl_qmap_batch_destroy": (c_int, [_P]),
}


def exported_names():
    return list(_SIGS)


def load(path=None):
    """Loads the shared object (once) and declares every entry point."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise QslError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                           f"or `python -m fastqsl_gb300._build` (no CPU fallback exists)")
        lib = ctypes.CDLL(p)
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(rc, what=""):
    if rc != 0:
        msg = load().qsl_last_error().decode(errors="replace")
        raise QslError(f"{what} failed ({rc}): {msg}")
    return rc
