"""The C-ABI library builds, loads without a GPU and exports every entry
point include/fastqsl_gb300.h declares (no compute calls here)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fastqsl_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(qsl_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from fastqsl_gb300 import _build, _lib
    _build.build()
    return _lib.load()


def test_header_declares_the_drop_in_entries():
    names = declared_functions()
    for n in ["qsl_trace_all_bline_rkf45", "qsl_trace_all_bline_rk4", "qsl_qcalc_plane", "qsl_cook_pseudo_line",
              "qsl_qcut", "qsl_qmerge", "qsl_trace", "qsl_field_create"]:
        assert n in names


def test_every_declared_symbol_is_exported(lib):
    from fastqsl_gb300 import _lib
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\sT\s(qsl_\w+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    # and the ctypes table covers the same set
    assert set(_lib.exported_names()) == set(declared_functions())


def test_reference_presets_match_python(lib):
    from fastqsl_gb300 import params as P
    for cfn, pfn in ((lib.qsl_params_reference_rk4, P.reference_rk4), (lib.qsl_params_reference_rkf45,
                                                                        P.reference_rkf45),
                     (lib.qsl_params_reference_scott, P.reference_scott)):
        c = P.TraceParams()
        cfn(ctypes.byref(c))
        assert c.as_dict() == pfn().as_dict()


def test_params_struct_layout():
    from fastqsl_gb300 import params as P, _lib
    # int32, int32, 5 doubles, int64, int32, int32, int32, (pad to 8)
    assert ctypes.sizeof(P.TraceParams) == 4 + 4 + 5 * 8 + 8 + 4 + 4 + 4 + 4
    assert ctypes.sizeof(_lib.TraceIO) == 25 * 8
    assert ctypes.sizeof(_lib.ScottIO) == 18 * 8
    assert ctypes.sizeof(_lib.Sched) == 4 + 4 + 3 * 8 + 8
    # field, params, io, n, s_len, tol_coef, cross[3], (pad), curB[3], order, n_dev
    assert ctypes.sizeof(_lib.BatchJob) == 8 + 72 + 200 + 8 + 4 + 4 + 12 + 4 + 24 + 8 + 8


def test_version_and_errors_without_gpu(lib):
    assert b"sm_103a" in lib.qsl_version()
    # argument validation runs before any CUDA call
    rc = lib.qsl_qcalc_plane(*([None] * 13), 2, 2, 1, 1.0, None, None, None, None)
    assert rc == -1
    assert b"null" in lib.qsl_last_error()
    assert lib.qsl_field_store_bytes(1, 5, 5, 1) == -1
    assert lib.qsl_field_store_bytes(9, 9, 9, 2) == 10368 + 4  # one brick of x-pair records + its scale
    assert lib.qsl_field_store_bytes(10, 10, 10, 1) == 16000


def test_new_entries_validate_without_gpu(lib):
    """The polyline, current-store and window entries reject bad arguments
    before any CUDA call."""
    import ctypes
    from fastqsl_gb300 import _lib
    # qsl_trace_path: index range outside the output rows, zero stride, nulls
    dummy = ctypes.c_void_p(16)
    args = [dummy, dummy, dummy, 4, 4, 4, dummy, 1]
    tail = [0.25, dummy, dummy, dummy, 10, None]
    assert lib.qsl_trace_path(*args, 5, 11, 1, *tail) == -1
    assert b"outside" in lib.qsl_last_error()
    assert lib.qsl_trace_path(*args, 5, -2, -1, *tail) == -1
    assert lib.qsl_trace_path(*args, 0, 5, 0, *tail) == -1
    assert lib.qsl_trace_path(None, None, None, 4, 4, 4, None, 1, 0, 5, 1, 0.25, None, None, None, 10, None) == -1
    assert lib.qsl_trace_path(*args, 0, 0, 1, *tail) == 0  # an empty range does nothing
    assert lib.qsl_sample_points(None, None, None, 4, 4, 4, None, 3, 1, None, None) == -1
    assert lib.qsl_sample_points(dummy, dummy, dummy, 1, 4, 4, dummy, 3, 1, dummy, None) == -1
    # qsl_trace_cur: a null current store
    from fastqsl_gb300 import params as P
    prm = P.absolute_rkf45()
    io = _lib.TraceIO()
    assert lib.qsl_trace_cur(None, None, ctypes.byref(prm), ctypes.byref(io), 10, None, 0.25, 1.0, None, None,
                             None) == -1
    assert b"null" in lib.qsl_last_error()
    # qsl_batch_run_window: null table
    info = _lib.BatchInfo()
    assert lib.qsl_batch_run_window(None, ctypes.byref(info), None, 0, -1, 0, 0, None) != 0
    assert lib.qsl_batch_run_window(ctypes.c_void_p(256), ctypes.byref(info), None, 0, -1, 0, 5, None) == -1
    assert b"occupancy" in lib.qsl_last_error()


def test_seed_geometry_entries_validate_without_gpu(lib):
    """qsl_plane_seeds and qsl_tile_order reject nulls, non-positive sizes
    and order maps beyond 2^32 seeds before any CUDA call."""
    import ctypes
    d3 = ctypes.c_double * 3
    dummy = ctypes.c_void_p(256)
    v = d3(0.0, 0.0, 1.0)
    assert lib.qsl_plane_seeds(None, v, v, v, 1.0, 4, 4, 1, dummy, dummy, dummy, None) == -1
    assert b"null" in lib.qsl_last_error()
    assert lib.qsl_plane_seeds(v, v, v, v, 1.0, 0, 4, 1, dummy, dummy, dummy, None) == -1
    assert b"positive" in lib.qsl_last_error()
    assert lib.qsl_plane_seeds(v, v, v, v, 1.0, 4, 4, 1, dummy, None, dummy, None) == -1
    assert lib.qsl_tile_order(1, 4, 4, 8, 8, 0, None, None) == -1
    assert b"null" in lib.qsl_last_error()
    assert lib.qsl_tile_order(1, 4, 4, 0, 8, 0, dummy, None) == -1
    assert lib.qsl_tile_order(2, 65536, 65536, 8, 8, 0, dummy, None) != 0
    assert b"2^32" in lib.qsl_last_error()


def test_qmap_batch_validates_without_gpu(lib):
    """qsl_qmap_batch_size / _create reject empty job lists, null fields and
    degenerate planes before any CUDA call."""
    import ctypes
    from fastqsl_gb300 import _lib, params as P
    d, h = ctypes.c_int64(0), ctypes.c_int64(0)
    jobs = (_lib.QmapJob * 1)()
    assert lib.qsl_qmap_batch_size(jobs, 0, ctypes.byref(d), ctypes.byref(h)) == -1
    assert b"at least one job" in lib.qsl_last_error()
    jobs[0].params = P.absolute_rkf45()
    jobs[0].n0, jobs[0].n1, jobs[0].nplanes, jobs[0].spacing = 5, 5, 1, 1.0
    assert lib.qsl_qmap_batch_size(jobs, 1, ctypes.byref(d), ctypes.byref(h)) == -1  # null field
    jobs[0].field = 256
    jobs[0].n0 = 2
    assert lib.qsl_qmap_batch_size(jobs, 1, ctypes.byref(d), ctypes.byref(h)) == -1
    out = ctypes.c_void_p()
    assert lib.qsl_qmap_batch_create(jobs, 1, None, 0, None, 0, None, ctypes.byref(out)) == -1
    assert lib.qsl_qmap_batch_run_main(None, 0, -1, 0, 0, None) == -1
    assert lib.qsl_qmap_batch_q(None, 0) is None
